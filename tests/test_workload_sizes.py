"""The seeded benchmark workloads have the sizes of the hot path's scope table
(elements, nodes with their vertices, and equations before boundary
conditions, 3 per node + 1 per vertex), so the measured configurations are
the ones the metric is quoted on.  CPU only: mesh generation, no kernels."""
import numpy as np
import pytest

from poromec_gb300 import meshgen


def _sizes(pb):
    nnode, nnodev = int(pb["nnode"]), int(pb["nnodev"])
    return int(pb["numel"]), nnode, nnodev, 3 * nnode + nnodev


@pytest.mark.parametrize("name,make,numel,nnode,nnodev,neq", [
    ("1: column 2x2x40", lambda: meshgen.column_problem(), 160, 1221, 369, 4032),
    ("2: cube 56^3", lambda: meshgen.cube_problem(56), 175616, 731025, 185193, 2378268),
    ("3: tetra10 48^3 x 6", lambda: meshgen.tetra_problem(48), 663552, 912673, 117649,
     2855668),
    ("5: cube 40^3", lambda: meshgen.cube_problem(40), 64000, 270641, 68921, 880844),
])
def test_single_mesh_workloads(name, make, numel, nnode, nnodev, neq):
    assert _sizes(make()) == (numel, nnode, nnodev, neq), name


def test_batch_workload():
    """96 unit cubes with n uniform in 8..32: 8,748 to 457,380 equations each
    before boundary conditions (the extremes n = 8 and n = 32 of the table)."""
    inst = meshgen.batch_instances(ninst=96, nmin=8, nmax=32, seed=4242)
    assert len(inst) == 96
    ns = np.array([p["n"] for p in inst])
    assert ns.min() >= 8 and ns.max() <= 32
    eqs = np.array([_sizes(p)[3] for p in inst])
    # hexa20 n^3: (n+1)^3 vertices and 3 n (n+1)^2 mid-edge nodes
    expect = 3 * ((ns + 1) ** 3 + 3 * ns * (ns + 1) ** 2) + (ns + 1) ** 3
    assert np.array_equal(eqs, expect)
    if ns.min() == 8:
        assert eqs.min() == 8748
    if ns.max() == 32:
        assert eqs.max() == 457380
    # the union holds every instance side by side
    u = meshgen.union_problem(inst)
    assert _sizes(u)[3] == int(eqs.sum())
