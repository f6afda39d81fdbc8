"""Deck reader (pm_deck_read, include/poromec_gb300.h): the mesh macro of
rdat_pm (Rdata.f:1-1037), the quadratic mesh from linear elements
(mk_elconn_quad_v1, Adjacency.f:583-700; mk_bound_quad / mk_forces_quad /
mk_initial_quad, Rdata.f:2337-2544), the end-of-mesh initial conditions
(boundc, bound_nodalloads) and the macro program of Main.f.  Reading needs
no GPU.

The golden fixtures were made from the reference's shipped decks by
tests/golden/make_golden.py, an independent restatement in Python; that
script also checks this reader against the shipped decks themselves.  Here a
deck written back from each fixture in the shipped decks' syntax must read
back to the fixture bit for bit; a hand-written deck covers the macros the
shipped decks do not use.
"""
import os

import numpy as np
import pytest

from deck_writer import write_linear_deck

pytest.importorskip("ctypes")
from poromec_gb300.deck import Deck, DeckError, read_vtk  # noqa: E402

ARRAYS = ["ix", "id", "fnno", "x", "e", "ie", "eload", "load", "u0", "fload"]


@pytest.mark.parametrize("name", ["exemplo1_mesh0_t2", "exemplo1_mesh0_t2_tetra", "solo1",
                                  "solo_cilindro_hexa_1", "solo_cilindro_tetra_1"])
def test_linear_deck_reads_back_to_the_fixture(golden, tmp_path, name):
    fx = golden(name)
    path = write_linear_deck(fx, str(tmp_path), name)
    d = Deck(path)
    pb = d.problem()
    for k in ARRAYS:
        assert pb[k].shape == np.asarray(fx[k]).shape, k
        assert np.array_equal(pb[k], fx[k]), k
    assert int(d.value("nnode")) == int(fx["nnode"])
    assert int(d.value("nnodev")) == int(fx["nnodev"])
    assert list(pb["print_nodes"]) == list(fx["hist_nodes"])
    assert pb["dt"] == float(fx["dt"]) and pb["maxnlit"] == max(2, int(fx["maxnlit"]))
    assert pb["solver"] == 1 and pb["maxit"] == int(fx["maxit"])
    assert pb["solvtol"] == float(fx["solver_tol"]) and pb["stop_crit"] == 1
    assert np.array_equal(pb["gravity"], fx["gravity"])
    assert d.value("mk_quad") == 1


CURRENT = """\
// a deck in the current macro syntax
solver solver.dat
gravity gravity.dat
mesh
nnode 8 numel 1 numat 1 maxno 20 ndf 4 dim 3
materials
1 17 10.0d0 0.25d0 1.0d-6 5.0d4 1.0d0 0.0d0 1.0d3 0.3d0
end materials
hexa8
1 1 2 3 4 5 6 7 8 1
end hexa8
insert coor.dat
constrainpmec
1 1 1 1 0
2 1 1 1 0
3 1 1 1 0
4 1 1 1 0
end constrainpmec
nodalforces
1 0.0 0.0 -1.0d-3 0.0
2 0.0 0.0 -3.0d-3 0.0
end nodalforces
nodalloads
5 0 0 0 2
end nodalloads
loads
1 40 load1.dat
2 2 0.5d0 1.0d-3
end loads
elmtloads
1 0 0 0 0 0 1 0
end elmtloads
initialstress
1 -1.0 -1.0 -2.0 0.0 0.0 0.0
2 -3.0 -3.0 -6.0 0.0 0.0 0.0
end initialstress
hydrostatic hydro.dat
end mesh
nl 3 1.0d-5 2
dt 10.0
setpnode nodes.dat
loop 2
solv
pnup
next
stop
"""


def _write_current(tmp):
    files = {
        "deck.dat": CURRENT,
        "solver.dat": "name gmres\nit 300\ntol 1.0d-9\nprecond diagm\nnkrylov 60\nend\n",
        "gravity.dat": "0.0 0.0 -10.0 10.0\n",
        "coor.dat": "coordinates\n" + "".join(
            "%d %g %g %g\n" % (i + 1, (i in (1, 2, 5, 6)), (i in (2, 3, 6, 7)), -(i >= 4))
            for i in range(8)) + "end coordinates\nreturn\n",
        "load1.dat": "4 2\n0.0 0.0 0.0 -1.0\n100.0 0.0 0.0 -2.0\n",
        "hydro.dat": "1.0d-3 0.5 0.0 1.0\n",
        "nodes.dat": "2\n1 5\n",
    }
    for k, v in files.items():
        with open(os.path.join(tmp, k), "w") as fh:
            fh.write(v)
    return os.path.join(tmp, "deck.dat")


def test_current_syntax_deck(tmp_path):
    d = Deck(_write_current(str(tmp_path)))
    pb = d.problem()
    # settings: solver file, nl, dt, gravity file
    assert (pb["solver"], pb["maxit"], pb["solvtol"], pb["precond"], pb["nkrylov"]) == (
        2, 300, 1e-9, 5, 60)
    assert (pb["maxnlit"], pb["tol"], pb["stop_crit"], pb["dt"]) == (3, 1e-5, 2, 10.0)
    assert np.array_equal(pb["gravity"], [0.0, 0.0, -10.0])
    # one hexa8 made hexa20: 12 mid-side nodes numbered after the vertices
    assert pb["nnode"] == 20 and pb["nnodev"] == 8
    assert list(pb["ix"][0, 8:20]) == list(range(9, 21)) and pb["ix"][0, 20] == 1
    x = pb["x"]
    assert np.allclose(x[8], 0.5 * (x[0] + x[1]))  # edge (1, 2) -> node 9
    # restraints of the top face propagate to its mid-side nodes (edges 1-4)
    top_mid = [8, 9, 10, 11]
    assert np.all(pb["id"][top_mid, :3] == 1) and not pb["id"][12:, :3].any()
    # nodal forces: the mid-side node of edge (1, 2) takes the average where
    # both vertices are restrained, and boundc copies them into u0
    assert pb["f"][8, 2] == 0.5 * (-1.0e-3 - 3.0e-3)
    assert pb["u0"][8, 2] == pb["f"][8, 2] and pb["u0"][0, 2] == -1.0e-3
    # loads: a type-40 table from a file, a type-2 load inline
    load = pb["load"]
    assert list(load[0]) == [40, 4, 2] and list(load[1]) == [2, 1, 1]
    assert pb["fload"].shape == (2, 6, 2)
    assert list(pb["fload"][0, :4, 1]) == [100.0, 0.0, 0.0, -2.0]
    # type 2, u(t) = a t + b: fload(1,1) = b, fload(2,1) = a (rows of column 1)
    assert list(pb["fload"][1, 0, :2]) == [0.5, 1.0e-3]
    # the pressure dof of node 5 carries nodal load 2, not restrained: u0 from
    # hydrostatic (density 1e-3, p0 0.5, datum 0, scale 1, |g| 10)
    assert pb["nload"][4, 3] == 2
    assert np.isclose(pb["u0"][4, 3], 0.5 + 1.0e-3 * 10.0 * (0.0 - x[4, 2]))
    # initial stress: mid-side nodes average their edge's vertices
    assert pb["fstress0"] == 1
    assert np.array_equal(pb["tx0"][8], 0.5 * (pb["tx0"][0] + pb["tx0"][1]))
    assert pb["eload"][0, 5] == 1
    assert list(pb["print_nodes"]) == [1, 5]
    assert d.value("nops") >= 5


def test_quadratic_input_and_nodal_load_at_t0(tmp_path):
    deck = """mesh
nnode 20 numel 1 numat 1 maxno 20 ndf 4 dim 3
materials
1 17 10.0 0.25 1.0d-6 5.0d4 1.0 0.0 1.0d3
end materials
hexa20
1 1 2 3 4 5 6 7 8
  9 10 11 12 13 14 15 16 17 18 19 20 1
end hexa20
coordinates
""" + "".join("%d %d.0 0.0 0.0\n" % (i + 1, i) for i in range(20)) + """end coordinates
constrainpmec
1 0 0 0 1
end constrainpmec
nodalloads
1 0 0 0 1
end nodalloads
loads
1 2 0.25 1.0
end loads
end mesh
stop
"""
    p = tmp_path / "q.dat"
    p.write_text(deck)
    d = Deck(str(p))
    pb = d.problem()
    assert pb["nnode"] == 20 and pb["nnodev"] == 8 and d.value("mk_quad") == 0
    assert list(pb["ix"][0, :20]) == list(range(1, 21))
    assert list(pb["fnno"]) == [1] * 8 + [0] * 12
    # bound_nodalloads: a restrained dof with a time load takes its t = 0 value
    assert pb["u0"][0, 3] == 0.25


@pytest.mark.parametrize("text,msg", [
    ("mesh\nnnode 8 numel 1 numat 1 maxno 20 ndf 4 dim 3\nconstrainpmec\n1 1 1 1 1\n"
     "end constrainpmec\nend mesh\n", "Unread Elements"),
    ("mesh\nnnode 8 numel 1 numat 1 maxno 20 ndf 4\n", "missing mesh parameter dim"),
    ("mesh\nnnode 8 numel 1 numat 1 maxno 20 ndf 4 dim 3\nmaterials\n1 17 1.0x\n",
     "expected a number"),
    ("mesh\nnnode 8 numel 1 numat 1 maxno 20 ndf 4 dim 3\ninsert nothere.dat\n", "not found"),
    ("loop 3\nsolv\n", "'loop' without 'next'"),
    ("mesh\nnnode 8 numel 1 numat 1 maxno 20 ndf 4 dim 3\nmaterials\n1 12 1.0\n"
     "end materials\nhexa8\n1 1 2 3 4 5 6 7 8 1\nend hexa8\nend mesh\n",
     "no elastic Biot element type"),
])
def test_errors_name_file_and_line(tmp_path, text, msg):
    p = tmp_path / "bad.dat"
    p.write_text(text)
    with pytest.raises(DeckError) as e:
        Deck(str(p))
    assert msg in str(e.value)
    if "not found" not in msg and "without 'next'" not in msg:
        assert "bad.dat:" in str(e.value)


@pytest.mark.parametrize("name", ["exemplo1_mesh0_t2", "solo1", "solo_cilindro_hexa_1",
                                  "solo_cilindro_tetra_1"])
def test_geometry_vtk_matches_the_golden_file(golden, tmp_path, name):
    """pgeo (write_mesh_geo_pm, Write_vtk.f:210-700) against the _bc.vtk the
    reference wrote for the same deck (its fields stored in the fixture by
    make_golden.py): the vertex mesh, node ids, initial pressures and
    restraint flags, cell materials, ids and element loads.  Values are
    printed with 5 digits (e15.5) by both writers."""
    fx = golden(name)
    d = Deck(write_linear_deck(fx, str(tmp_path), name))
    g = read_vtk(d.write_geo(os.path.join(str(tmp_path), name)))
    assert np.array_equal(g["points"], fx["vtk_points"])
    assert np.array_equal(np.stack(g["cells"]), fx["vtk_cells"])
    assert np.array_equal(g["cell_types"], fx["vtk_types"])
    for k in fx:
        if k.startswith("vtkp_"):
            assert np.array_equal(g["point_data"][k[5:]], fx[k]), k
        elif k.startswith("vtkc_"):
            assert np.array_equal(g["cell_data"][k[5:]], fx[k]), k


def test_quadratic_geometry_vtk(golden, tmp_path):
    fx = golden("exemplo1_mesh0_t2")
    d = Deck(write_linear_deck(fx, str(tmp_path), "q"))
    g = read_vtk(d.write_geo(os.path.join(str(tmp_path), "q"), quad=True))
    assert g["points"].shape == (int(fx["nnode"]), 3)
    assert set(g["cell_types"]) == {25}
    # VTK quadratic hexahedron order (elm_vtk): top face first, then its edges
    ix = fx["ix"][0]
    order = [5, 6, 7, 8, 1, 2, 3, 4, 13, 14, 15, 16, 9, 10, 11, 12, 17, 18, 19, 20]
    assert list(g["cells"][0]) == [ix[k - 1] - 1 for k in order]
    p = g["point_data"]["initialpres"][:, 0]
    for a, b, c in [(1, 2, 9), (4, 1, 12)]:
        na, nb, nc = ix[a - 1] - 1, ix[b - 1] - 1, ix[c - 1] - 1
        assert abs(p[nc] - 0.5 * (p[na] + p[nb])) <= 1e-5 * max(1e-3, abs(p[nc]))
