"""The benchmark's step settings carry the heterogeneous cube through all 50
steps of its load history (the 10-step traction ramp and the consolidation
after it) on the oracle: every step's nonlinear loop converges.

The settings are the ones bench.py times (the reference's nonlinear defaults
maxnlit 500 and tol 1e-4, Main.f:269-273, stop_crit 1, diagonal PCG to
1e-10).  CPU only: the oracle steps the 8^3 and 12^3 cubes, and the 8^3
tetra box with the tetra workload's solver."""
import os

import numpy as np
import pytest

import oracle
import bench
from poromec_gb300 import meshgen


@pytest.mark.parametrize("n", [8, 12])
def test_cube_steps_converge_with_bench_settings(n):
    kw = bench.step_kwargs(bench.parse([]))
    kw.pop("reassemble")  # the oracle re-assembles every nonlinear iteration 1
    pb = meshgen.cube_problem(n)
    o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                      int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"],
                      pb["e"])
    o.set_loads(eload=pb["eload"], load=pb["load"], fload=pb["fload"])
    o.set_env(pb["gravity"], float(pb["dt"]))
    o.set_state(u=pb["u0"], u0=pb["u0"])
    nlit = []
    for _ in range(50):
        info = o.step(nthreads=os.cpu_count(), **kw)  # raises if a step does not converge
        nlit.append(info.nlit)
    # one solve per step (the second nonlinear iteration accepts it)
    assert max(nlit) == 2, nlit


def test_tetra_steps_pcg_matches_rpsqmr():
    """The tetra workload's solver (pcg, bench.py's --tetra-solver default)
    carries the jittered two-layer tetra10 box through 30 steps of its point
    source with the bench's settings, one solve per step, and ends where
    rpsqmr (the reference's default solver) ends, within 500 x the solver
    tolerance; it takes fewer iterations.  Oracle, 8^3 x 6 tets."""
    args = bench.parse([])
    assert args.tetra_solver == 1
    pb = meshgen.tetra_problem(8)
    states, its = {}, {}
    for solver in (1, 11):
        kw = bench.step_kwargs(args, solver=solver)
        kw.pop("reassemble")
        o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]),
                          int(pb["nen"]), int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"],
                          pb["x"], pb["ie"], pb["e"])
        o.set_loads(eload=pb["eload"], load=pb["load"], fload=pb["fload"])
        o.set_env(pb["gravity"], float(pb["dt"]))
        o.set_state(u=pb["u0"], u0=pb["u0"])
        total = 0
        for _ in range(30):
            info = o.step(nthreads=os.cpu_count(), **kw)
            assert info.nlit == 2
            total += info.iters
        states[solver], _, _ = o.get_state()
        its[solver] = total
    u1, u11 = states[1], states[11]
    for sl in (slice(0, 3), slice(3, 4)):
        ref = np.abs(u11[:, sl]).max()
        assert np.abs(u1[:, sl] - u11[:, sl]).max() <= 500 * kw["solvtol"] * ref
    assert its[1] < its[11], its
