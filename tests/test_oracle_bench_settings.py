"""The benchmark's step settings carry the heterogeneous cube through all 50
steps of its load history (the 10-step traction ramp and the consolidation
after it) on the oracle: every step's nonlinear loop converges.

The settings are the ones bench.py times (the reference's nonlinear defaults
maxnlit 500 and tol 1e-4, Main.f:269-273, stop_crit 1, diagonal PCG to
1e-10).  CPU only: the oracle steps the 8^3 and 12^3 cubes."""
import os

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
