"""The oracle's timing build (-O3, FMA contraction), which bench.py times as
the CPU baseline, computes what the parity build computes: the same matrix,
products and solutions up to rounding."""
import numpy as np

import oracle
from poromec_gb300 import meshgen


def _make(pb, timing):
    o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                      int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"],
                      pb["e"], timing=timing)
    o.set_loads(eload=pb["eload"], load=pb["load"], fload=pb["fload"])
    o.set_env(pb["gravity"], float(pb["dt"]))
    o.set_state(u=pb["u0"], u0=pb["u0"])
    return o


def test_timing_build_matches_the_parity_build():
    rng = np.random.default_rng(21)
    for pb in (meshgen.cube_problem(n=4), meshgen.tetra_problem(n=3)):
        a, b = _make(pb, False), _make(pb, True)
        assert a._L is not b._L
        du = rng.standard_normal((a.nnode, 4)) * 1e-3
        ba, bb = a.pform(2, True, True, du, np.zeros(a.neq)), b.pform(2, True, True, du,
                                                                        np.zeros(b.neq))
        _, _, ada, ala = a.get_csrd()
        _, _, adb, alb = b.get_csrd()
        scale = max(np.abs(ada).max(), np.abs(ala).max())
        assert np.abs(ada - adb).max() <= 1e-12 * scale
        assert np.abs(ala - alb).max() <= 1e-12 * scale
        assert np.abs(ba - bb).max() <= 1e-11 * max(1.0, np.abs(ba).max())
        x = rng.standard_normal(a.neq)
        ya = a.matvec(x, nthreads=2)
        assert np.abs(b.matvec(x, nthreads=2) - ya).max() <= 1e-12 * np.abs(ya).max()
        rhs = rng.standard_normal(a.neq)
        xa, _ = a.solve(rhs, tol=1e-10, maxit=100000)
        xb, _ = b.solve(rhs, tol=1e-10, maxit=100000)
        assert np.abs(xa - xb).max() <= 1e4 * 1e-10 * np.abs(xa).max()
