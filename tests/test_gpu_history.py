"""Whole load histories of the benchmark's workloads: GPU against the oracle.

bench.py times the heterogeneous hexa20 cube with the reference's nonlinear
defaults (maxnlit 500, tol 1e-4, Main.f:269-273) and stop_crit 1, diagonal
PCG to 1e-10, and the unstructured tetra10 box with PCG (and rpsqmr) under
the same settings.  These tests run the same generators and settings on smaller
meshes through every step of the load history (the cube's 10-step traction
ramp and the consolidation after it, 50 steps; 30 steps of the tetra box's
point source), on the GPU and on the oracle, step by step.

Bars.  Both sides run the same recurrences and differ only in summation
order (node panels against CSRD rows).  Under a stopping test at 1e-10 two
correct runs stop at different iterates: two oracle runs of the 12^3 cube
that differ only in the summation order of the OpenMP SpMV (1 and 8 threads)
differ by up to 6.6e-9 of max |p| in one ramp step (684 against 688
iterations) and by 1e-14 after the ramp.  At the bench tolerance the bar is
therefore 5e-8 (500 x the PCG tolerance) of max |u| and max |p| per step,
with the same number of nonlinear iterations in every step and the PCG
iterations within 3 % on average (FP64).  The 1e-10 bar of the plain FP64 path
holds where the solver resolves it: the first 12 steps (the ramp and two
steps after it) with PCG to 1e-13, where the two oracle runs above differ
by at most 2.2e-11.  The compensated operator in FP64 refinement
(PM_FP32C_REFINE) meets the same bars against the FP64 oracle.
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import poromec_gb300 as pg  # noqa: E402
from poromec_gb300 import meshgen  # noqa: E402

BENCH = dict(maxnlit=500, tol=1e-4, stop_crit=1, precond=2, solvtol=1e-10, maxit=200000)
TIGHT = dict(BENCH, solvtol=1e-13)
THREADS = os.cpu_count()
# mean Krylov iterations per step against the oracle's: within 3 % in FP64.
# PCG on the compensated operator replaces its residual by the FP64 one and
# goes on (a few per cent more); rpsqmr on it restarts for each correction
# sweep, which costs up to 65 % more iterations on the tetra box at 1e-10
ITS_BAR = {(1, pg.capi.PM_FP64): 0.03, (1, pg.capi.PM_FP32C_REFINE): 0.1,
           (11, pg.capi.PM_FP64): 0.03, (11, pg.capi.PM_FP32C_REFINE): 1.0}
# on the two-layer tetra box (1e2 contrast in k) the compensated operator's
# 2^-32 per entry costs PCG up to ~20 % more iterations at 48^3
TETRA_ITS_BAR = {(1, pg.capi.PM_FP32C_REFINE): 0.25}


def _oracle(pb):
    o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                      int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"], pb["e"])
    o.set_loads(eload=pb.get("eload"), nload=pb.get("nload"), load=pb["load"],
                fload=pb["fload"])
    o.set_env(pb["gravity"], float(pb["dt"]))
    o.set_state(u=pb["u0"], u0=pb["u0"])
    return o


def _oracle_history(pb, steps, solver, kw):
    o = _oracle(pb)
    hist = []
    for _ in range(steps):
        info = o.step(solver=solver, nthreads=THREADS, **kw)
        u, _, _ = o.get_state()
        hist.append((u, info.nlit, info.iters))
    return hist


def _gpu_history(pb, steps, solver, kw, mode=pg.capi.PM_FP64):
    m = pg.from_problem(pb)
    m.set_precision(mode)
    hist = []
    for _ in range(steps):
        info = m.step(solver=solver, **kw)
        u, _, _ = m.get_state()
        hist.append((u, info.nlit, int(m.timers()[4])))
    m.close()
    return hist


def _compare(gpu, ref, bar, its_bar):
    worst = [0.0, 0.0]
    its_g, its_o = [], []
    for k, ((ug, nlg, itg), (uo, nlo, ito)) in enumerate(zip(gpu, ref)):
        assert nlg == nlo, (k + 1, nlg, nlo)
        eu = np.abs(ug[:, :3] - uo[:, :3]).max() / np.abs(uo[:, :3]).max()
        ep = np.abs(ug[:, 3] - uo[:, 3]).max() / np.abs(uo[:, 3]).max()
        worst = [max(worst[0], eu), max(worst[1], ep)]
        assert eu <= bar and ep <= bar, (k + 1, eu, ep)
        its_g.append(itg)
        its_o.append(ito)
    if its_bar is not None:
        # the oracle's count is that of the step's last solve; with one solve
        # per step (nlit 2) it is the step's total
        rel = abs(np.mean(its_g) - np.mean(its_o)) / np.mean(its_o)
        assert rel <= its_bar, (rel, its_g, its_o)
    return worst


@pytest.fixture(scope="module")
def cube16():
    pb = meshgen.cube_problem(16)
    return pb, _oracle_history(pb, 50, 1, BENCH)


@pytest.mark.parametrize("mode", [pg.capi.PM_FP64, pg.capi.PM_FP32C_REFINE])
def test_cube_history_bench_settings(cube16, mode):
    """The 16^3 cube, 50 steps with the bench's settings (PCG 1e-10)."""
    pb, ref = cube16
    gpu = _gpu_history(pb, 50, 1, BENCH, mode)
    worst = _compare(gpu, ref, 500 * BENCH["solvtol"], ITS_BAR[1, mode])
    print("cube 16^3, 50 steps, mode %d: max rel. difference u %.2e p %.2e" % (mode, *worst))


@pytest.mark.parametrize("mode,bar", [(pg.capi.PM_FP64, 1e-10), (pg.capi.PM_FP32C_REFINE, 1e-8)])
def test_cube_history_tight_tolerance(mode, bar):
    """The 12^3 cube's ramp (12 steps) with PCG to 1e-13: the FP64 path
    within 1e-10, the compensated operator within 1e-8 of the FP64 oracle."""
    pb = meshgen.cube_problem(12)
    ref = _oracle_history(pb, 12, 1, TIGHT)
    gpu = _gpu_history(pb, 12, 1, TIGHT, mode)
    worst = _compare(gpu, ref, bar, None)
    print("cube 12^3, 12 steps at 1e-13, mode %d: u %.2e p %.2e" % (mode, *worst))


@pytest.fixture(scope="module")
def tetra8():
    pb = meshgen.tetra_problem(8)
    return pb, {}


@pytest.mark.parametrize("solver", [1, 11])
@pytest.mark.parametrize("mode", [pg.capi.PM_FP64, pg.capi.PM_FP32C_REFINE])
def test_tetra_history_bench_settings(tetra8, mode, solver):
    """The jittered two-layer tetra10 box at 8^3 x 6 with its point source,
    30 steps of pcg (the bench's tetra solver) and of rpsqmr with the bench's
    settings."""
    pb, refs = tetra8
    if solver not in refs:
        refs[solver] = _oracle_history(pb, 30, solver, BENCH)
    gpu = _gpu_history(pb, 30, solver, BENCH, mode)
    its_bar = TETRA_ITS_BAR.get((solver, mode), ITS_BAR[solver, mode])
    worst = _compare(gpu, refs[solver], 500 * BENCH["solvtol"], its_bar)
    print("tetra 8^3, 30 steps, solver %d, mode %d: u %.2e p %.2e" % (solver, mode, *worst))


def test_tetra_history_tight_tolerance():
    """rpsqmr on the 6^3 tetra box to 1e-13 for 6 steps: within 1e-10."""
    pb = meshgen.tetra_problem(6)
    ref = _oracle_history(pb, 6, 11, TIGHT)
    gpu = _gpu_history(pb, 6, 11, TIGHT)
    worst = _compare(gpu, ref, 1e-10, None)
    print("tetra 6^3, 6 steps at 1e-13: u %.2e p %.2e" % tuple(worst))
