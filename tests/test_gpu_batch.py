"""Batched solver: a batch of independent meshes in one handle gives each
instance the result it gets alone on its own handle.

Each instance runs its own PCG (own scalars, stopping test and nonlinear
test); only the launches are shared.  The per-instance dot products are
summed in a different order than a single handle's, so iteration counts
may differ by rounding; solutions agree within the solver tolerance times
the conditioning (the bars below).  The batch is also checked against the
oracle stepping each instance alone (the reference's algorithm on the CPU)."""
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


@pytest.fixture(scope="module")
def instances():
    return meshgen.batch_instances(ninst=5, nmin=2, nmax=5, seed=11)


def _split(u, ptr):
    return [u[ptr[k]:ptr[k + 1]] for k in range(len(ptr) - 1)]


def test_batch_layout(instances):
    pb = meshgen.union_problem(instances)
    m = pg.from_problem(pb)
    assert m.ninst == len(instances)
    assert m.neq == sum(pg.from_problem(p).neq for p in instances)


@pytest.mark.parametrize("precision", [pg.capi.PM_FP64, pg.capi.PM_FP32C_REFINE])
def test_batch_solve_matches_single(instances, precision):
    pb = meshgen.union_problem(instances)
    mb = pg.from_problem(pb)
    mb.set_precision(precision)
    mb.pform(2, True, False, np.zeros((mb.nnode, 4)), None)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(mb.neq)
    tol = 1e-11
    xb, info = mb.solve(b, solver=1, precond=2, tol=tol, maxit=100000)
    its, _ = mb.batch_iters()
    off = 0
    for k, p in enumerate(instances):
        ms = pg.from_problem(p)
        ms.set_precision(precision)
        ms.pform(2, True, False, np.zeros((ms.nnode, 4)), None)
        bs = b[off:off + ms.neq]
        xs, si = ms.solve(bs, solver=1, precond=2, tol=tol, maxit=100000)
        xk = xb[off:off + ms.neq]
        assert np.abs(xk - xs).max() <= 1e4 * tol * np.abs(xs).max(), k
        assert its[k] > 0 and abs(int(its[k]) - si.iters) <= max(3, si.iters // 5)
        off += ms.neq
    assert info.iters == its.max()


@pytest.mark.parametrize("precision", [pg.capi.PM_FP64, pg.capi.PM_FP32C_REFINE])
def test_batch_steps_match_single(instances, precision):
    pb = meshgen.union_problem(instances)
    mb = pg.from_problem(pb)
    mb.set_precision(precision)
    singles = [pg.from_problem(p) for p in instances]
    for ms in singles:
        ms.set_precision(precision)
    kw = dict(maxnlit=2, stop_crit=1, solvtol=1e-11, maxit=100000)
    for step in range(3):
        ib = mb.step(**kw)
        for ms in singles:
            ms.step(**kw)
        _, nl = mb.batch_iters()
        assert ib.nlit == nl.max() and (nl >= 1).all()
    ub, _, _ = mb.get_state()
    for k, (ms, part) in enumerate(zip(singles, _split(ub, pb["inst_node_ptr"]))):
        us, _, _ = ms.get_state()
        for sl in (slice(0, 3), slice(3, 4)):
            ref = us[:, sl]
            assert np.abs(part[:, sl] - ref).max() <= 1e-8 * np.abs(ref).max(), (k, sl)


@pytest.mark.parametrize("precision,bar", [(pg.capi.PM_FP64, 1e-10),
                                           (pg.capi.PM_FP32C_REFINE, 1e-8)])
def test_batch_steps_match_oracle(precision, bar):
    """Eight instances of uneven size (edges 2..6, own E and k) stepped three
    times in one handle, against the oracle stepping each instance alone:
    every instance stops at the oracle's nonlinear iteration, and u and p
    agree within 1e-10 (FP64) or 1e-8 (compensated operator in FP64
    refinement) of their largest value.  PCG runs to 1e-13, where the solver
    resolves these bars."""
    inst = meshgen.batch_instances(ninst=8, nmin=2, nmax=6, seed=23)
    assert len({p["n"] for p in inst}) > 2
    pb = meshgen.union_problem(inst)
    mb = pg.from_problem(pb)
    mb.set_precision(precision)
    kw = dict(maxnlit=500, tol=1e-4, stop_crit=1, precond=2, solvtol=1e-13, maxit=200000)
    orcs = []
    for p in inst:
        o = oracle.Oracle(int(p["nnode"]), int(p["nnodev"]), int(p["numel"]), int(p["nen"]),
                          int(p["nenv"]), p["ix"], p["id"], p["fnno"], p["x"], p["ie"], p["e"])
        o.set_loads(eload=p["eload"], load=p["load"], fload=p["fload"])
        o.set_env(p["gravity"], float(p["dt"]))
        o.set_state(u=p["u0"], u0=p["u0"])
        orcs.append(o)
    for step in range(3):
        mb.step(solver=1, **kw)
        _, nl = mb.batch_iters()
        for k, o in enumerate(orcs):
            info = o.step(solver=1, nthreads=os.cpu_count(), **kw)
            assert nl[k] == info.nlit, (step, k, nl[k], info.nlit)
    ub, _, _ = mb.get_state()
    for k, (o, part) in enumerate(zip(orcs, _split(ub, pb["inst_node_ptr"]))):
        uo, _, _ = o.get_state()
        for sl in (slice(0, 3), slice(3, 4)):
            ref = uo[:, sl]
            assert np.abs(part[:, sl] - ref).max() <= bar * np.abs(ref).max(), (k, sl)


def _steps(pb, precision, host_loop, steps, **kw):
    """A batch stepped `steps` times by the device-driven step graph or by the
    host loop (PM_BATCH_HOST_STEP); returns the state, per-instance counts,
    step infos (or the PMError of a failed step) and timers."""
    old = os.environ.pop("PM_BATCH_HOST_STEP", None)
    try:
        if host_loop:
            os.environ["PM_BATCH_HOST_STEP"] = "1"
        m = pg.from_problem(pb)
        m.set_precision(precision)
        out = []
        for _ in range(steps):
            try:
                i = m.step(**kw)
                out.append((i.nlit, i.iters, i.refine, m.batch_iters(), m.timers()))
            except pg.PMError as e:
                out.append((e.status, str(e)))
                break
        u = m.get_state()
        m.close()
        return u, out
    finally:
        os.environ.pop("PM_BATCH_HOST_STEP", None)
        if old is not None:
            os.environ["PM_BATCH_HOST_STEP"] = old


@pytest.mark.parametrize("precision,stop_crit", [(pg.capi.PM_FP64, 1),
                                                  (pg.capi.PM_FP32C_REFINE, 1),
                                                  (pg.capi.PM_FP64, 2)])
def test_batch_step_graph_matches_host_loop(instances, precision, stop_crit, monkeypatch):
    """The batch step as one CUDA graph (conditional nodes for the nonlinear
    loop, the refinement sweeps and the PCG iterations, decided on the
    device) runs the host loop's kernels in the host loop's order: the same
    state bit for bit, the same per-instance iterations and nonlinear
    counts, under both stop tests of cal_residuo_pm (with stop_crit 2 some of
    these instances stop at the nonlinear limit within a few steps, as they do
    on the oracle: both drivers fail the same step with the same status).
    The compensated SpMV shape is fixed so both handles run the same kernel
    (the autotuner times kernels)."""
    monkeypatch.setenv("PM_SPMV_SHAPE", "314")
    pb = meshgen.union_problem(instances)
    kw = dict(maxnlit=500, tol=1e-4, stop_crit=stop_crit, solver=1, precond=2, solvtol=1e-11,
              maxit=100000)
    ug, og = _steps(pb, precision, False, 4, **kw)
    uh, oh = _steps(pb, precision, True, 4, **kw)
    for a, b in zip(ug, uh):
        assert np.array_equal(a, b)
    assert len(og) == len(oh)
    graph_steps = done = 0
    for g, h in zip(og, oh):
        if len(g) == 2 or len(h) == 2:  # a failed step: the same status and message
            assert g == h
            continue
        (gl, gi, gr, (git, gnl), gt), (hl, hi, hr, (hit, hnl), ht) = g, h
        assert (gl, gi, gr) == (hl, hi, hr)
        assert np.array_equal(git, hit) and np.array_equal(gnl, hnl)
        assert ht[0] > 0.0  # the host loop times its phases
        graph_steps += gt[0] == 0.0 and gt[3] > 0.0  # the graph: one time for the step
        done += 1
    # the compensated handle's first step tunes and splits on the host loop
    assert done >= 1
    assert graph_steps == done - (precision == pg.capi.PM_FP32C_REFINE)


@pytest.mark.parametrize("case", ["maxnlit", "maxit"])
def test_batch_step_graph_errors_match_host_loop(instances, case):
    """Failures decided on the device give the host loop's status, message
    and state: the nonlinear limit (maxnlit 1 with an unreachable test) and
    the PCG iteration limit (maxit 3)."""
    pb = meshgen.union_problem(instances)
    kw = dict(maxnlit=500, tol=1e-4, stop_crit=1, solver=1, precond=2, solvtol=1e-11,
              maxit=100000)
    if case == "maxnlit":
        kw.update(maxnlit=1, tol=1e-30)
        status = 5
    else:
        kw.update(maxit=3)
        status = 4
    ug, og = _steps(pb, pg.capi.PM_FP64, False, 2, **kw)
    uh, oh = _steps(pb, pg.capi.PM_FP64, True, 2, **kw)
    assert og[-1] == oh[-1] and og[-1][0] == status
    for a, b in zip(ug, uh):
        assert np.array_equal(a, b)


def test_batch_rejects_minres(instances):
    mb = pg.from_problem(meshgen.union_problem(instances))
    mb.pform(2, True, False, np.zeros((mb.nnode, 4)), None)
    with pytest.raises(pg.PMError) as e:
        mb.solve(np.ones(mb.neq), solver=7, precond=5)
    assert e.value.status == 1
