"""Batched solver: a batch of independent meshes in one handle gives each
instance the result it gets alone on its own handle.

Each instance runs its own PCG (own scalars, stopping test and nonlinear
test); only the launches are shared.  The per-instance dot products are
summed in a different order than a single handle's, so iteration counts
may differ by rounding; solutions agree within the solver tolerance times
the conditioning (the bars below)."""
import numpy as np
import pytest

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


def test_batch_rejects_minres(instances):
    mb = pg.from_problem(meshgen.union_problem(instances))
    mb.pform(2, True, False, np.zeros((mb.nnode, 4)), None)
    with pytest.raises(pg.PMError) as e:
        mb.solve(np.ones(mb.neq), solver=7, precond=5)
    assert e.value.status == 1
