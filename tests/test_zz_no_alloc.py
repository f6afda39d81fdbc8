"""The solve that allocates no device memory (pm_pcg_csrd_noalloc).

Some callers cannot allocate device memory while they solve: a driver whose
memory is owned by its own arena, or a framework that has reserved the device
pool.  This entry point takes all its scratch from a fixed array inside the
library, so the test checks that it gives the same answer as the regular
solve (pm_solve), twice in a row on the same shared scratch, and that it
refuses a system larger than that array.  The file sorts last so that a run
stopping at its first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import poromec_gb300 as pg  # noqa: E402
from poromec_gb300 import meshgen  # noqa: E402

PM_NOALLOC_MAX_NEQ = 262144
PM_E_TOO_LARGE = 10


def _fn():
    lib = pg.load()
    f = lib.pm_pcg_csrd_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 6 + [ctypes.c_double, ctypes.c_int,
                                                             ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_noalloc_solve_matches_pm_solve_twice():
    pb = meshgen.column_problem()
    m = pg.from_problem(pb)
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    ia, ja, ad, al = m.get_csrd()
    dev = {k: torch.from_numpy(v).cuda() for k, v in dict(ia=ia, ja=ja, ad=ad, al=al).items()}
    f = _fn()
    stream = torch.cuda.Stream()
    tol = 1e-10
    rng = np.random.default_rng(11)
    for call in range(2):
        b = rng.standard_normal(m.neq)
        x_ref, info = m.solve(b, solver=1, precond=2, tol=tol, maxit=100000)
        bt = torch.from_numpy(b).cuda()
        xt = torch.full_like(bt, float("nan"))
        its = ctypes.c_int(-1)
        torch.cuda.synchronize()
        st = f(m.neq, dev["ia"].data_ptr(), dev["ja"].data_ptr(), dev["ad"].data_ptr(),
               dev["al"].data_ptr(), bt.data_ptr(), xt.data_ptr(), tol, 100000,
               ctypes.byref(its), ctypes.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        assert st == 0, st
        x = xt.cpu().numpy()
        # the same PCG and stopping test as pm_solve; the products differ only in
        # summation order, so the solutions agree within the solve tolerance
        # amplified by the conditioning (the bar of the other solve tests)
        assert np.abs(x - x_ref).max() <= 1e4 * tol * np.abs(x_ref).max(), call
        assert its.value > 0


def _csrd_on_device(pb):
    m = pg.from_problem(pb)
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    ia, ja, ad, al = m.get_csrd()
    return m, {k: torch.from_numpy(v).cuda() for k, v in dict(ia=ia, ja=ja, ad=ad, al=al).items()}


def _call(f, neq, dev, b, tol, stream):
    bt = torch.from_numpy(b).cuda()
    xt = torch.full_like(bt, float("nan"))
    its = ctypes.c_int(-1)
    torch.cuda.synchronize()
    st = f(neq, dev["ia"].data_ptr(), dev["ja"].data_ptr(), dev["ad"].data_ptr(),
           dev["al"].data_ptr(), bt.data_ptr(), xt.data_ptr(), tol, 100000, ctypes.byref(its),
           ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return st, xt.cpu().numpy()


def test_noalloc_scratch_stays_usable_after_an_early_return_and_a_larger_system():
    """A call that stops at a zero diagonal (status 3, before its iterations)
    leaves the shared scratch usable: a normal solve of the same system, and
    then one of a smaller system on the larger one's leftovers, both match
    pm_solve."""
    f = _fn()
    stream = torch.cuda.Stream()
    tol = 1e-10
    rng = np.random.default_rng(5)
    big, dbig = _csrd_on_device(meshgen.column_problem())
    small, dsmall = _csrd_on_device(meshgen.column_problem(nz=10))
    assert small.neq < big.neq
    b = rng.standard_normal(big.neq)
    bad = dict(dbig, ad=dbig["ad"].clone())
    bad["ad"][7] = 0.0
    st, _ = _call(f, big.neq, bad, b, tol, stream)
    assert st == 3, st
    for m, dev in ((big, dbig), (small, dsmall)):
        b = rng.standard_normal(m.neq)
        x_ref, _ = m.solve(b, solver=1, precond=2, tol=tol, maxit=100000)
        st, x = _call(f, m.neq, dev, b, tol, stream)
        assert st == 0, st
        assert np.abs(x - x_ref).max() <= 1e4 * tol * np.abs(x_ref).max(), m.neq


def test_noalloc_rejects_systems_larger_than_its_scratch():
    f = _fn()
    its = ctypes.c_int(0)
    st = f(PM_NOALLOC_MAX_NEQ + 1, None, None, None, None, None, None, 1e-8, 10,
           ctypes.byref(its), None)
    assert st == PM_E_TOO_LARGE
