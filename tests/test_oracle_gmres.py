"""The oracle's GMRES(l) (gmres2, Iters.f:1411-1700) and the rpsqmr ->
GMRES(l) switch of solv_pm (Solv.f:707-766).

No golden run uses GMRES (the decks select PCG), so these are properties of
the restated algorithm: its stopping test |M (b - A x)| <= tol |M b| on the
implicit residual, agreement with a dense direct solve, restarts with a small
basis, the cycle limit, and the fallback starting GMRES(l) from x = 0.
"""
import numpy as np
import pytest

import oracle


def _system(fx):
    o = oracle.from_fixture(fx)
    b = np.zeros(o.neq)
    o.pform(2, True, False, np.zeros((o.nnode, 4)), b)
    ia, ja, ad, al = o.get_csrd()
    A = np.diag(ad)
    for r in range(o.neq):
        for p in range(ia[r] - 1, ia[r + 1] - 1):
            c = ja[p] - 1
            A[r, c] = al[p]
            A[c, r] = al[p]
    return o, A, ad


@pytest.mark.parametrize("name", ["exemplo1_mesh0_t2", "exemplo1_mesh0_t2_tetra"])
@pytest.mark.parametrize("precond", [2, 5])
def test_gmres_solves_golden_systems(golden, name, precond):
    o, A, ad = _system(golden(name))
    b = np.random.default_rng(2).standard_normal(o.neq)
    tol = 1e-11
    x, info = o.solve(b, solver=2, precond=precond, tol=tol, maxit=1000)
    m = 1.0 / ad if precond == 2 else np.abs(1.0 / ad)
    assert np.linalg.norm(m * (b - A @ x)) <= 10 * tol * np.linalg.norm(m * b)
    xd = np.linalg.solve(A, b)
    assert np.abs(x - xd).max() <= 1e4 * tol * np.abs(xd).max()
    assert 0 < info.iters <= 150 * 1000


def test_gmres_restarts_and_cycle_limit(golden):
    o, A, _ = _system(golden("exemplo1_mesh0_t2"))
    b = np.random.default_rng(3).standard_normal(o.neq)
    x150, i150 = o.solve(b, solver=2, tol=1e-10, maxit=1000)
    # 160 equations: 150 directions converge in one cycle; a basis of 30
    # needs about ten restarts (GMRES(10) stagnates on this indefinite system)
    o.set_nkrylov(30)
    x30, i30 = o.solve(b, solver=2, tol=1e-10, maxit=1000)
    assert i30.iters > 2 * 30 and i30.iters > i150.iters
    assert np.abs(x30 - x150).max() <= 1e-5 * np.abs(x150).max()
    with pytest.raises(oracle.OracleError):
        o.solve(b, solver=2, tol=1e-10, maxit=1)


def test_rpsqmr_falls_back_to_gmres(golden):
    o, A, _ = _system(golden("exemplo1_mesh0_t2"))
    b = np.random.default_rng(4).standard_normal(o.neq)
    xg, ig = o.solve(b, solver=2, tol=1e-11, maxit=10)
    xs, isq = o.solve(b, solver=11, tol=1e-11, maxit=10)
    # rpsqmr stops at maxit = 10, then GMRES(l) restarts from x = 0
    assert np.array_equal(xs, xg)
    assert isq.iters == 10 + ig.iters
    xc, ic = o.solve(b, solver=11, tol=1e-11, maxit=100000)
    assert ic.iters < 100000
    assert np.abs(xc - xg).max() <= 1e-6 * np.abs(xg).max()
