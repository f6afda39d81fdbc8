"""GPU parity: the C-ABI library against the CPU oracle and the reference's
golden runs.

Tolerances: index work (equation numbers, CSRD ia/ja) is compared bit for
bit; FP64 assembly entries within 1e-12 of the matrix's largest entry in the
row block; solutions within 1e-10 relative (the plain FP64 bar); golden node
histories within 1e-10 absolute (the reference prints 10 decimals).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import poromec_gb300 as pg  # noqa: E402
from poromec_gb300 import meshgen  # noqa: E402

GOLDEN_CASES = ["exemplo1_mesh0_t2", "exemplo1_mesh0_t2_tetra"]


def _pair(pb):
    m = pg.from_problem(pb)
    o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                      int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"], pb["e"])
    has = "load" in pb and len(pb["load"]) > 0
    o.set_loads(eload=pb.get("eload"), nload=pb.get("nload"),
                load=pb["load"] if has else None, fload=pb["fload"] if has else None)
    o.set_env(pb["gravity"], float(pb["dt"]))
    o.set_state(u=pb["u0"], u0=pb["u0"])
    return m, o


def _problems(golden):
    out = [golden(n) for n in GOLDEN_CASES]
    out.append(meshgen.column_problem())
    out.append(meshgen.tetra_problem(n=3))
    c = meshgen.cube_problem(n=4)
    out.append(c)
    return out


@pytest.fixture(scope="module")
def problems(golden):
    return _problems(golden)


def test_numbering_and_pattern_bit_exact(problems):
    for pb in problems:
        m, o = _pair(pb)
        assert m.neq == o.neq and m.nad == o.nad
        assert np.array_equal(m.get_id(), o.get_id())
        ia, ja, _, _ = m.get_csrd(values=False)
        ia_o, ja_o, _, _ = o.get_csrd()
        assert np.array_equal(ia, ia_o)
        assert np.array_equal(ja, ja_o)


def test_assembly_matches_oracle(problems):
    rng = np.random.default_rng(0)
    for pb in problems:
        m, o = _pair(pb)
        du = rng.standard_normal((m.nnode, 4)) * 1e-3
        b = rng.standard_normal(m.neq)
        bg, bo = b.copy(), b.copy()
        m.pform(2, True, True, du, bg)
        o.pform(2, True, True, du, bo)
        _, _, ad, al = m.get_csrd()
        _, _, ado, alo = o.get_csrd()
        scale = max(np.abs(ado).max(), np.abs(alo).max())
        assert np.abs(ad - ado).max() <= 1e-12 * scale
        assert np.abs(al - alo).max() <= 1e-12 * scale
        assert np.abs(bg - bo).max() <= 1e-11 * max(1.0, np.abs(bo).max())


def test_fused_assembly_product_is_deterministic(problems):
    """pform with lhs and rhs takes b -= K_e u_e from the blocks it assembles:
    it matches the separate matrix-free pass within rounding, fills the same
    panels bit for bit, and repeats bit for bit (no atomics in the sums)."""
    rng = np.random.default_rng(5)
    for pb in problems:
        m = pg.from_problem(pb)
        u = rng.standard_normal((m.nnode, 4)) * 1e-3
        b0 = rng.standard_normal(m.neq)
        fused = [m.pform(2, True, True, u, b0.copy()) for _ in range(2)]
        _, _, ad_f, al_f = m.get_csrd()
        assert np.array_equal(fused[0], fused[1])
        m.pform(2, True, False, u, None)
        _, _, ad_s, al_s = m.get_csrd()
        sep = m.pform(2, False, True, u, b0.copy())
        assert np.array_equal(ad_f, ad_s) and np.array_equal(al_f, al_s)
        assert np.abs(fused[0] - sep).max() <= 1e-12 * max(1.0, np.abs(b0 - sep).max())


def test_rhs_isw4_matches_oracle(problems):
    rng = np.random.default_rng(1)
    for pb in problems:
        m, o = _pair(pb)
        u = pb["u0"] + rng.standard_normal((m.nnode, 4)) * 1e-3
        dp = rng.standard_normal(m.nnode) * 1e-3
        m.set_state(dp=dp)
        o.set_state(dp=dp)
        b = np.zeros(m.neq)
        bg, bo = b.copy(), b.copy()
        m.pform(4, False, True, u, bg)
        o.pform(4, False, True, u, bo)
        assert np.abs(bg - bo).max() <= 1e-11 * max(1e-12, np.abs(bo).max())


def test_spmv_matches_oracle(problems):
    rng = np.random.default_rng(2)
    for pb in problems:
        m, o = _pair(pb)
        du = np.zeros((m.nnode, 4))
        m.pform(2, True, False, du, None)
        _, _, ad, al = m.get_csrd()
        o.set_csrd_values(ad, al)  # same values on both sides
        x = rng.standard_normal(m.neq)
        y = m.matvec(x)
        yo = o.matvec(x)
        assert np.abs(y - yo).max() <= 1e-13 * np.abs(yo).max()
        yo4 = o.matvec(x, nthreads=4)
        assert np.abs(yo4 - yo).max() <= 1e-13 * np.abs(yo).max()


def test_csrd_reference_layout_on_device(problems):
    pb = problems[0]
    m, o = _pair(pb)
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    ia, ja, ad, al = m.get_csrd()
    o.set_csrd_values(ad, al)
    x = np.random.default_rng(3).standard_normal(m.neq)
    t = {k: torch.from_numpy(v).cuda() for k, v in dict(ia=ia, ja=ja, ad=ad, al=al, x=x).items()}
    y = torch.empty(m.neq, dtype=torch.float64, device="cuda")
    pg.matvec_csrd_dev(m.neq, t["ia"].data_ptr(), t["ja"].data_ptr(), t["ad"].data_ptr(),
                       t["al"].data_ptr(), t["x"].data_ptr(), y.data_ptr(),
                       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    yo = o.matvec(x)
    assert np.abs(y.cpu().numpy() - yo).max() <= 1e-13 * np.abs(yo).max()


@pytest.mark.parametrize("solver,precond,tol,cases", [(1, 2, 1e-12, 3), (7, 5, 1e-10, 2)])
def test_solve_matches_oracle(problems, solver, precond, tol, cases):
    for pb in problems[:cases]:
        m, o = _pair(pb)
        m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
        _, _, ad, al = m.get_csrd()
        o.set_csrd_values(ad, al)
        b = np.random.default_rng(4).standard_normal(m.neq)
        x, info = m.solve(b, solver=solver, precond=precond, tol=tol, maxit=400000)
        xo, info_o = o.solve(b, solver=solver, precond=precond, tol=tol, maxit=400000)
        # both stop on the same preconditioned-residual test; on this
        # indefinite system the solution error is that tolerance times the
        # conditioning, so the bar is 1e4 * tol
        assert np.abs(x - xo).max() <= 1e4 * tol * np.abs(xo).max()
        # Krylov iteration counts on this indefinite system follow rounding;
        # the solutions, not the counts, are the parity quantity
        assert info.iters > 0 and info_o.iters > 0


@pytest.mark.parametrize("precond", [2, 5])
def test_rpsqmr_matches_oracle(problems, precond):
    """rpsqmr (solver 11, Iters.f:6100-6439), the reference's default solver:
    GPU and oracle stop on the same test ||r|| < tol ||b||."""
    tol = 1e-10
    for pb in problems[2:]:
        m, o = _pair(pb)
        m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
        _, _, ad, al = m.get_csrd()
        o.set_csrd_values(ad, al)
        b = np.random.default_rng(8).standard_normal(m.neq)
        x, info = m.solve(b, solver=11, precond=precond, tol=tol, maxit=200000)
        xo, io = o.solve(b, solver=11, precond=precond, tol=tol, maxit=200000)
        assert np.abs(x - xo).max() <= 1e4 * tol * np.abs(xo).max()
        # iteration counts on these indefinite systems follow rounding (as for
        # PCG and MINRES above): the solutions are the parity quantity
        assert info.iters > 0 and io.iters > 0
        assert np.linalg.norm(b - m.matvec(x)) <= 1e2 * tol * np.linalg.norm(b)


@pytest.mark.parametrize("precond", [2, 5])
def test_gmres_matches_oracle(problems, precond):
    """GMRES(l) (solver 2, gmres2 Iters.f:1411-1700) with the default basis of
    150: GPU and oracle stop on the same test |e| <= tol |M b|.  The tetra10
    problem with |1/ad| takes two cycles (a restart).  The column with |1/ad|
    needs 77 cycles and is left to the oracle's own tests."""
    tol = 1e-10
    for i, pb in enumerate(problems):
        if precond == 5 and i == 2:
            continue
        m, o = _pair(pb)
        m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
        _, _, ad, al = m.get_csrd()
        o.set_csrd_values(ad, al)
        b = np.random.default_rng(8).standard_normal(m.neq)
        x, info = m.solve(b, solver=2, precond=precond, tol=tol, maxit=200)
        xo, io = o.solve(b, solver=2, precond=precond, tol=tol, maxit=200)
        assert np.abs(x - xo).max() <= 1e4 * tol * np.abs(xo).max(), i
        assert info.iters > 0 and abs(info.iters - io.iters) <= max(3, io.iters // 20), (
            i, info.iters, io.iters)
        mm = 1.0 / ad if precond == 2 else np.abs(1.0 / ad)
        assert np.linalg.norm(mm * (b - m.matvec(x))) <= 10 * tol * np.linalg.norm(mm * b)


def test_rpsqmr_falls_back_to_gmres_on_gpu(problems):
    """Solv.f:765: rpsqmr stopped at maxit switches to GMRES(l) from x = 0
    with maxit cycles; the iteration count covers both."""
    tol = 1e-10
    for pb in problems[2:]:
        m, o = _pair(pb)
        m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
        _, _, ad, al = m.get_csrd()
        o.set_csrd_values(ad, al)
        b = np.random.default_rng(8).standard_normal(m.neq)
        x, info = m.solve(b, solver=11, precond=2, tol=tol, maxit=10)
        xo, io = o.solve(b, solver=11, precond=2, tol=tol, maxit=10)
        xg, ig = m.solve(b, solver=2, precond=2, tol=tol, maxit=10)
        assert np.array_equal(x, xg)
        assert info.iters == 10 + ig.iters
        assert np.abs(x - xo).max() <= 1e4 * tol * np.abs(xo).max()


def test_gmres_steps_match_oracle():
    pb = meshgen.column_problem()
    m, o = _pair(pb)
    for k in range(3):
        m.step(maxnlit=2, stop_crit=1, solver=2, precond=2, solvtol=1e-10, maxit=200)
        o.step(maxnlit=2, stop_crit=1, solver=2, precond=2, solvtol=1e-10, maxit=200)
    u, _, _ = m.get_state()
    uo, _, _ = o.get_state()
    for sl in (slice(0, 3), slice(3, 4)):
        assert np.abs(u[:, sl] - uo[:, sl]).max() <= 1e-8 * np.abs(uo[:, sl]).max()


def test_rpsqmr_step_matches_oracle():
    """Steps of the consolidation column with the reference's default solver."""
    pb = meshgen.column_problem()
    m, o = _pair(pb)
    for k in range(5):
        m.step(maxnlit=2, stop_crit=1, solver=11, precond=2, solvtol=1e-10)
        o.step(maxnlit=2, stop_crit=1, solver=11, precond=2, solvtol=1e-10)
    u, _, _ = m.get_state()
    uo, _, _ = o.get_state()
    for sl in (slice(0, 3), slice(3, 4)):
        assert np.abs(u[:, sl] - uo[:, sl]).max() <= 1e-8 * np.abs(uo[:, sl]).max()


def test_solve_dev_torch_tensors(problems):
    pb = problems[2]
    m, o = _pair(pb)
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    b = np.random.default_rng(5).standard_normal(m.neq)
    x_ref, _ = m.solve(b, tol=1e-11)
    bt = torch.from_numpy(b).cuda()
    xt = torch.empty_like(bt)
    m.solve_dev(bt.data_ptr(), xt.data_ptr(), tol=1e-11,
                stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(xt.cpu().numpy(), x_ref)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_histories_on_gpu(golden, name):
    fx = golden(name)
    m = pg.from_problem(fx)
    worst = 0.0
    for k in range(1, 601):
        m.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]), maxit=int(fx["maxit"]))
        u, _, _ = m.get_state()
        for a, n in enumerate(fx["hist_nodes"]):
            worst = max(worst, np.abs(u[n - 1] - fx["hist"][a][k][2:6]).max())
    assert worst < 1e-10, worst


def test_rcm_numbering_pattern_and_values_match_oracle(problems):
    """reord true (the reference's default): with the node order of pm_reord
    (host) and of the oracle's or_reord, the equation numbers and the CSRD
    pattern are equal bit for bit, the assembled values within the assembly
    bar, and the order differs from the natural one."""
    rng = np.random.default_rng(4)
    for pb in problems:
        num = pg.reord(pb["nnode"], pb["numel"], pb["nen"], pb["ix"])
        num_o = oracle.reord(pb["nnode"], pb["numel"], pb["nen"], pb["ix"])
        assert np.array_equal(num, num_o)
        m = pg.from_problem(pb, num=num)
        o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]),
                          int(pb["nen"]), int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"],
                          pb["x"], pb["ie"], pb["e"], num=num_o)
        o.set_env(pb["gravity"], float(pb["dt"]))  # dt enters the pressure block
        assert m.neq == o.neq and m.nad == o.nad
        assert np.array_equal(m.get_id(), o.get_id())
        du = rng.standard_normal((m.nnode, 4)) * 1e-3
        bg, bo = np.zeros(m.neq), np.zeros(m.neq)
        m.pform(2, True, True, du, bg)
        o.pform(2, True, True, du, bo)
        ia, ja, ad, al = m.get_csrd()
        iao, jao, ado, alo = o.get_csrd()
        assert np.array_equal(ia, iao) and np.array_equal(ja, jao)
        scale = max(np.abs(ado).max(), np.abs(alo).max())
        assert np.abs(ad - ado).max() <= 1e-12 * scale
        assert np.abs(al - alo).max() <= 1e-12 * scale


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_histories_with_rcm_order(golden, name):
    """The golden Terzaghi columns rerun with the equations in RCM order
    (their decks say reord false): the 600-step node histories still match
    the reference's printed values within 1e-10."""
    fx = golden(name)
    m = pg.from_problem(fx, rcm=True)
    worst = 0.0
    for k in range(1, 601):
        m.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]), maxit=int(fx["maxit"]))
        u, _, _ = m.get_state()
        for a, n in enumerate(fx["hist_nodes"]):
            worst = max(worst, np.abs(u[n - 1] - fx["hist"][a][k][2:6]).max())
    assert worst < 1e-10, worst


def test_column_steps_match_oracle():
    pb = meshgen.column_problem()
    m, o = _pair(pb)
    for k in range(20):
        # stop_crit 1: on a column in hydrostatic equilibrium the pressure
        # residual of the first iteration is pure rounding, which makes the
        # reference's stop_crit 2 outcome rounding-dependent
        gi = m.step(maxnlit=2, stop_crit=1, solvtol=1e-10)
        oi = o.step(maxnlit=2, stop_crit=1, solvtol=1e-10)
        u, u0, dp = m.get_state()
        uo, u0o, dpo = o.get_state()
        for comp, sl in (("u", slice(0, 3)), ("p", slice(3, 4))):
            ref = uo[:, sl]
            err = np.abs(u[:, sl] - ref).max() / np.abs(ref).max()
            assert err < 1e-10, (k, comp, err)
        assert gi.nlit == oi.nlit


def test_stop_crit2_reference_semantics(golden):
    """With stop_crit 2 the reference resets the pressure reference norm to
    max(resp0, gresu) on the second iteration (Residuo.f); on the hydrostatic
    golden column this makes the check fail, so the step reports
    non-convergence like the reference's stop_mef."""
    fx = golden("exemplo1_mesh0_t2")
    m = pg.from_problem(fx)
    with pytest.raises(pg.PMError) as e:
        m.step(maxnlit=2, stop_crit=2, solvtol=float(fx["solver_tol"]))
    assert e.value.status == 5


def test_mixed_precision_refinement():
    """FP32 values and FP32 SpMV in the inner PCG of an FP64 iterative
    refinement reach the FP64 solution within 1e-8 relative."""
    pb = meshgen.cube_problem(n=6)
    m64 = pg.from_problem(pb)
    m32 = pg.from_problem(pb)
    m32.set_precision(pg.capi.PM_FP32_REFINE)
    m32.set_refine(1e-5)
    for k in range(3):
        m64.step(maxnlit=2, stop_crit=1, solvtol=1e-11)
        info = m32.step(maxnlit=2, stop_crit=1, solvtol=1e-11)
        assert info.refine >= 1
    u, _, _ = m64.get_state()
    v, _, _ = m32.get_state()
    for sl in (slice(0, 3), slice(3, 4)):
        assert np.abs(u[:, sl] - v[:, sl]).max() <= 1e-8 * np.abs(u[:, sl]).max()


def _abs_product(m, x):
    """(|A| |x|) from the host CSRD copy: the scale of the rounding bound."""
    import scipy.sparse as sp
    ia, ja, ad, al = m.get_csrd()
    L = sp.csr_matrix((np.abs(al), ja - 1, ia - 1), shape=(m.neq, m.neq))
    ax = np.abs(x)
    return np.abs(ad) * ax + L @ ax + L.T @ ax


@pytest.mark.parametrize("shape", [None, 1, 14, 24, 90, 91, 104, 112, 114, 124, 214, 312, 314])
def test_compensated_spmv_rounding_bound(problems, shape, monkeypatch):
    """PM_FP32C_REFINE operator: values FP32 + an int8 relative correction
    (within 2^-32 |v|), x as an FP32 pair (2^-48), compensated sums: each row
    is within 2^-30 (|A| |x|)_i of the FP64 product."""
    if shape is not None:  # a fixed kernel shape instead of the autotuner's choice
        monkeypatch.setenv("PM_SPMV_SHAPE", str(shape))
    rng = np.random.default_rng(6)
    for pb in problems:
        m = pg.from_problem(pb)
        m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
        x = rng.standard_normal(m.neq)
        y64 = m.matvec(x)
        m.set_precision(pg.capi.PM_FP32C_REFINE)
        yc = m.matvec(x)
        bound = 2.0 ** -30 * _abs_product(m, x) + 1e-300
        assert np.all(np.abs(yc - y64) <= bound), np.max(np.abs(yc - y64) / bound)
        assert not np.array_equal(yc, y64)  # the compensated path did run
        if shape is not None:
            assert m.tune_spmv() == shape


@pytest.mark.parametrize("shape", [None, 14, 91, 104, 114, 124, 214, 314])
# MINRES cases: the jittered tetra mesh and the cube; on the golden tetra
# column MINRES itself stalls (the reference's FP64 MINRES and the oracle
# need ~8e5 iterations there), which says nothing about the operator
@pytest.mark.parametrize("solver,precond,cases", [(1, 2, [2, 4]), (7, 5, [3, 4]),
                                                  (11, 2, [2, 3, 4])])
def test_compensated_solve_matches_fp64(problems, solver, precond, cases, shape, monkeypatch):
    """The compensated operator inside the FP64 refinement reaches the FP64
    solution: same stopping test, FP64 outer residual."""
    if shape is not None:  # a fixed kernel shape instead of the autotuner's choice
        monkeypatch.setenv("PM_SPMV_SHAPE", str(shape))
    for k in cases:
        pb = problems[k]
        m = pg.from_problem(pb)
        m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
        b = np.random.default_rng(7).standard_normal(m.neq)
        tol = 1e-11
        # maxit is per MINRES cycle (10 restarts, as call_minres): on these small,
        # ill-conditioned tetra meshes the recursion can stall in a cycle, which
        # the next restart (an FP64 residual) resolves
        cap = 400000 if solver in (1, 11) else 20000
        x64, _ = m.solve(b, solver=solver, precond=precond, tol=tol, maxit=cap)
        m.set_precision(pg.capi.PM_FP32C_REFINE)
        xc, info = m.solve(b, solver=solver, precond=precond, tol=tol, maxit=cap)
        assert info.refine >= 1
        assert np.abs(xc - x64).max() <= 1e4 * tol * np.abs(x64).max()
        # the FP64 residual of the result meets the solver's own test:
        # sqrt|(r, m r)| < tol sqrt|(b, m b)|, m = 1/ad (PCG) or |1/ad| (MINRES);
        # rpsqmr: ||r|| < tol ||b|| (Iters.f:6221-6223)
        m.set_precision(pg.capi.PM_FP64)  # matvec follows the precision mode
        r = b - m.matvec(xc)
        _, _, ad, _ = m.get_csrd()
        w = np.ones_like(ad) if solver == 11 else 1.0 / ad if precond == 2 else np.abs(1.0 / ad)
        rn = np.sqrt(abs(np.sum(r * r * w)))
        bn = np.sqrt(abs(np.sum(b * b * w)))
        assert rn <= 1.01 * tol * bn, (rn, tol * bn)


def test_compensated_rpsqmr_steps_on_tetra():
    """Steps of the unstructured tetra10 problem with the reference's default
    solver on the compensated operator stay within 1e-7 relative of the FP64
    rpsqmr steps (both to 1e-9)."""
    pb = meshgen.tetra_problem(n=4)
    m64 = pg.from_problem(pb)
    mc = pg.from_problem(pb)
    mc.set_precision(pg.capi.PM_FP32C_REFINE)
    kw = dict(maxnlit=2, stop_crit=1, solver=11, precond=2, solvtol=1e-9, maxit=200000)
    for _ in range(3):
        m64.step(**kw)
        info = mc.step(**kw)
        assert info.refine >= 1
    u64, _, _ = m64.get_state()
    uc, _, _ = mc.get_state()
    for sl in (slice(0, 3), slice(3, 4)):
        assert np.abs(uc[:, sl] - u64[:, sl]).max() <= 1e-7 * np.abs(u64[:, sl]).max()


def test_compensated_steps_match_fp64():
    """Three steps of the heterogeneous cube in PM_FP32C_REFINE stay within
    1e-8 relative of the FP64 steps at the same tolerance."""
    pb = meshgen.cube_problem(n=6)
    m64 = pg.from_problem(pb)
    mc = pg.from_problem(pb)
    mc.set_precision(pg.capi.PM_FP32C_REFINE)
    for k in range(3):
        a = m64.step(maxnlit=2, stop_crit=1, solvtol=1e-10)
        c = mc.step(maxnlit=2, stop_crit=1, solvtol=1e-10)
        assert c.refine >= 1 and c.nlit == a.nlit
    u, _, _ = m64.get_state()
    v, _, _ = mc.get_state()
    for sl in (slice(0, 3), slice(3, 4)):
        assert np.abs(u[:, sl] - v[:, sl]).max() <= 1e-8 * np.abs(u[:, sl]).max()


def test_errors_are_returned_not_fatal(problems):
    # maxit exceeded -> status 4, and the handle stays usable
    pb = problems[2]
    m, _ = _pair(pb)
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    b = np.ones(m.neq)
    with pytest.raises(pg.PMError) as e:
        m.solve(b, maxit=1, tol=1e-14)
    assert e.value.status == 4
    x, _ = m.solve(b, tol=1e-10)
    assert np.isfinite(x).all()
    # inverted element -> status 2 (det <= 1e-14), no fault
    bad = dict(pb)
    bad["x"] = pb["x"].copy()
    bad["x"][:, 2] *= -1.0
    mb = pg.from_problem(bad)
    with pytest.raises(pg.PMError) as e:
        mb.pform(2, True, False, np.zeros((mb.nnode, 4)), None)
    assert e.value.status == 2
