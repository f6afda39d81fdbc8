"""GPU stress recovery (pm_stress: tform_pm isw 3 + effective_stress,
Pform.f:433-640 and 2487-2505, Elmlib03.f:2206-2256 / 440-495) against the
oracle and the reference's golden node histories.

Tolerances: whole nodal fields within 1e-10 of each quantity's largest
magnitude (for the flux at least the hydraulic conductivity) against the oracle (the GPU sums the elements of a vertex in colour
order, the oracle in element order, and contracts to FMA); golden histories
within 1e-10 absolute (10 printed decimals).  The tetra10 golden run pins the
flux only: its printed stresses come from an earlier tetra10 stress pass.
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


def _oracle(pb):
    o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                      int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"], pb["e"])
    has = "load" in pb and len(pb["load"]) > 0
    o.set_loads(eload=pb.get("eload"), nload=pb.get("nload"),
                load=pb["load"] if has else None, fload=pb["fload"] if has else None)
    o.set_env(pb["gravity"], float(pb["dt"]))
    o.set_state(u=pb["u0"], u0=pb["u0"])
    return o


def _compare(gpu, ref, what, pb):
    # a hydrostatic state has zero flux up to rounding: the flux scale is the
    # hydraulic conductivity (perm rho_f |g|, material column 3)
    kh = np.abs(np.asarray(pb["e"]).reshape(-1, oracle.PROP)[:, 2]).max()
    for name, a, b in zip(("stress", "stressB", "stressE", "flux"), gpu, ref):
        scale = max(np.abs(b).max(), kh if name == "flux" else 0.0, 1e-300)
        err = np.abs(a - b).max() / scale
        assert err < 1e-10, (what, name, err)


@pytest.mark.parametrize("which", ["column", "tetra", "cube"])
def test_stress_matches_oracle(which):
    pb = {"column": lambda: meshgen.column_problem(),
          "tetra": lambda: meshgen.tetra_problem(n=3),
          "cube": lambda: meshgen.cube_problem(n=4)}[which]()
    m = pg.from_problem(pb)
    o = _oracle(pb)
    # the initial state, then after steps: the same state is loaded into both
    # so that only the recovery is compared
    _compare(m.stress(), o.stress(), (which, 0), pb)
    for k in range(1, 4):
        m.step(maxnlit=2, stop_crit=1, solvtol=1e-12)
        u, u0, dp = m.get_state()
        o.set_state(u=u, u0=u0, dp=dp)
        _compare(m.stress(), o.stress(), (which, k), pb)


@pytest.mark.parametrize("name,keys", [
    ("exemplo1_mesh0_t2", (("stress", 0, 6), ("stressB", 1, 6), ("stressE", 2, 6),
                           ("flux", 3, 3))),
    ("exemplo1_mesh0_t2_tetra", (("flux", 3, 3),)),
])
def test_stress_golden_histories_on_gpu(golden, name, keys):
    fx = golden(name)
    m = pg.from_problem(fx)
    worst = {k: 0.0 for k, _, _ in keys}
    for k in range(0, 601):
        if k > 0:
            m.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]),
                   maxit=int(fx["maxit"]))
        out = m.stress()
        for a, n in enumerate(fx["hist_nodes"]):
            for key, idx, ncol in keys:
                ref = fx["hist_" + key][a][k][2:2 + ncol]
                worst[key] = max(worst[key], np.abs(out[idx][n - 1] - ref).max())
    for key, err in worst.items():
        assert err < 1e-10, (key, err)


def test_stress_dev_on_torch_stream():
    pb = meshgen.tetra_problem(n=3)
    m = pg.from_problem(pb)
    m.step(maxnlit=2, stop_crit=1, solvtol=1e-12)
    nn = m.nnode
    f64 = dict(dtype=torch.float64, device="cuda")
    tx, txb, txe = (torch.full((nn, 6), 7.0, **f64) for _ in range(3))
    fl = torch.full((nn, 3), 7.0, **f64)
    s = torch.cuda.current_stream()
    torch.cuda.synchronize()
    m.stress_dev(tx.data_ptr(), txb.data_ptr(), txe.data_ptr(), fl.data_ptr(), s.cuda_stream)
    ref = m.stress()
    for a, b in zip((tx, txb, txe, fl), ref):
        assert np.array_equal(a.cpu().numpy(), b)


def _poro_fixture(fx, poro0=0.3):
    fx = dict(fx)
    fx["e"] = np.array(fx["e"], float).copy()
    fx["e"][:, 7] = poro0
    E, nu, _, M, alpha = fx["e"][0][:5]
    k_tr = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu)) * (1 + 2 * nu / (1 - nu))
    return fx, k_tr, M, alpha


def test_porosity_golden_derived_on_gpu(golden):
    """porosity_form on the GPU against the golden hexa20 run: the summed
    changes equal alpha avg tr(eps(u_N)) + dp_N/M, with avg tr(eps) from the
    printed total stress (normals sum to a (1 + 2b) tr(eps) - 3 alpha dp)."""
    fx, k_tr, M, alpha = _poro_fixture(golden("exemplo1_mesh0_t2"))
    m = pg.from_problem(fx)
    worst = 0.0
    for k in range(1, 601):
        m.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]), maxit=int(fx["maxit"]))
        poro = m.get_porosity()
        for a, n in enumerate(fx["hist_nodes"]):
            dpn = fx["hist"][a][k][5] - fx["hist"][a][0][5]
            sn = fx["hist_stress"][a][k][2:5].sum()
            ref = 0.3 + alpha * (sn + 3 * alpha * dpn) / k_tr + dpn / M
            worst = max(worst, abs(poro[n - 1] - ref))
    assert worst < 1e-10, worst


@pytest.mark.parametrize("name", ["exemplo1_mesh0_t2", "exemplo1_mesh0_t2_tetra"])
def test_porosity_stress_relation_on_gpu(golden, name):
    fx, k_tr, M, alpha = _poro_fixture(golden(name))
    m = pg.from_problem(fx)
    v = fx["fnno"] == 1
    for _ in range(5):
        m.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]), maxit=int(fx["maxit"]))
    poro = m.get_porosity()
    tx, _, _, _ = m.stress()
    _, _, dp = m.get_state()
    ref = 0.3 + alpha * (tx[v, :3].sum(1) + 3 * alpha * dp[v]) / k_tr + dp[v] / M
    assert np.abs(poro[v] - ref).max() < 1e-12
    assert not np.any(poro[~v])


@pytest.mark.parametrize("which", ["tetra", "cube"])
def test_porosity_matches_oracle(which):
    """Per-element materials (cube) and distorted tetra10: GPU and oracle
    step independently; their states agree to the solver tolerance, so the
    porosity changes are compared at 1e-9 of their largest magnitude."""
    pb = {"tetra": lambda: meshgen.tetra_problem(n=3),
          "cube": lambda: meshgen.cube_problem(n=4)}[which]()
    e = np.array(pb["e"], float).reshape(-1, oracle.PROP).copy()
    e[:, 7] = np.random.default_rng(11).uniform(0.1, 0.4, len(e))
    pb = dict(pb)
    pb["e"] = e
    m = pg.from_problem(pb)
    o = _oracle(pb)
    p0 = o.get_porosity()
    assert np.array_equal(m.get_porosity(), p0)
    for _ in range(3):
        m.step(maxnlit=2, stop_crit=1, solvtol=1e-13, maxit=200000)
        o.step(maxnlit=2, stop_crit=1, solvtol=1e-13, maxit=200000)
        dg, do = m.get_porosity() - p0, o.get_porosity() - p0
        assert np.abs(dg - do).max() < 1e-9 * np.abs(do).max()
    m.set_porosity(p0)
    assert np.array_equal(m.get_porosity(), p0)
