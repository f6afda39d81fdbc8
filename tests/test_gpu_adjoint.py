"""Adjoint gradient of a time-stepped misfit against central finite
differences: of the GPU forward (16 seeded directions) and of the oracle,
the CPU restatement of the reference solver (4 directions), on a small
heterogeneous cube with per-element log E, log k and log M.

Bar: |FD - adjoint| <= 1e-5 ||grad|| ||d|| per direction (the FD step is
1e-6 on the log parameters, forwards solved to 1e-13)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import poromec_gb300 as pg  # noqa: E402
from poromec_gb300 import adjoint, meshgen  # noqa: E402

NSTEPS = 4
TOL = 1e-13


@pytest.fixture(scope="module")
def model():
    pb = meshgen.cube_problem(n=3, seed=9, steps=NSTEPS)
    ds, tz, ps, tp = adjoint.sensors_and_targets(pb, n_sensors=8, seed=3)
    return adjoint.TimeSteppedMisfit(pb, NSTEPS, ds, tz, ps, tp, solvtol=TOL, ckpt_every=2)


@pytest.fixture(scope="module")
def point(model):
    rng = np.random.default_rng(21)
    theta = model.theta0() + 0.1 * rng.standard_normal(model.theta0().shape)
    th = torch.tensor(theta, dtype=torch.float64, device="cuda", requires_grad=True)
    J = adjoint.BiotMisfit.apply(th, model)
    J.backward()
    return theta, float(J.detach()), th.grad.cpu().numpy()


def test_apply_matches_assembled_matrix(model):
    """For lam with zero pressure part, K lam = [Kuu lam_u ; Kpu lam_u]: the
    apply kernel's mu (u rows) and nu (p rows) are minus those rows."""
    m = model.m
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    idr = m.get_id()
    peq = idr[:, 3][idr[:, 3] > 0] - 1
    lam = np.random.default_rng(4).standard_normal(m.neq)
    lam[peq] = 0.0
    Kl = m.matvec(lam)
    t = {k: torch.zeros(m.neq, dtype=torch.float64, device="cuda") for k in ("mu", "nu")}
    tl = torch.from_numpy(lam).cuda()
    torch.cuda.synchronize()
    m.adjoint_apply_dev(tl.data_ptr(), t["mu"].data_ptr(), t["nu"].data_ptr())
    mu, nu = t["mu"].cpu().numpy(), t["nu"].cpu().numpy()
    ueq = np.setdiff1d(np.arange(m.neq), peq)
    scale = np.abs(Kl).max()
    assert np.abs(mu[ueq] + Kl[ueq]).max() <= 1e-12 * scale
    assert np.abs(nu[peq] + Kl[peq]).max() <= 1e-12 * scale
    assert np.abs(mu[peq]).max() == 0.0  # lam_p = 0: no Kpp_perm term


def test_gradient_vs_gpu_finite_differences(model, point):
    theta, J, g = point
    rng = np.random.default_rng(17)
    h = 1e-6
    gn = np.linalg.norm(g)
    assert gn > 0 and np.isfinite(g).all()
    for k in range(16):
        d = rng.standard_normal(theta.shape)
        d /= np.linalg.norm(d)
        fd = (model.forward(theta + h * d, False) - model.forward(theta - h * d, False)) / (2 * h)
        ad = float(np.sum(g * d))
        assert abs(fd - ad) <= 1e-5 * gn, (k, fd, ad, gn)


def _oracle_J(model, theta):
    pb = model.pb
    o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                      int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"],
                      model.materials(theta))
    o.set_loads(eload=pb["eload"], load=pb["load"], fload=pb["fload"])
    o.set_env(pb["gravity"], float(pb["dt"]))
    o.set_state(u=pb["u0"], u0=pb["u0"])
    for _ in range(model.nsteps):
        o.step(maxnlit=2, tol=1e-4, stop_crit=1, solvtol=TOL, maxit=400000)
    u, _, _ = o.get_state()
    return model.misfit(u)


def test_gradient_vs_oracle_finite_differences(model, point):
    theta, J, g = point
    assert abs(_oracle_J(model, theta) - J) <= 1e-9 * abs(J)
    rng = np.random.default_rng(29)
    h = 1e-6
    gn = np.linalg.norm(g)
    for k in range(4):
        d = rng.standard_normal(theta.shape)
        d /= np.linalg.norm(d)
        fd = (_oracle_J(model, theta + h * d) - _oracle_J(model, theta - h * d)) / (2 * h)
        assert abs(fd - float(np.sum(g * d))) <= 1e-5 * gn, (k, fd)


def test_gradient_components_nonzero(point):
    """All three parameter families carry gradient (E, k and M all enter)."""
    _, _, g = point
    for c in range(3):
        assert np.abs(g[:, c]).max() > 0.0
