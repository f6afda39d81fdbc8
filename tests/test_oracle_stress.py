"""Pin the oracle's stress recovery and porosity update (tform_pm with the element pass isw 3,
Pform.f:433-640, Elmlib03.f:2206-2256 / 440-495, and effective_stress,
Pform.f:2487-2505) against the reference's golden node histories
(printnode stress / stressE / stressB / flux, 10 decimals) over the 600 steps
of output/poro_mec/elastico/{hexa,tetra}.

The hexa20 run pins all four quantities.  The tetra10 run pins the Darcy flux;
its printed stresses come from an earlier version of the tetra10 stress pass
(they differ from the vertex-point recovery of Elmlib03.f by up to 1e-2 MPa,
also in the shear components, which a zero-shear column cannot produce at the
vertices), so the tetra10 stresses are checked through their relations to each
other and to the flux-pinned pressure only.

Porosity (initial_porosity, Pform.f:1343-1432; porosity_form, Pform.f:969-1175
with isw 7, Elmlib03.f:2605-2631) is not printed by the golden runs.  It is
pinned through linearity: the step changes alpha tr(eps(du)) + dp/M sum to
alpha avg tr(eps(u_N)) + dp_N/M, and the vertex average of tr(eps) follows
from the printed total stress, whose normal components sum to
a (1 + 2b) tr(eps) - 3 alpha dp (stress3d, Elmlib.f:2906-2939).  The initial
porosity (material column 8) does not enter the elastic solve, so the golden
histories hold for any value of it.
"""
import numpy as np
import pytest

import oracle

KEYS = (("stress", 0, 6), ("stressE", 2, 6), ("stressB", 1, 6), ("flux", 3, 3))


def _histories(fx, nsteps, keys):
    o = oracle.from_fixture(fx)
    worst = {k: 0.0 for k, _, _ in keys}
    for k in range(0, nsteps + 1):
        if k > 0:
            o.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]),
                   maxit=int(fx["maxit"]))
        out = o.stress()
        for a, n in enumerate(fx["hist_nodes"]):
            for key, idx, ncol in keys:
                ref = fx["hist_" + key][a][k][2:2 + ncol]
                worst[key] = max(worst[key], np.abs(out[idx][n - 1] - ref).max())
    return worst, o


def test_stress_histories_hexa(golden):
    worst, _ = _histories(golden("exemplo1_mesh0_t2"), 600, KEYS)
    # 10 printed decimals: half a unit of the last digit plus the solver
    # tolerance
    for key, err in worst.items():
        assert err < 1e-10, (key, err)


def test_flux_histories_tetra(golden):
    worst, _ = _histories(golden("exemplo1_mesh0_t2_tetra"), 600, KEYS[3:])
    assert worst["flux"] < 1e-10, worst


@pytest.mark.parametrize("name,nsteps,keys,tol_stress", [
    ("solo1", 3, KEYS, 1e-10),
    # the hexa cylinder's histories sit close to the solver tolerance: its
    # displacements move by ~1e-9 with rounding alone, its stresses by ~2e-9
    ("solo_cilindro_hexa_1", 5, KEYS, 4e-9),
    # tetra10 stresses of the shipped runs come from the earlier stress pass
    # (module docstring): the flux is the pin
    ("solo_cilindro_tetra_1", 5, KEYS[3:], None),
])
def test_histories_of_the_other_decks(golden, name, nsteps, keys, tol_stress):
    """The shipped solo1 and cylinder decks' printed stress and flux histories
    over their first steps."""
    worst, _ = _histories(golden(name), nsteps, keys)
    assert worst["flux"] < 1e-10, worst
    for key in ("stress", "stressE", "stressB"):
        if key in worst:
            assert worst[key] < tol_stress, (key, worst[key])


@pytest.mark.parametrize("name", ["exemplo1_mesh0_t2", "exemplo1_mesh0_t2_tetra"])
def test_stress_relations(golden, name):
    fx = golden(name)
    o = oracle.from_fixture(fx)
    for _ in range(3):
        o.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]), maxit=int(fx["maxit"]))
    tx, txb, txe, fl = o.stress()
    u, _, _ = o.get_state()
    fnno = fx["fnno"]
    # effective = total + p on the normal components, shear unchanged
    assert np.array_equal(txe[:, 3:], tx[:, 3:])
    assert np.allclose(txe[:, :3] - tx[:, :3], u[:, 3:4], rtol=0, atol=1e-13)
    assert np.array_equal(txb[:, 3:], tx[:, 3:])
    # mid-side nodes carry no recovered values
    mid = fnno != 1
    assert not np.any(tx[mid]) and not np.any(txb[mid]) and not np.any(fl[mid])
    # Biot stress = total + alpha p on the normals (one material)
    e = np.asarray(fx["e"]).reshape(-1, oracle.PROP)
    assert len(e) == 1
    v = ~mid
    assert np.allclose(txb[v, :3] - tx[v, :3], e[0, 4] * u[v, 3:4], rtol=0, atol=1e-12)


def _poro_case(fx, poro0=0.3):
    fx = dict(fx)
    fx["e"] = np.array(fx["e"], float).copy()
    fx["e"][:, 7] = poro0
    E, nu, _, M, alpha = fx["e"][0][:5]
    a = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
    b = nu / (1 - nu)
    return fx, a * (1 + 2 * b), M, alpha


def porosity_from_stress(poro0, sn, dp, k_tr, M, alpha):
    """poro0 + alpha avg tr(eps) + dp/M with avg tr(eps) from the normal
    total stresses sn (summed) at a vertex."""
    return poro0 + alpha * (sn + 3 * alpha * dp) / k_tr + dp / M


def test_porosity_golden_derived_hexa(golden):
    fx, k_tr, M, alpha = _poro_case(golden("exemplo1_mesh0_t2"))
    o = oracle.from_fixture(fx)
    assert np.all(o.get_porosity()[fx["fnno"] == 1] == 0.3)
    worst = 0.0
    for k in range(1, 601):
        o.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]), maxit=int(fx["maxit"]))
        poro = o.get_porosity()
        for a, n in enumerate(fx["hist_nodes"]):
            dpn = fx["hist"][a][k][5] - fx["hist"][a][0][5]
            sn = fx["hist_stress"][a][k][2:5].sum()
            ref = porosity_from_stress(0.3, sn, dpn, k_tr, M, alpha)
            worst = max(worst, abs(poro[n - 1] - ref))
    assert worst < 1e-10, worst


@pytest.mark.parametrize("name", ["exemplo1_mesh0_t2", "exemplo1_mesh0_t2_tetra"])
def test_porosity_stress_relation(golden, name):
    fx, k_tr, M, alpha = _poro_case(golden(name))
    o = oracle.from_fixture(fx)
    v = fx["fnno"] == 1
    for _ in range(5):
        o.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]), maxit=int(fx["maxit"]))
    poro = o.get_porosity()
    tx, _, _, _ = o.stress()
    _, _, dp = o.get_state()
    ref = porosity_from_stress(0.3, tx[v, :3].sum(1), dp[v], k_tr, M, alpha)
    assert np.abs(poro[v] - ref).max() < 1e-12
    assert not np.any(poro[~v])


def test_initial_porosity_average():
    from poromec_gb300 import meshgen
    pb = meshgen.tetra_problem(n=3)
    e = np.array(pb["e"], float).reshape(-1, oracle.PROP).copy()
    rng = np.random.default_rng(3)
    e[:, 7] = rng.uniform(0.1, 0.4, len(e))
    o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                      int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"], e)
    nen, nenv = int(pb["nen"]), int(pb["nenv"])
    ix = np.asarray(pb["ix"]).reshape(-1, nen + 1)
    acc = np.zeros(int(pb["nnode"]))
    cnt = np.zeros(int(pb["nnode"]))
    np.add.at(acc, ix[:, :nenv].ravel() - 1, np.repeat(e[ix[:, nen] - 1, 7], nenv))
    np.add.at(cnt, ix[:, :nenv].ravel() - 1, 1)
    v = np.asarray(pb["fnno"]) == 1
    assert np.allclose(o.get_porosity()[v], acc[v] / cnt[v], rtol=1e-15, atol=0)
    assert not np.any(o.get_porosity()[~v])
    o.set_porosity(np.full(int(pb["nnode"]), 0.25))
    assert np.all(o.get_porosity() == 0.25)
