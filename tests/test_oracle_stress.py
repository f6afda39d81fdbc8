"""Pin the oracle's stress recovery (tform_pm with the element pass isw 3,
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
