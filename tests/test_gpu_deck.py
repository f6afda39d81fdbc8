"""Decks run end to end on the GPU (pm_deck_run): the golden Terzaghi
columns written back as decks in the shipped decks' syntax, their macro
program (600 steps of solv / pnup / pnsf) run by the library, and the
history files compared with the reference's printed histories.

Both sides print 10 decimals in the golden layout, so the bar is one unit
in the last printed digit plus the solver tolerance.  The tetra10 run pins
u, p and the flux; its printed stresses come from an earlier tetra10 stress
pass (tests/test_oracle_stress.py).
"""
import os
import re

import numpy as np
import pytest

from deck_writer import write_linear_deck

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from poromec_gb300.deck import Deck, read_history  # noqa: E402

GOLDEN_HEADERS = {"up": "DeslocAndPress", "stress": "stressTotal", "stressE": "stressE",
                  "stressB": "stressBiot", "flux": "stressFlux"}


@pytest.mark.parametrize("name,keys", [
    ("exemplo1_mesh0_t2", ("up", "stress", "stressE", "stressB", "flux")),
    ("exemplo1_mesh0_t2_tetra", ("up", "flux")),
])
def test_deck_run_matches_golden_histories(golden, tmp_path, name, keys):
    fx = golden(name)
    path = write_linear_deck(fx, str(tmp_path), name)
    prefix = os.path.join(str(tmp_path), "out", name)
    os.makedirs(os.path.dirname(prefix))
    _, nsteps = Deck(path).run(prefix, fmt="golden")
    assert nsteps == int(fx["nsteps"]) == 600
    ref = {"up": fx["hist"], "stress": fx["hist_stress"], "stressE": fx["hist_stressE"],
           "stressB": fx["hist_stressB"], "flux": fx["hist_flux"]}
    for a, n in enumerate(fx["hist_nodes"]):
        for k in keys:
            fn = "%s_%s_node_%d.txt" % (prefix, k, n)
            with open(fn) as fh:
                head = fh.readline()
            assert head == "# Variacao %s no tempo no ponto%9d\n" % (GOLDEN_HEADERS[k], n)
            h = read_history(fn)
            r = ref[k][a]
            assert h.shape == r.shape, (k, h.shape, r.shape)
            assert np.array_equal(h[:, 0], r[:, 0])                       # istep
            assert np.abs(h[:, 1] - r[:, 1]).max() <= 1e-6                # t, 6 decimals
            assert np.abs(h[:, 2:] - r[:, 2:]).max() <= 1.5e-10, (k, n)
        assert os.path.exists("%s_poro_node_%d.txt" % (prefix, n))
    # the solver log against the reference's: one PCG line per step; counts
    # follow rounding on this indefinite system (the mean within 10 %, as the
    # oracle's); energy norms x.Kx within 1e-8 relative (printed to 10 digits)
    with open(prefix + "_log_1.txt") as fh:
        lines = fh.read().splitlines()
    assert lines[0] == "Solver control flop." and len(lines) == 601
    its = np.array([int(ln.split()[2]) for ln in lines[1:]])
    xkx = np.array([float(ln.split()[5].replace("D", "E")) for ln in lines[1:]])
    ref = fx["pcg_iters"][:600]
    assert its[0] == ref[0] or abs(its[0] - ref[0]) <= 2
    assert abs(its.mean() - ref.mean()) <= 0.1 * ref.mean()
    # sizes of the run's log against the reference's _t_1.txt (make_golden.py)
    with open(prefix + "_t_1.txt") as fh:
        kv = dict(ln.split()[:2] for ln in fh if len(ln.split()) == 2)
    assert int(kv["neq"]) == int(fx["neq_ref"]) and int(kv["nad"]) == int(fx["nad_ref"])
    assert int(kv["nnode"]) == int(fx["nnode_ref"])
    assert float(kv["SOLVR"]) > 0 and float(kv["TOTAL"]) >= float(kv["SOLVR"])
    assert lines[1].startswith("PCG:  it ")
    assert np.all(np.abs(xkx - fx["pcg_xkx"]) <= 1e-8 * np.abs(fx["pcg_xkx"]) + 1e-13)


@pytest.mark.parametrize("name,nsteps,tol", [
    ("solo1", 3, 1.5e-10),
    ("solo_cilindro_hexa_1", 5, 1e-9),
    ("solo_cilindro_tetra_1", 5, 1e-9),
])
def test_larger_decks_first_steps(golden, tmp_path, name, nsteps, tol):
    """The other shipped decks (element loads read from files, cylinders) for
    their first steps through the deck runner: u and p histories against the
    reference's, at the oracle's bars for the same decks."""
    fx = golden(name)
    path = write_linear_deck(fx, str(tmp_path), name, nsteps=nsteps)
    prefix = os.path.join(str(tmp_path), name)
    _, n = Deck(path).run(prefix, fmt="golden")
    assert n == nsteps
    for a, node in enumerate(fx["hist_nodes"]):
        h = read_history("%s_up_node_%d.txt" % (prefix, node))
        r = fx["hist"][a][:nsteps + 1]
        assert h.shape == r.shape
        assert np.abs(h[:, 2:] - r[:, 2:]).max() <= tol, (name, node)


def test_printnode_layout(golden, tmp_path):
    """pnup / pnsf in printnode's (i9,10e18.10) rows (Pdata.f:760)."""
    fx = golden("exemplo1_mesh0_t2")
    path = write_linear_deck(fx, str(tmp_path), "t", nsteps=3)
    prefix = os.path.join(str(tmp_path), "t")
    Deck(path).run(prefix, fmt="printnode")
    for k, ncol in (("up", 4), ("stress", 6), ("flux", 3), ("poro", 1)):
        with open("%s_%s_node_1.txt" % (prefix, k)) as fh:
            lines = fh.read().splitlines()
        assert lines[0].startswith("# Variacao ")
        assert len(lines) == 5
        for ln in lines[1:]:
            assert len(ln) == 9 + 18 * (ncol + 1)
            fields = [ln[9 + 18 * j:9 + 18 * (j + 1)] for j in range(ncol + 1)]
            for f in fields:
                assert re.fullmatch(r" *-?0\.\d{10}E[+-]\d{2}", f), f
    h = read_history("%s_up_node_1.txt" % prefix)
    r = fx["hist"][0][:4]
    assert np.abs(h[:, 2:] - r[:, 2:]).max() <= 1.5e-10


def test_result_vtk_holds_the_state(golden, tmp_path):
    """pres (write_mesh_res_pm, Write_vtk.f:912-1399): the state and the
    recovered fields in <prefix>_istep_<n>.vtk, printed with 5 digits."""
    from poromec_gb300.deck import read_vtk
    fx = golden("exemplo1_mesh0_t2")
    path = write_linear_deck(fx, str(tmp_path), "r", nsteps=2)
    with open(path) as fh:
        text = fh.read().replace("pnsf\nnext", "pnsf\npres\nnext")
    with open(path, "w") as fh:
        fh.write(text)
    d = Deck(path)
    prefix = os.path.join(str(tmp_path), "r")
    m, n = d.run(prefix)
    assert n == 2
    g = read_vtk(prefix + "_istep_2.vtk")
    assert g["field"]["CYCLE"] == [2] and g["field"]["TIME_S"] == [2 * float(fx["dt"])]
    assert set(g["cell_types"]) == {25} and g["points"].shape[0] == int(fx["nnode"])
    u, _, dp = m.get_state()
    tx, txb, txe, fl = m.stress()

    def close(a, b):
        return np.all(np.abs(a - b) <= 5e-5 * np.abs(b) + 1e-12 * max(1.0, np.abs(b).max()))

    assert close(g["point_data"]["desloc"], u[:, :3])
    fnno = fx["fnno"] == 1
    assert close(g["point_data"]["pressao"][fnno, 0], u[fnno, 3])
    assert close(g["point_data"]["deltaPressao"][fnno, 0], dp[fnno])
    full = g["point_data"]["totalStress"].reshape(-1, 3, 3)
    assert close(full[fnno, 0, 0], tx[fnno, 0]) and close(full[fnno, 2, 2], tx[fnno, 2])
    assert close(full[fnno, 0, 1], tx[fnno, 3]) and close(full[fnno, 1, 2], tx[fnno, 4])
    assert close(g["point_data"]["darcyFlux"][fnno], fl[fnno])
    assert close(g["point_data"]["porosity"][fnno, 0], m.get_porosity()[fnno])
