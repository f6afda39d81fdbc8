"""Pin the CPU oracle against the reference's own golden runs.

The fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from
output/poro_mec/elastico/{hexa,tetra}) hold the reference's node histories
(printnode, 10 decimals), its neq/nad counts and its PCG iteration log.
"""
import numpy as np
import pytest

import oracle

CASES = ["exemplo1_mesh0_t2", "exemplo1_mesh0_t2_tetra", "solo1", "solo1_tetra",
         "solo_cilindro_hexa_1", "solo_cilindro_tetra_1"]


@pytest.mark.parametrize("name", CASES)
def test_pattern_counts(golden, name):
    fx = golden(name)
    o = oracle.from_fixture(fx)
    assert int(fx["nnode"]) == int(fx["nnode_ref"])
    assert o.neq == int(fx["neq_ref"])
    assert o.nad == int(fx["nad_ref"])
    ia, ja, _, _ = o.get_csrd()
    assert ia[0] == 1 and ia[-1] == o.nad + 1
    for r in range(0, o.neq, max(1, o.neq // 50)):
        cols = ja[ia[r] - 1:ia[r + 1] - 1]
        assert np.all(np.diff(cols) > 0) and (len(cols) == 0 or cols[-1] < r + 1)


def _run(fx, nsteps):
    o = oracle.from_fixture(fx)
    hist = fx["hist"]
    worst = 0.0
    iters = []
    for k in range(1, nsteps + 1):
        # one linear solve per step, as the golden runs do (stop_crit 1 accepts
        # the second nonlinear iteration of a linear problem)
        info = o.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]),
                      maxit=int(fx["maxit"]))
        iters.append(info.iters)
        u, _, _ = o.get_state()
        for a, n in enumerate(fx["hist_nodes"]):
            worst = max(worst, np.abs(u[n - 1] - hist[a][k][2:6]).max())
    return worst, iters


# (deck, steps, bar, first PCG count equal to the reference's)
@pytest.mark.parametrize("name,nsteps,tol,first_exact", [
    ("exemplo1_mesh0_t2", 600, 1e-10, True),
    ("exemplo1_mesh0_t2_tetra", 600, 1e-10, True),
    ("solo1", 3, 1e-10, False),
    # the shipped cylinder decks: element loads read from files, 41 colours for
    # the tetra.  Their histories sit close to the solver tolerance: rounding
    # alone moves them by up to ~1e-9 (the hexa deck with this oracle on 1
    # thread: 9.4e-10; on 8 threads, whose SpMV sums in another order: 5.4e-11)
    ("solo_cilindro_hexa_1", 5, 2e-9, False),
    ("solo_cilindro_tetra_1", 5, 2e-9, False),
])
def test_node_histories(golden, name, nsteps, tol, first_exact):
    fx = golden(name)
    worst, iters = _run(fx, nsteps)
    # printed with 10 decimals: half a unit of the last digit plus the
    # solver tolerance
    assert worst < tol, worst
    ref_its = fx["pcg_iters"][:nsteps]
    if len(ref_its) == 0:  # the run's log holds no iteration counts
        return
    assert iters[0] == ref_its[0] or not first_exact
    # PCG on this indefinite system is sensitive to rounding: the counts agree
    # on average, not step by step
    assert abs(np.mean(iters) - np.mean(ref_its)) <= 0.1 * np.mean(ref_its)


@pytest.mark.parametrize("name", ["exemplo1_mesh0_t2", "exemplo1_mesh0_t2_tetra"])
def test_energy_norms_of_the_solver_log(golden, name):
    """x.Kx of every step's solve against the reference's solver log (the
    'energy norm' of its PCG lines, 10 significant digits)."""
    fx = golden(name)
    o = oracle.from_fixture(fx)
    xkx = np.array([o.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]),
                           maxit=int(fx["maxit"])).xkx for _ in range(600)])
    ref = fx["pcg_xkx"]
    assert np.all(np.abs(xkx - ref) <= 1e-9 * np.abs(ref) + 1e-13)


def test_first_step_known_answers(golden):
    fx = golden("exemplo1_mesh0_t2")
    o = oracle.from_fixture(fx)
    o.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]))
    u, _, _ = o.get_state()
    assert abs(u[0, 2] - (-0.0159674582)) < 1e-10
    fx = golden("exemplo1_mesh0_t2_tetra")
    o = oracle.from_fixture(fx)
    o.step(maxnlit=2, stop_crit=1, solvtol=float(fx["solver_tol"]))
    u, _, _ = o.get_state()
    assert abs(u[0, 2] - (-0.0159146280)) < 1e-10
    assert abs(u[43, 3] - 3.9123311721) < 1e-10
