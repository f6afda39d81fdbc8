"""Error paths of the C ABI on the GPU.  Where the reference calls stop_mef
(Paralelo.f:1158-1165) the library returns a status and the handle stays
usable; the oracle returns the same status for the same input.  Every case
here is a host-side check or a flag a kernel sets: none reads out of bounds
or waits on the device."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import poromec_gb300 as pg  # noqa: E402
from poromec_gb300 import meshgen  # noqa: E402

PM_E_ARG, PM_E_ZERO_DIAG, PM_E_ELTYPE, PM_E_STATE = 1, 3, 6, 9


def _oracle(pb):
    return oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                         int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"],
                         pb["e"])


def test_zero_diagonal_is_a_status_and_the_handle_recovers():
    """E = 0 leaves every displacement row without a diagonal: pcg's
    pre_diag check (Iters.f:401-406) stops the reference; here pm_solve
    returns PM_E_ZERO_DIAG, as the oracle does, and the same handle solves
    once the materials are restored."""
    pb = meshgen.column_problem()
    e0 = np.array(pb["e"], dtype=np.float64).reshape(-1, 15)
    bad = dict(pb)
    bad["e"] = e0.copy()
    bad["e"][:, 0] = 0.0
    m = pg.from_problem(bad)
    z = np.zeros((m.nnode, 4))
    m.pform(2, True, False, z, None)
    b = np.ones(m.neq)
    with pytest.raises(pg.PMError) as e:
        m.solve(b, tol=1e-10)
    assert e.value.status == PM_E_ZERO_DIAG
    o = _oracle(bad)
    o.pform(2, True, False, z, np.zeros(o.neq))
    with pytest.raises(oracle.OracleError, match="status 3"):
        o.solve(b, tol=1e-10)
    m.set_materials(e0)
    m.pform(2, True, False, z, None)
    x, info = m.solve(b, tol=1e-10)
    assert np.isfinite(x).all() and info.iters > 0
    assert np.linalg.norm(b - m.matvec(x)) <= 1e-6 * np.linalg.norm(b)


def test_calls_out_of_order_return_a_status():
    """A solve or a product before the first assembly is PM_E_STATE; the
    handle then assembles and solves normally."""
    pb = meshgen.column_problem()
    m = pg.from_problem(pb)
    b = np.ones(m.neq)
    with pytest.raises(pg.PMError) as e:
        m.solve(b)
    assert e.value.status == PM_E_STATE
    with pytest.raises(pg.PMError) as e:
        m.matvec(b)
    assert e.value.status == PM_E_STATE
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    x, _ = m.solve(b, tol=1e-10)
    assert np.isfinite(x).all()


def test_element_type_and_empty_system_are_rejected_at_creation():
    """An element type other than 15 / 17 is PM_E_ELTYPE at creation (the
    oracle returns the same status from its element loop); a mesh whose dofs
    are all prescribed has no equations and is PM_E_ARG, before any panel is
    built."""
    pb = meshgen.column_problem()
    bad = dict(pb)
    bad["ie"] = np.full_like(np.asarray(pb["ie"]), 99)
    with pytest.raises(pg.PMError) as e:
        pg.from_problem(bad)
    assert e.value.status == PM_E_ELTYPE
    o = _oracle(bad)  # the oracle checks the type per element, in pform
    with pytest.raises(oracle.OracleError, match="status 6"):
        o.pform(2, True, False, np.zeros((o.nnode, 4)), np.zeros(o.neq))
    fixed = dict(pb)
    fixed["id"] = np.ones_like(np.asarray(pb["id"]))
    with pytest.raises(pg.PMError) as e:
        pg.from_problem(fixed)
    assert e.value.status == PM_E_ARG
    # the library still creates and steps a valid mesh afterwards
    m = pg.from_problem(pb)
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    x, _ = m.solve(np.ones(m.neq), tol=1e-10)
    assert np.isfinite(x).all()
