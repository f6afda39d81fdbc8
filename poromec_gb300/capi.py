"""ctypes binding of the GB300 library and a host-side mirror of the
reference's element/solver call surface.

The reference (lmn-labest/poroMec) is Fortran; its per-step hot path is the
set of subroutines called by the ``solv`` macro (Main.f:876-1123):
``pform_pm`` (element loop + assembly), ``matvec_csrc_sym_pm`` (CSRD SpMV),
``solv_pm`` (PCG / MINRES) and the nodal updates.  :class:`Mesh` exposes the
same operations with the same argument meaning, on top of the C ABI declared
in ``include/poromec_gb300.h``.  There is no CPU fallback: without the CUDA
library, or without a GPU, every call raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libporomec_gb300.so")

PM_PROP = 15
PM_NFLOAD = 6
PM_FP64 = 0
PM_FP32_REFINE = 1
PM_FP32C_REFINE = 2

STATUS = {0: "ok", 1: "invalid argument", 2: "element Jacobian determinant <= 1e-14",
          3: "zero diagonal coefficient", 4: "Krylov solver did not converge",
          5: "nonlinear iteration did not converge", 6: "unsupported element type",
          7: "CUDA error", 8: "device allocation failed", 9: "call out of order",
          10: "problem larger than the fixed scratch of pm_pcg_csrd_noalloc"}


class PMError(RuntimeError):
    def __init__(self, status, what, detail=""):
        self.status = status
        msg = "%s failed: %s" % (what, STATUS.get(status, status))
        if detail:
            msg += " (%s)" % detail
        super().__init__(msg)


class StepInfo(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("nlit", ctypes.c_int), ("refine", ctypes.c_int),
                ("conv", ctypes.c_double), ("xkx", ctypes.c_double),
                ("res_u", ctypes.c_double), ("res_p", ctypes.c_double)]


_lib = None


def load(path=None):
    """Load the CUDA library (building it first if only the sources exist)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build as _b
        _b.build()
    lib = ctypes.CDLL(path)
    c_i, c_d, c_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    lib.pm_last_error.restype = ctypes.c_char_p
    lib.pm_last_error.argtypes = [c_p]
    lib.pm_status_string.restype = ctypes.c_char_p
    lib.pm_destroy.restype = None
    lib.pm_destroy.argtypes = [c_p]
    lib.pm_mesh_create.argtypes = [c_i] * 7 + [c_p] * 4 + [c_i] + [c_p] * 4
    lib.pm_reord.argtypes = [c_i, c_i, c_i, c_p, c_p]
    lib.pm_batch_create.argtypes = [c_i] * 7 + [c_p] * 4 + [c_i] + [c_p] * 2 + [c_i] + [c_p] * 2
    lib.pm_get_batch_iters.argtypes = [c_p, c_p, c_p, c_i]
    lib.pm_set_loads.argtypes = [c_p] * 5 + [c_i, c_i, c_p, c_p]
    lib.pm_set_env.argtypes = [c_p, c_p, c_d, c_d, c_i]
    lib.pm_set_state.argtypes = [c_p] * 4
    lib.pm_get_state.argtypes = [c_p] * 4
    lib.pm_set_initial_stress.argtypes = [c_p, c_p]
    lib.pm_set_precision.argtypes = [c_p, c_i]
    lib.pm_set_refine.argtypes = [c_p, c_d]
    lib.pm_tune_spmv.argtypes = [c_p, ctypes.POINTER(ctypes.c_int)]
    lib.pm_get_sizes.argtypes = [c_p] * 5
    lib.pm_get_id.argtypes = [c_p, c_p]
    lib.pm_get_csrd.argtypes = [c_p] * 5
    lib.pm_assemble.argtypes = [c_p, c_i, c_i, c_i, c_p, c_p]
    lib.pm_spmv.argtypes = [c_p, c_p, c_p]
    lib.pm_solve.argtypes = [c_p, c_i, c_i, c_p, c_p, c_d, c_i, c_p]
    lib.pm_step.argtypes = [c_p, c_i, c_d, c_i, c_i, c_i, c_d, c_i, c_i, c_p]
    lib.pm_spmv_dev.argtypes = [c_p, c_p, c_p, c_p]
    lib.pm_solve_dev.argtypes = [c_p, c_i, c_i, c_p, c_p, c_d, c_i, c_p, c_p]
    lib.pm_matvec_csrd_dev.argtypes = [c_i, c_p, c_p, c_p, c_p, c_p, c_p, c_p]
    lib.pm_get_timers.argtypes = [c_p, c_p, c_i]
    lib.pm_set_materials.argtypes = [c_p, c_p, c_i]
    lib.pm_stress.argtypes = [c_p] * 5
    lib.pm_get_porosity.argtypes = [c_p, c_p]
    lib.pm_set_nkrylov.argtypes = [c_p, c_i]
    lib.pm_deck_read.argtypes = [ctypes.c_char_p, c_p]
    lib.pm_deck_error.restype = ctypes.c_char_p
    lib.pm_deck_free.argtypes = [c_p]
    lib.pm_deck_free.restype = None
    lib.pm_deck_value.argtypes = [c_p, ctypes.c_char_p, c_p]
    lib.pm_deck_int_array.argtypes = [c_p, ctypes.c_char_p, c_p, c_p]
    lib.pm_deck_real_array.argtypes = [c_p, ctypes.c_char_p, c_p, c_p]
    lib.pm_deck_create.argtypes = [c_p, c_p]
    lib.pm_deck_run.argtypes = [c_p, c_p, ctypes.c_char_p, c_i, c_p]
    lib.pm_deck_write_geo.argtypes = [c_p, ctypes.c_char_p, c_i]
    lib.pm_deck_write_res.argtypes = [c_p, c_p, ctypes.c_char_p, c_i, c_d, c_i, c_i]
    lib.pm_set_porosity.argtypes = [c_p, c_p]
    lib.pm_stress_dev.argtypes = [c_p] * 6
    lib.pm_adjoint_apply_dev.argtypes = [c_p] * 5
    lib.pm_adjoint_grad_dev.argtypes = [c_p] * 6
    _lib = lib
    return lib


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Mesh:
    """Device-resident mesh, matrix and state: the 'mesh' macro of the
    reference (Main.f:481-870) and the operations of its 'solv' macro.

    Arrays follow the Fortran layouts transposed into C order:
    ix (numel, nen+1) with the material id last, idflag (nnode, 4) restraint
    flags (1 = prescribed), fnno (nnode), x (nnode, 3), ie (numat,),
    e (numat, PM_PROP), u (nnode, 4).  Node, material and equation numbers
    are 1-based as in the reference.
    """

    def __init__(self, nnode, nnodev, numel, nen, nenv, ix, idflag, fnno, x, ie, e, num=None,
                 inst_node_ptr=None):
        self.lib = load()
        self.nnode, self.numel, self.nen, self.nenv = int(nnode), int(numel), int(nen), int(nenv)
        ix, idflag, fnno, ie, num = map(_i32, (ix, idflag, fnno, ie, num))
        x, e = _f64(x), _f64(e)
        if e.ndim == 1:
            e = e.reshape(1, -1)
        if e.shape[1] < PM_PROP:
            e = np.pad(e, ((0, 0), (0, PM_PROP - e.shape[1])))
        h = ctypes.c_void_p()
        self.ninst = 0
        if inst_node_ptr is None:
            st = self.lib.pm_mesh_create(self.nnode, int(nnodev), self.numel, self.nen,
                                         self.nenv, 3, 4, _p(ix), _p(idflag), _p(fnno), _p(x),
                                         len(ie), _p(ie), _p(e), _p(num), ctypes.byref(h))
            what = "pm_mesh_create"
        else:
            ptr = _i32(inst_node_ptr)
            self.ninst = len(ptr) - 1
            st = self.lib.pm_batch_create(self.nnode, int(nnodev), self.numel, self.nen,
                                          self.nenv, 3, 4, _p(ix), _p(idflag), _p(fnno), _p(x),
                                          len(ie), _p(ie), _p(e), self.ninst, _p(ptr),
                                          ctypes.byref(h))
            what = "pm_batch_create"
        if st != 0:
            raise PMError(st, what)
        self.h = h
        neq, nad, nc, nnz = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_int64()
        self.lib.pm_get_sizes(h, ctypes.byref(neq), ctypes.byref(nad), ctypes.byref(nc),
                              ctypes.byref(nnz))
        self.neq, self.nad, self.numcolors, self.nnz_panel = neq.value, nad.value, nc.value, nnz.value

    @classmethod
    def adopt(cls, h, nnode, numel, nen, nenv):
        """A Mesh around a handle created elsewhere in the library
        (pm_deck_create); it is destroyed with the Mesh."""
        m = cls.__new__(cls)
        m.lib = load()
        m.nnode, m.numel, m.nen, m.nenv = int(nnode), int(numel), int(nen), int(nenv)
        m.ninst = 0
        m.h = h
        neq, nad, nc, nnz = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_int64()
        m.lib.pm_get_sizes(h, ctypes.byref(neq), ctypes.byref(nad), ctypes.byref(nc),
                           ctypes.byref(nnz))
        m.neq, m.nad, m.numcolors, m.nnz_panel = neq.value, nad.value, nc.value, nnz.value
        return m

    # ------------------------------------------------------------------
    def _check(self, st, what):
        if st != 0:
            raise PMError(st, what, self.lib.pm_last_error(self.h).decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            self.lib.pm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- set-up ---------------------------------------------------------
    def set_loads(self, eload=None, eloadp=None, nload=None, f=None, load=None, fload=None):
        eload, eloadp, nload, load = map(_i32, (eload, eloadp, nload, load))
        f, fload = _f64(f), _f64(fload)
        nl = 0 if load is None else len(load)
        maxt = 1 if fload is None else fload.shape[-1]
        self._check(self.lib.pm_set_loads(self.h, _p(eload), _p(eloadp), _p(nload), _p(f), nl,
                                          maxt, _p(load), _p(fload)), "pm_set_loads")

    def set_env(self, gravity, dt, t=0.0, istep=0):
        g = _f64(gravity)
        self._check(self.lib.pm_set_env(self.h, _p(g), float(dt), float(t), int(istep)),
                    "pm_set_env")

    def set_state(self, u=None, u0=None, dp=None):
        u, u0, dp = map(_f64, (u, u0, dp))
        self._check(self.lib.pm_set_state(self.h, _p(u), _p(u0), _p(dp)), "pm_set_state")

    def get_state(self):
        u, u0, dp = np.zeros((self.nnode, 4)), np.zeros((self.nnode, 4)), np.zeros(self.nnode)
        self._check(self.lib.pm_get_state(self.h, _p(u), _p(u0), _p(dp)), "pm_get_state")
        return u, u0, dp

    def set_initial_stress(self, tx0):
        t = _f64(tx0)
        self._check(self.lib.pm_set_initial_stress(self.h, _p(t)), "pm_set_initial_stress")

    def set_precision(self, mode):
        self._check(self.lib.pm_set_precision(self.h, int(mode)), "pm_set_precision")

    def set_refine(self, inner_tol=1e-5):
        self._check(self.lib.pm_set_refine(self.h, float(inner_tol)), "pm_set_refine")

    def set_nkrylov(self, k):
        """GMRES(l) basis size (default 150)."""
        self._check(self.lib.pm_set_nkrylov(self.h, int(k)), "pm_set_nkrylov")

    def get_porosity(self):
        poro = np.zeros(self.nnode)
        self._check(self.lib.pm_get_porosity(self.h, _p(poro)), "pm_get_porosity")
        return poro

    def set_porosity(self, poro):
        a = np.ascontiguousarray(poro, dtype=np.float64)
        self._check(self.lib.pm_set_porosity(self.h, _p(a)), "pm_set_porosity")

    def stress(self):
        """tform_pm isw 3 + effective_stress of the current state: total, Biot
        and effective stress (nnode, 6), Darcy flux (nnode, 3)."""
        tx, txb, txe = np.zeros((self.nnode, 6)), np.zeros((self.nnode, 6)), np.zeros((self.nnode, 6))
        fl = np.zeros((self.nnode, 3))
        self._check(self.lib.pm_stress(self.h, _p(tx), _p(txb), _p(txe), _p(fl)), "pm_stress")
        return tx, txb, txe, fl

    def stress_dev(self, tx_ptr, txb_ptr, txe_ptr, flux_ptr, stream=None):
        """stress() into device arrays (6, 6, 6, 3 doubles per node)."""
        self._check(self.lib.pm_stress_dev(self.h, ctypes.c_void_p(tx_ptr),
                                           ctypes.c_void_p(txb_ptr), ctypes.c_void_p(txe_ptr),
                                           ctypes.c_void_p(flux_ptr),
                                           ctypes.c_void_p(stream) if stream else None),
                    "pm_stress_dev")

    def set_materials(self, e):
        """Replace the material table (numat rows of PM_PROP values)."""
        ea = _f64(e)
        if ea.ndim == 1:
            ea = ea.reshape(1, -1)
        if ea.shape[1] < PM_PROP:
            ea = np.pad(ea, ((0, 0), (0, PM_PROP - ea.shape[1])))
        ea = np.ascontiguousarray(ea)
        self._check(self.lib.pm_set_materials(self.h, _p(ea), ea.shape[0]), "pm_set_materials")

    def adjoint_apply_dev(self, lam_ptr, mu_ptr, nu_ptr, stream=None):
        """mu -= [Kuu lam_u ; Kpp_perm lam_p], nu -= Kpu lam_u (device pointers)."""
        self._check(self.lib.pm_adjoint_apply_dev(self.h, ctypes.c_void_p(lam_ptr),
                                                  ctypes.c_void_p(mu_ptr),
                                                  ctypes.c_void_p(nu_ptr),
                                                  ctypes.c_void_p(stream) if stream else None),
                    "pm_adjoint_apply_dev")

    def adjoint_grad_dev(self, lam_ptr, un_ptr, dun_ptr, grad_ptr, stream=None):
        """grad += per-element log-parameter contractions (device pointers)."""
        self._check(self.lib.pm_adjoint_grad_dev(self.h, ctypes.c_void_p(lam_ptr),
                                                 ctypes.c_void_p(un_ptr),
                                                 ctypes.c_void_p(dun_ptr),
                                                 ctypes.c_void_p(grad_ptr),
                                                 ctypes.c_void_p(stream) if stream else None),
                    "pm_adjoint_grad_dev")

    def batch_iters(self):
        """Per instance of a batch: Krylov iterations of the last solve or
        step and the nonlinear iteration at which the last step stopped."""
        it = np.zeros(self.ninst, np.int32)
        nl = np.zeros(self.ninst, np.int32)
        self._check(self.lib.pm_get_batch_iters(self.h, _p(it), _p(nl), self.ninst),
                    "pm_get_batch_iters")
        return it, nl

    def tune_spmv(self):
        """Autotune the compensated SpMV on the assembled matrix; returns the
        chosen shape code: 10 * (0, 1, 2 for 8, 16, 32 lanes per node) +
        columns per lane and trip."""
        u = ctypes.c_int(0)
        self._check(self.lib.pm_tune_spmv(self.h, ctypes.byref(u)), "pm_tune_spmv")
        return u.value

    def get_id(self):
        idr = np.zeros((self.nnode, 4), np.int32)
        self._check(self.lib.pm_get_id(self.h, _p(idr)), "pm_get_id")
        return idr

    def get_csrd(self, values=True):
        ia = np.zeros(self.neq + 1, np.int64)
        ja = np.zeros(self.nad, np.int32)
        ad = np.zeros(self.neq) if values else None
        al = np.zeros(self.nad) if values else None
        self._check(self.lib.pm_get_csrd(self.h, _p(ia), _p(ja), _p(ad), _p(al)), "pm_get_csrd")
        return ia, ja, ad, al

    # ---- the reference's hot-path routines ---------------------------------
    def pform(self, isw, lhs, rhs, u, b):
        """pform_pm (Pform.f:1-429): b -= p in place; K assembled if lhs."""
        ua = _f64(u)
        if rhs:
            assert b.dtype == np.float64 and b.flags.c_contiguous and b.shape == (self.neq,)
        self._check(self.lib.pm_assemble(self.h, int(isw), int(lhs), int(rhs), _p(ua),
                                         _p(b) if rhs else None), "pm_assemble")
        return b

    def matvec(self, x):
        """matvec_csrc_sym_pm (Matvec.f:1504-1598): y = A x."""
        xa = _f64(x)
        y = np.zeros(self.neq)
        self._check(self.lib.pm_spmv(self.h, _p(xa), _p(y)), "pm_spmv")
        return y

    def solve(self, b, solver=1, precond=2, tol=1e-11, maxit=50000):
        """solv_pm (Solv.f:27-780): solver 1 PCG, 2 GMRES(l) (maxit = cycles),
        7 MINRES, 11 rpsqmr (GMRES(l) fallback at maxit)."""
        ba = _f64(b)
        x = np.zeros(self.neq)
        info = StepInfo()
        self._check(self.lib.pm_solve(self.h, int(solver), int(precond), _p(ba), _p(x),
                                      float(tol), int(maxit), ctypes.byref(info)), "pm_solve")
        return x, info

    def step(self, maxnlit=2, tol=1e-4, stop_crit=2, solver=1, precond=2, solvtol=1e-11,
             maxit=50000, reassemble=True):
        """One 'solv' macro step (Main.f:876-1123) on the device state."""
        info = StepInfo()
        self._check(self.lib.pm_step(self.h, int(maxnlit), float(tol), int(stop_crit),
                                     int(solver), int(precond), float(solvtol), int(maxit),
                                     int(bool(reassemble)), ctypes.byref(info)), "pm_step")
        return info

    def timers(self):
        t = np.zeros(8)
        self._check(self.lib.pm_get_timers(self.h, _p(t), 8), "pm_get_timers")
        return t

    # ---- device-pointer entry points (torch tensors) -----------------------
    def spmv_dev(self, x_ptr, y_ptr, stream=None):
        self._check(self.lib.pm_spmv_dev(self.h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr),
                                         ctypes.c_void_p(stream) if stream else None),
                    "pm_spmv_dev")

    def solve_dev(self, b_ptr, x_ptr, solver=1, precond=2, tol=1e-11, maxit=50000, stream=None):
        info = StepInfo()
        self._check(self.lib.pm_solve_dev(self.h, int(solver), int(precond),
                                          ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr),
                                          float(tol), int(maxit), ctypes.byref(info),
                                          ctypes.c_void_p(stream) if stream else None),
                    "pm_solve_dev")
        return info


def matvec_csrd_dev(neq, ia_ptr, ja_ptr, ad_ptr, al_ptr, x_ptr, y_ptr, stream=None):
    """The reference CSRD layout on the device (Matvec.f:1504-1598)."""
    lib = load()
    st = lib.pm_matvec_csrd_dev(int(neq), *[ctypes.c_void_p(p) for p in
                                            (ia_ptr, ja_ptr, ad_ptr, al_ptr, x_ptr, y_ptr)],
                                ctypes.c_void_p(stream) if stream else None)
    if st != 0:
        raise PMError(st, "pm_matvec_csrd_dev")


def reord(nnode, numel, nen, ix):
    """reord (Reord.f:1-44): the reference's reverse Cuthill-McKee node
    order; num[i] is the 1-based node visited i-th (pm_mesh_create's num).
    ix is (numel, nen+1)."""
    num = np.zeros(int(nnode), np.int32)
    ixa = _i32(ix)
    st = load().pm_reord(int(nnode), int(numel), int(nen), _p(ixa), _p(num))
    if st != 0:
        raise PMError(st, "pm_reord")
    return num


def from_problem(pb, num=None, rcm=False):
    """Mesh for a problem dict (the keys of tests/golden fixtures and of
    poromec_gb300.meshgen problems) with loads, gravity, dt and the initial
    state applied.  rcm=True numbers the equations in the reference's
    reverse Cuthill-McKee node order (reord true) unless num is given."""
    if num is None and rcm:
        num = reord(pb["nnode"], pb["numel"], pb["nen"], pb["ix"])
    m = Mesh(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
             int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"], pb["e"],
             num=num, inst_node_ptr=pb.get("inst_node_ptr"))
    has_loads = "load" in pb and len(pb["load"]) > 0
    m.set_loads(eload=pb.get("eload"), eloadp=pb.get("eloadp"), nload=pb.get("nload"),
                f=pb.get("f"), load=pb["load"] if has_loads else None,
                fload=pb["fload"] if has_loads else None)
    m.set_env(pb["gravity"], float(pb["dt"]))
    m.set_state(u=pb["u0"], u0=pb["u0"], dp=pb.get("dp"))
    return m
