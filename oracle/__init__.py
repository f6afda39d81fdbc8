"""CPU oracle for the poroMec Biot hot path -- TEST INFRASTRUCTURE ONLY.

``oracle/poromec_oracle.cpp`` restates the reference Fortran routines
(lmn-labest/poroMec mef/src: Elmlib03.f elmt17_pm/elmt15_pm, Elmlib.f shape
functions, Pform.f pform_pm, Assbly.f csr, Csr.f/Graph.f/Numeq.f CSRD pattern,
Matvec.f matvec_csrc_sym_pm, Iters.f pcg/pminres, Main.f solv macro).  This
module builds it with g++ (a parity build, and a timing build of the same
source for the CPU baseline) and wraps it with ctypes.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may import it; the
GPU library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libporomec_oracle.so")
# the same source built for timing (bench.py's CPU baseline and reference
# arm): -O3 with FMA contraction, the flags of a release build of the
# reference on a host whose compiler contracts (GCC does by default on
# aarch64); results differ from the parity build by rounding only
LIB_TIMING = os.path.join(BUILD, "libporomec_oracle_o3.so")
SRC = os.path.join(HERE, "poromec_oracle.cpp")
PROP = 15
NFLOAD = 6


def build(force=False, timing=False):
    """Compile the oracle: -O2 without FMA contraction, so the arithmetic
    follows the reference's x86-64 gfortran -O2 build operation for operation.
    timing=True builds the timing variant instead (-O3, FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    out = LIB_TIMING if timing else LIB
    if (not force and os.path.exists(out)
            and os.path.getmtime(out) >= os.path.getmtime(SRC)
            and os.path.getmtime(out) >= os.path.getmtime(SRC.replace(".cpp", ".h"))):
        return out
    flags = ["-O3", "-ffp-contract=fast"] if timing else ["-O2", "-ffp-contract=off"]
    cmd = ["g++"] + flags + ["-fopenmp", "-fPIC", "-shared", "-std=c++17", "-o", out + ".tmp",
                             SRC]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


class StepInfo(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("nlit", ctypes.c_int), ("conv", ctypes.c_double),
                ("xkx", ctypes.c_double), ("res_u", ctypes.c_double),
                ("res_p", ctypes.c_double)]


_libs = {}


def lib(timing=False):
    if timing not in _libs:
        L = ctypes.CDLL(build(timing=timing))
        L.or_element_flops.restype = ctypes.c_double
        L.or_destroy.restype = None
        _libs[timing] = L
    return _libs[timing]


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleError(RuntimeError):
    pass


def _check(st, what):
    if st != 0:
        raise OracleError("%s failed with status %d" % (what, st))


class Oracle:
    """One mesh + state, mirroring the reference's mesh/solv macros.

    Arrays use the Fortran layouts transposed into C order: ix (numel, nen+1),
    id (nnode, 4) restraint flags, x (nnode, 3), e (numat, 15), u (nnode, 4).
    """

    def __init__(self, nnode, nnodev, numel, nen, nenv, ix, idf, fnno, x, ie, e, num=None,
                 timing=False):
        L = self._L = lib(timing)
        self.nnode, self.numel, self.nen, self.nenv = nnode, numel, nen, nenv
        self._keep = [_i32(ix), _i32(idf), _i32(fnno), _f64(x), _i32(ie), _f64(e)]
        numa = None if num is None else _i32(num)
        h = ctypes.c_void_p()
        _check(L.or_create(nnode, nnodev, numel, nen, nenv, 4, _p(self._keep[0]),
                           _p(self._keep[1]), _p(self._keep[2]), _p(self._keep[3]),
                           len(ie), _p(self._keep[4]), _p(self._keep[5]), _p(numa),
                           ctypes.byref(h)), "or_create")
        self.h = h
        neq = ctypes.c_int()
        nad = ctypes.c_int64()
        nc = ctypes.c_int()
        L.or_sizes(h, ctypes.byref(neq), ctypes.byref(nad), ctypes.byref(nc))
        self.neq, self.nad, self.numcolors = neq.value, nad.value, nc.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self._L.or_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def set_loads(self, eload=None, eloadp=None, nload=None, f=None, load=None, fload=None):
        L = self._L
        keep = [None if a is None else _i32(a) for a in (eload, eloadp, nload)]
        fa = None if f is None else _f64(f)
        nl = 0 if load is None else len(load)
        la = None if load is None else _i32(load)
        fl = None if fload is None else _f64(fload)
        maxt = 1 if fload is None else fload.shape[-1]
        _check(L.or_set_loads(self.h, _p(keep[0]), _p(keep[1]), _p(keep[2]), _p(fa), nl, maxt,
                              _p(la), _p(fl)), "or_set_loads")

    def set_env(self, gravity, dt, t=0.0, istep=0):
        g = _f64(gravity)
        _check(self._L.or_set_env(self.h, _p(g), ctypes.c_double(dt), ctypes.c_double(t), istep),
               "or_set_env")

    def set_state(self, u=None, u0=None, dp=None):
        a = [None if v is None else _f64(v) for v in (u, u0, dp)]
        _check(self._L.or_set_state(self.h, _p(a[0]), _p(a[1]), _p(a[2])), "or_set_state")

    def get_state(self):
        u = np.zeros((self.nnode, 4))
        u0 = np.zeros((self.nnode, 4))
        dp = np.zeros(self.nnode)
        _check(self._L.or_get_state(self.h, _p(u), _p(u0), _p(dp)), "or_get_state")
        return u, u0, dp

    def stress(self):
        """tform_pm isw 3 + effective_stress: total, Biot and effective stress
        (nnode, 6) and Darcy flux (nnode, 3) of the current state."""
        tx, txb, txe = np.zeros((self.nnode, 6)), np.zeros((self.nnode, 6)), np.zeros((self.nnode, 6))
        fl = np.zeros((self.nnode, 3))
        _check(self._L.or_stress(self.h, _p(tx), _p(txb), _p(txe), _p(fl)), "or_stress")
        return tx, txb, txe, fl

    def set_nkrylov(self, k):
        _check(self._L.or_set_nkrylov(self.h, int(k)), "or_set_nkrylov")

    def get_porosity(self):
        poro = np.zeros(self.nnode)
        _check(self._L.or_get_porosity(self.h, _p(poro)), "or_get_porosity")
        return poro

    def set_porosity(self, poro):
        a = _f64(poro)
        _check(self._L.or_set_porosity(self.h, _p(a)), "or_set_porosity")

    def get_id(self):
        idr = np.zeros((self.nnode, 4), np.int32)
        _check(self._L.or_get_id(self.h, _p(idr)), "or_get_id")
        return idr

    def get_csrd(self):
        ia = np.zeros(self.neq + 1, np.int64)
        ja = np.zeros(self.nad, np.int32)
        ad = np.zeros(self.neq)
        al = np.zeros(self.nad)
        _check(self._L.or_get_csrd(self.h, _p(ia), _p(ja), _p(ad), _p(al)), "or_get_csrd")
        return ia, ja, ad, al

    def set_csrd_values(self, ad, al):
        a, b = _f64(ad), _f64(al)
        _check(self._L.or_set_csrd_values(self.h, _p(a), _p(b)), "or_set_csrd_values")

    def element(self, nel, isw, ul, dpl):
        nst = 3 * self.nen + self.nenv
        s = np.zeros((nst, nst))
        p = np.zeros(nst)
        u, d = _f64(ul), _f64(dpl)
        _check(self._L.or_element(self.h, nel, isw, _p(u), _p(d), _p(s), _p(p)), "or_element")
        return s.T.copy(), p  # s is column-major in the reference

    def pform(self, isw, lhs, rhs, u, b, nthreads=1):
        ua = _f64(u)
        assert b.dtype == np.float64 and b.flags.c_contiguous
        _check(self._L.or_pform(self.h, isw, int(lhs), int(rhs), _p(ua), _p(b), nthreads),
               "or_pform")
        return b

    def pform_range(self, isw, lhs, rhs, u, b, nthreads, e_begin, e_end):
        ua = _f64(u)
        _check(self._L.or_pform_range(self.h, isw, int(lhs), int(rhs), _p(ua), _p(b), nthreads,
                                    e_begin, e_end), "or_pform_range")
        return b

    def matvec(self, x, nthreads=1):
        xa = _f64(x)
        y = np.zeros(self.neq)
        _check(self._L.or_matvec(self.h, _p(xa), _p(y), nthreads), "or_matvec")
        return y

    def solve(self, b, solver=1, precond=2, tol=1e-11, maxit=50000, nthreads=1):
        ba = _f64(b)
        x = np.zeros(self.neq)
        info = StepInfo()
        _check(self._L.or_solve(self.h, solver, precond, _p(ba), _p(x), ctypes.c_double(tol),
                              maxit, nthreads, ctypes.byref(info)), "or_solve")
        return x, info

    def step(self, maxnlit=2, tol=1e-4, stop_crit=2, solver=1, precond=2, solvtol=1e-11,
             maxit=50000, nthreads=1):
        info = StepInfo()
        _check(self._L.or_step(self.h, maxnlit, ctypes.c_double(tol), stop_crit, solver, precond,
                             ctypes.c_double(solvtol), maxit, nthreads, ctypes.byref(info)),
               "or_step")
        return info


def reord(nnode, numel, nen, ix, afl=True):
    """reord (Reord.f:1-44): the reverse Cuthill-McKee node permutation,
    num[i] = the (1-based) node visited i-th; ix is (numel, nen+1)."""
    num = np.zeros(int(nnode), np.int32)
    ixa = _i32(ix)
    _check(lib().or_reord(int(nnode), int(numel), int(nen), _p(ixa), int(bool(afl)), _p(num)),
           "or_reord")
    return num


def element_flops(nen, isw=2):
    return lib().or_element_flops(nen, isw)


def from_fixture(fx):
    """Oracle for a golden fixture (tests/golden/*.npz) with its loads and
    initial state applied."""
    o = Oracle(int(fx["nnode"]), int(fx["nnodev"]), int(fx["numel"]), int(fx["nen"]),
               int(fx["nenv"]), fx["ix"], fx["id"], fx["fnno"], fx["x"], fx["ie"], fx["e"])
    o.set_loads(eload=fx["eload"], load=fx["load"] if len(fx["load"]) else None,
                fload=fx["fload"] if len(fx["load"]) else None)
    o.set_env(fx["gravity"], float(fx["dt"]))
    o.set_state(u=fx["u0"], u0=fx["u0"])
    return o
