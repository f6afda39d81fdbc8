"""CPU-side checks of the C ABI and the host code (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from poromec_gb300 import build as gbuild
from poromec_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "poromec_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pm_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_every_declared_symbol():
    lib_path = gbuild.build()
    lib = ctypes.CDLL(lib_path)
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_status_strings_without_gpu():
    lib = ctypes.CDLL(gbuild.build())
    lib.pm_status_string.restype = ctypes.c_char_p
    assert lib.pm_status_string(0) == b"ok"
    assert b"converge" in lib.pm_status_string(4)


def test_python_status_table_matches_the_library():
    """capi.STATUS gives every status code the library's own text."""
    from poromec_gb300 import capi
    lib = ctypes.CDLL(gbuild.build())
    lib.pm_status_string.restype = ctypes.c_char_p
    src = open(os.path.join(ROOT, "include", "poromec_gb300.h")).read()
    codes = sorted(int(v) for v in re.findall(r"PM_(?:OK|E_[A-Z_]+)\s*=\s*(\d+)", src))
    assert codes == list(range(len(codes))) and len(codes) >= 11
    for c in codes:
        assert capi.STATUS[c] == lib.pm_status_string(c).decode(), c


def test_create_rejects_bad_arguments_without_touching_the_gpu():
    lib = ctypes.CDLL(gbuild.build())
    h = ctypes.c_void_p()
    # nen/nenv mismatch is rejected before any CUDA call
    st = lib.pm_mesh_create(10, 8, 1, 20, 4, 3, 4, None, None, None, None, 1, None, None,
                            None, ctypes.byref(h))
    assert st == 1


def test_hexa_mesh_generator():
    m = meshgen.hexa20_box(2, 3, 4, 1.0, 2.0, 3.0)
    assert m["numel"] == 24
    nv = 3 * 4 * 5
    assert m["nnodev"] == nv
    # vertices + one mid-edge node per edge
    edges = 2 * 4 * 5 + 3 * 3 * 5 + 3 * 4 * 4
    assert m["nnode"] == nv + edges
    ix = m["ix"]
    x = m["x"]
    # every element: positive Jacobian of the reference's vertex order
    v = x[ix[:, :8] - 1]
    assert np.all(v[:, 0, 0] > v[:, 1, 0]) and np.all(v[:, 0, 2] > v[:, 4, 2])
    mid = x[ix[:, 8] - 1]
    assert np.allclose(mid, 0.5 * (v[:, 0] + v[:, 1]))


def test_tetra_mesh_generator_orientation():
    m = meshgen.tetra10_kuhn_box(3, 3, 3, jitter=0.1, seed=1)
    assert m["numel"] == 6 * 27
    assert m["nnode"] == 7 ** 3
    x = m["x"]
    P = x[m["ix"][:, :4] - 1]
    det = np.einsum("ij,ij->i", P[:, 0] - P[:, 3], np.cross(P[:, 1] - P[:, 3], P[:, 2] - P[:, 3]))
    assert np.all(det > 0)


def test_random_field_moments():
    f = meshgen.gaussian_random_field((24, 24, 24), 0.1, (1 / 24,) * 3, seed=3)
    assert abs(f.mean()) < 1e-12 and abs(f.std() - 1) < 1e-12
    g = meshgen.gaussian_random_field((24, 24, 24), 0.1, (1 / 24,) * 3, seed=3)
    assert np.array_equal(f, g)


@pytest.mark.parametrize("nen", [20, 10])
def test_oracle_flop_count(nen):
    import oracle
    f = oracle.element_flops(nen)
    if nen == 20:
        assert 1.8e6 < f < 1.95e6
    else:
        assert 2e4 < f < 5e4


def _fortran_bindings(text):
    """name -> [(arg, passed by value)] for every ISO_C_BINDING interface in
    the integration guide's Fortran module."""
    lines, out, cur = [], {}, None
    for raw in text.splitlines():
        line = raw.split("!")[0].rstrip()
        if lines and lines[-1].endswith("&"):
            lines[-1] = lines[-1][:-1] + " " + line.strip()
        else:
            lines.append(line)
    for line in lines:
        m = re.search(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\(c,\s*name='(\w+)'\)",
                      line)
        if m:
            args = [a.strip() for a in m.group(2).split(",") if a.strip()]
            cur = (m.group(3), args, {})
            out[m.group(3)] = cur
            continue
        if cur and re.match(r"\s*end\s+(function|subroutine)", line):
            cur = None
            continue
        if cur and "::" in line:
            typ, names = line.split("::", 1)
            for nm in names.split(","):
                nm = nm.strip().split("(")[0]
                if nm:
                    cur[2][nm] = ("value" in typ, "c_ptr" in typ)
    return {k: [(a,) + decl[a] for a in args] for k, (_, args, decl) in out.items()}


def _c_prototypes(text):
    """name -> [param declaration] for every pm_* prototype of the header."""
    flat = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(pm_\w+)\s*\(([^;{]*?)\)\s*;", flat, flags=re.S):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = params
    return out


def test_fortran_bindings_match_the_header():
    """The Fortran ISO_C_BINDING module that the integration guide gives the
    reference's maintainers binds only functions the header declares, with
    the header's argument count, and passes each argument the way the C
    parameter takes it: numbers by value, arrays, strings and handle outputs
    by reference, and a type(c_ptr) by value only where C takes a pointer or
    an opaque handle (a nullable array is passed as c_loc(a) or c_null_ptr)."""
    guide = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    header = open(os.path.join(ROOT, "include", "poromec_gb300.h")).read()
    binds, protos = _fortran_bindings(guide), _c_prototypes(header)
    assert len(binds) >= 20
    for name, args in binds.items():
        assert name in protos, name
        params = protos[name]
        assert len(args) == len(params), (name, args, params)
        for (arg, by_value, is_cptr), p in zip(args, params):
            c_pointer = "*" in p
            handle = p.startswith(("pm_handle", "pm_deck"))
            if not by_value:
                assert c_pointer, (name, arg, p)
            elif is_cptr:
                assert c_pointer or handle, (name, arg, p)
            else:
                assert not c_pointer and not handle, (name, arg, p)


def test_ctypes_signatures_match_the_header():
    """Every argtypes list that the Python mirror (poromec_gb300/capi.py)
    declares has the header's length, and pointers, handles, ints and
    doubles in the header's places: a drifted signature would pass
    arguments in the wrong registers without any error."""
    from poromec_gb300 import capi
    lib = capi.load()
    protos = _c_prototypes(open(os.path.join(ROOT, "include", "poromec_gb300.h")).read())
    pointer_types = (ctypes.c_void_p, ctypes.c_char_p)
    checked = 0
    for name, params in protos.items():
        argtypes = getattr(lib, name).argtypes
        if argtypes is None:
            continue
        assert len(argtypes) == len(params), (name, argtypes, params)
        for a, p in zip(argtypes, params):
            if "*" in p or p.startswith(("pm_handle", "pm_deck")):
                assert a in pointer_types or issubclass(a, ctypes._Pointer), (name, p, a)
            elif p.startswith(("int ", "int32_t ")):
                assert a is ctypes.c_int, (name, p, a)
            elif p.startswith("double "):
                assert a is ctypes.c_double, (name, p, a)
            else:
                raise AssertionError((name, p, a))
        checked += 1
    assert checked >= 40
