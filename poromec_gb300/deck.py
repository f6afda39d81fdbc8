"""Input decks of the reference, read and run by the library (pm_deck_* in
include/poromec_gb300.h): the macro program of Main.f and the mesh macro of
rdat_pm (Rdata.f:1-1037), linear meshes made quadratic as the reference does
(mk_elconn_quad_v1, Adjacency.f:583-700), and a runner for loop / solv / pnup /
pnsf writing the printnode history files (Pdata.f:733-790).

    d = Deck("exemplo1_mesh0_t2.dat")
    pb = d.problem()          # arrays in the poromec_gb300.from_problem layout
    m, nsteps = d.run("out/exemplo1_mesh0_t2", fmt="golden")

Reading needs no GPU; creating the mesh and running do.
"""
import ctypes
import os
import sys

import numpy as np

from . import capi


class DeckError(RuntimeError):
    pass


_INT_SHAPES = {"ix": ("numel", "nen+1"), "id": ("nnode", 4), "nload": ("nnode", 4),
               "eload": ("numel", 7), "eloadp": ("numel", 7), "fnno": ("nnode",),
               "load": ("nloads", 3), "ie": ("numat",), "print_nodes": (-1,)}
_REAL_SHAPES = {"e": ("numat", capi.PM_PROP), "x": ("nnode", 3), "f": ("nnode", 4),
                "u0": ("nnode", 4), "tx0": ("nnode", 6),
                "fload": ("nloads", capi.PM_NFLOAD, "maxt")}


class Deck:
    """A parsed deck.  Arrays come back as copies in C order, transposed from
    the Fortran layouts as in poromec_gb300.capi."""

    def __init__(self, path):
        self.lib = capi.load()
        self.path = os.fspath(path)
        d = ctypes.c_void_p()
        st = self.lib.pm_deck_read(self.path.encode(), ctypes.byref(d))
        if st != 0:
            raise DeckError("%s: %s" % (self.path, self.lib.pm_deck_error().decode()))
        self.d = d

    def __del__(self):
        try:
            if getattr(self, "d", None):
                self.lib.pm_deck_free(self.d)
                self.d = None
        except Exception:
            pass

    def value(self, name):
        v = ctypes.c_double()
        if self.lib.pm_deck_value(self.d, name.encode(), ctypes.byref(v)) != 0:
            raise KeyError(name)
        return v.value

    def _dims(self, shape):
        out = []
        for s in shape:
            if s == "nen+1":
                out.append(int(self.value("nen")) + 1)
            elif isinstance(s, str):
                out.append(int(self.value(s)))
            else:
                out.append(s)
        return out

    def ints(self, name):
        p, n = ctypes.POINTER(ctypes.c_int32)(), ctypes.c_int64()
        if self.lib.pm_deck_int_array(self.d, name.encode(), ctypes.byref(p),
                                      ctypes.byref(n)) != 0:
            raise KeyError(name)
        a = np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0, np.int32)
        return a.reshape(self._dims(_INT_SHAPES[name]))

    def reals(self, name):
        p, n = ctypes.POINTER(ctypes.c_double)(), ctypes.c_int64()
        if self.lib.pm_deck_real_array(self.d, name.encode(), ctypes.byref(p),
                                       ctypes.byref(n)) != 0:
            raise KeyError(name)
        a = np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0)
        return a.reshape(self._dims(_REAL_SHAPES[name]))

    def problem(self):
        """The mesh, loads, initial state and settings as a problem dict
        (the keys poromec_gb300.from_problem reads, plus tx0 and the solver
        settings in force at the deck's first solv)."""
        pb = {k: int(self.value(k)) for k in ("nnode", "nnodev", "numel", "nen", "nenv")}
        for k in ("ix", "id", "fnno", "ie", "eload", "eloadp", "nload", "load", "print_nodes"):
            pb[k] = self.ints(k)
        for k in ("x", "e", "f", "u0", "tx0", "fload"):
            pb[k] = self.reals(k)
        pb["gravity"] = np.array([self.value("gravity_" + c) for c in "xyz"])
        for k in ("dt", "solvtol", "tol"):
            pb[k] = self.value(k)
        for k in ("solver", "precond", "maxit", "maxnlit", "stop_crit", "nkrylov", "fstress0"):
            pb[k] = int(self.value(k))
        return pb

    def mesh(self):
        """A device mesh with the deck's loads, gravity, dt, initial state and
        initial stress (pm_deck_create)."""
        h = ctypes.c_void_p()
        st = self.lib.pm_deck_create(self.d, ctypes.byref(h))
        if st != 0:
            raise capi.PMError(st, "pm_deck_create")
        return capi.Mesh.adopt(h, self.value("nnode"), self.value("numel"), self.value("nen"),
                               self.value("nenv"))

    def write_geo(self, prefix, quad=False):
        """<prefix>_bc.vtk: the mesh as read (the pgeo macro)."""
        st = self.lib.pm_deck_write_geo(self.d, os.fspath(prefix).encode(), int(bool(quad)))
        if st != 0:
            raise DeckError(self.lib.pm_deck_error().decode())
        return os.fspath(prefix) + "_bc.vtk"

    def write_res(self, mesh, prefix, istep, t, quad=True, fields=0x3F):
        """<prefix>_istep_<istep>.vtk: the state of mesh (the pres macro);
        fields bits: 1 deltaPressao, 2 totalStress, 4 terzaghiStress,
        8 BiotStress, 16 darcyFlux, 32 porosity."""
        st = self.lib.pm_deck_write_res(self.d, mesh.h, os.fspath(prefix).encode(), int(istep),
                                        float(t), int(bool(quad)), int(fields))
        if st != 0:
            raise capi.PMError(st, "pm_deck_write_res")
        return "%s_istep_%d.vtk" % (os.fspath(prefix), istep)

    def run(self, prefix, fmt="printnode", mesh=None):
        """Run the deck's macro program; history files go to <prefix>_*.txt.
        fmt 'printnode' writes the reference's (i9,10e18.10) rows, 'golden'
        the column layout of the golden runs shipped with the reference."""
        m = mesh or self.mesh()
        n = ctypes.c_int()
        st = self.lib.pm_deck_run(self.d, m.h, os.fspath(prefix).encode(),
                                  {"printnode": 0, "golden": 1}[fmt], ctypes.byref(n))
        if st != 0:
            detail = self.lib.pm_deck_error().decode() or m.lib.pm_last_error(m.h).decode()
            raise capi.PMError(st, "pm_deck_run", detail)
        return m, n.value


def read_history(path):
    """Rows (istep, t, values...) of a printnode history file."""
    rows = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#"):
                continue
            rows.append([float(v.replace("D", "E")) for v in line.split()])
    return np.array(rows)


def read_vtk(path):
    """Arrays of a legacy ASCII VTK unstructured grid (the reference's
    _bc.vtk / _istep_N.vtk files, or ours): dict with points (n, 3), cells
    (list of node-index arrays), cell_types, point_data and cell_data
    ({name: (n, ncomp) array}) and the FieldData values (TIME_S, CYCLE ...)."""
    with open(path, errors="replace") as fh:
        lines = fh.read().splitlines()
    toks = []
    for ln in lines[4:]:
        toks.extend(ln.split())
    out = {"point_data": {}, "cell_data": {}, "field": {}}
    i, section = 0, None

    def nums(count, conv=float):
        nonlocal i
        v = [conv(t.replace("D", "E")) for t in toks[i:i + count]]
        i += count
        return v

    while i < len(toks):
        key = toks[i]
        if key == "FIELD":
            nf = int(toks[i + 2])
            i += 3
            for _ in range(nf):
                name, nc, nt = toks[i], int(toks[i + 1]), int(toks[i + 2])
                i += 4
                out["field"][name] = nums(nc * nt)
        elif key == "POINTS":
            n = int(toks[i + 1])
            i += 3
            out["points"] = np.array(nums(3 * n)).reshape(n, 3)
        elif key == "CELLS":
            n, size = int(toks[i + 1]), int(toks[i + 2])
            i += 3
            flat = nums(size, int)
            cells, k = [], 0
            for _ in range(n):
                cells.append(np.array(flat[k + 1:k + 1 + flat[k]]))
                k += 1 + flat[k]
            out["cells"] = cells
        elif key == "CELL_TYPES":
            n = int(toks[i + 1])
            i += 2
            out["cell_types"] = np.array(nums(n, int))
        elif key in ("POINT_DATA", "CELL_DATA"):
            section = "point_data" if key == "POINT_DATA" else "cell_data"
            out[section + "_n"] = int(toks[i + 1])
            i += 2
        elif key == "SCALARS":
            name, typ = toks[i + 1], toks[i + 2]
            nc = 1
            j = i + 3
            if j < len(toks) and toks[j].isdigit():
                nc = int(toks[j])
                j += 1
            assert toks[j] == "LOOKUP_TABLE"
            i = j + 2
            n = out[section + "_n"]
            conv = int if typ == "int" else float
            out[section][name] = np.array(nums(n * nc, conv)).reshape(n, nc)
        elif key in ("VECTORS", "TENSORS"):
            name = toks[i + 1]
            i += 3
            n, nc = out[section + "_n"], 3 if key == "VECTORS" else 9
            out[section][name] = np.array(nums(n * nc)).reshape(n, nc)
        else:
            raise ValueError("unexpected VTK token %r in %s" % (key, path))
    return out


def main(argv=None):
    """python -m poromec_gb300.deck DECK [PREFIX] [printnode|golden]"""
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        print(main.__doc__)
        return 2
    deck = argv[0]
    prefix = argv[1] if len(argv) > 1 else os.path.splitext(deck)[0]
    fmt = argv[2] if len(argv) > 2 else "printnode"
    _, n = Deck(deck).run(prefix, fmt)
    print("%s: %d steps, histories in %s_*_node_*.txt" % (deck, n, prefix))
    return 0


if __name__ == "__main__":
    sys.exit(main())
