"""Convert the reference's golden runs into compact test fixtures.

The reference (lmn-labest/poroMec) ships six complete runs under
output/poro_mec/elastico/{hexa,tetra}: the input decks (old macro syntax), the
per-step node histories printed by ``printnode`` (Pdata.f:733-790, format
``(i9,10e18.10)``), the solver log (one PCG line per solve) and the timer file
with neq/nad.  This script, run once in a container where the reference is
mounted, parses each deck, rebuilds the quadratic mesh exactly as the reference
does when it reads a linear one (Rdata.f:477-520 + mk_elconn_quad_v1,
Adjacency.f:583-700; mk_coor_quad, Adjacency.f:907-955; mk_bound_quad,
Rdata.f:2337-2405; boundc, Rdata.f:1729-1749), and writes one ``.npz`` per case
holding the mesh arrays, loads, initial state, solver settings and the expected
outputs.  The fixtures are what the tests read; nothing at test time touches
the reference tree.

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT
        (or with the environment variable POROMEC_REFERENCE set to it)
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

HEXA20_EDGES = [(1, 2, 9), (2, 3, 10), (3, 4, 11), (4, 1, 12), (5, 6, 13), (6, 7, 14),
                (7, 8, 15), (8, 5, 16), (1, 5, 17), (2, 6, 18), (3, 7, 19), (4, 8, 20)]
TETRA10_EDGES = [(1, 2, 5), (1, 3, 6), (1, 4, 7), (2, 3, 8), (3, 4, 9), (4, 2, 10)]

CASES = [
    ("hexa", "exemplo1_mesh0_t2.dat", "exemplo1_mesh0_t2"),
    ("tetra", "exemplo1_mesh0_t2_tetra.dat", "exemplo1_mesh0_t2_tetra"),
    ("hexa", "solo1.dat", "solo1"),
    ("tetra", "solo1_tetra.dat", "solo1_tetra"),
    ("hexa", "solo_cilindro_hexa_1.dat", "solo_cilindro_hexa_1"),
    ("tetra", "solo_cilindro_tetra_1.dat", "solo_cilindro_tetra_1"),
]


def fnum(tok):
    return float(tok.replace("d", "e").replace("D", "e"))


MISSING = []


def read_lines(path, base):
    """Deck lines with 'insert' files expanded; '//' and '#' lines dropped."""
    out = []
    with open(path, errors="replace") as fh:
        for raw in fh:
            line = raw.strip()
            if not line or line.startswith("//") or line.startswith("#"):
                continue
            toks = line.split()
            if toks[0] == "insert":
                inc = os.path.join(base, toks[1])
                if not os.path.exists(inc):
                    # solo1_tetra.dat names an element-load file the reference
                    # does not ship; the case is kept for its pattern counts.
                    MISSING.append(toks[1])
                    continue
                out.extend(read_lines(inc, base))
                continue
            if toks[0] == "return":
                continue
            out.append(toks)
    return out


def parse_deck(path):
    base = os.path.dirname(path)
    lines = read_lines(path, base)
    d = dict(gravity=[0.0, 0.0, -9.81], solver_tol=1e-11, maxit=50000, maxnlit=500,
             dt=1.0, nsteps=0, reord=True, elmtloads={}, loads={}, coords={},
             elems=[], restr={}, initialpres={}, print_nodes=[], materials={})
    i = 0
    block = None
    while i < len(lines):
        t = lines[i]
        key = t[0]
        if block is not None:
            if key == "end":
                block = None
            elif block == "config":
                for k in range(0, len(t) - 1, 2):
                    if t[k] == "reord":
                        d["reord"] = t[k + 1] == "true"
            elif block == "materials":
                d["materials"][int(t[0])] = (int(t[1]), [fnum(v) for v in t[2:]])
            elif block in ("hexa8", "tetra4"):
                nv = 8 if block == "hexa8" else 4
                d["elems"].append((int(t[0]), [int(v) for v in t[1:1 + nv]], int(t[1 + nv])))
                d["elem_kind"] = block
            elif block == "coordinates":
                d["coords"][int(t[0])] = [fnum(v) for v in t[1:4]]
            elif block == "constrainpmec":
                d["restr"][int(t[0])] = [int(v) for v in t[1:5]]
            elif block == "initialpres":
                d["initialpres"][int(t[0])] = fnum(t[1])
            elif block == "elmtloads":
                d["elmtloads"][int(t[0])] = [int(v) for v in t[1:]]
            elif block == "loads":
                d["loads"][int(t[0])] = (int(t[1]), int(t[2]), [fnum(v) for v in t[3:]])
            i += 1
            continue
        if key in ("config", "materials", "hexa8", "tetra4", "coordinates", "constrainpmec",
                   "initialpres", "elmtloads", "loads", "faceR1", "nodalsources"):
            block = key
        elif key == "pcg":
            d["solver"] = 1
            d["maxit"] = int(t[1])
            d["solver_tol"] = fnum(t[2])
        elif key == "gravity":
            d["gravity"] = [fnum(v) for v in t[1:4]]
        elif key == "nnode":
            kv = dict(zip(t[0::2], t[1::2]))
            d["nnodev"] = int(kv["nnode"])
            d["numel"] = int(kv["numel"])
        elif key == "setpnode":
            with open(os.path.join(base, t[1])) as fh:
                vals = [int(v) for v in fh.read().split()]
            d["print_nodes"] = vals[1:1 + vals[0]]
        elif key == "maxnlit":
            d["maxnlit"] = int(t[1])
        elif key == "dt":
            d["dt"] = fnum(t[1])
        elif key == "loop":
            d["nsteps"] = int(t[1])
        i += 1
    return d


def quadratic_mesh(d):
    """mk_elconn_quad_v1 / mk_coor_quad / mk_bound_quad restated."""
    hexa = d["elem_kind"] == "hexa8"
    nen, nenv = (20, 8) if hexa else (10, 4)
    edges = HEXA20_EDGES if hexa else TETRA10_EDGES
    nnodev, numel = d["nnodev"], d["numel"]
    ix = np.zeros((numel, nen + 1), np.int32)
    for (el, nodes, mat) in d["elems"]:
        ix[el - 1, :nenv] = nodes
        ix[el - 1, nen] = mat
    # vertex -> incident elements (nodegrade / elmincid)
    incid = [[] for _ in range(nnodev + 1)]
    for el in range(numel):
        for k in range(nenv):
            incid[ix[el, k]].append(el)
    nno = nnodev
    for el in range(numel):
        for j in range(nenv, nen):  # local slots nenv+1..nen (1-based)
            if ix[el, j] == 0:
                nno += 1
                ix[el, j] = nno
        for (a, b, c) in edges:
            no1, no2, no3 = ix[el, a - 1], ix[el, b - 1], ix[el, c - 1]
            for nel in incid[no1]:
                if nel == el:
                    continue
                for (a2, b2, c2) in edges:
                    v1, v2 = ix[nel, a2 - 1], ix[nel, b2 - 1]
                    if (no1 == v1 and no2 == v2) or (no1 == v2 and no2 == v1):
                        if ix[nel, c2 - 1] == 0:
                            ix[nel, c2 - 1] = no3
    nnode = nno
    x = np.zeros((nnode, 3))
    for n, c in d["coords"].items():
        x[n - 1] = c
    for el in range(numel):
        for (a, b, c) in edges:
            no1, no2, no3 = ix[el, a - 1], ix[el, b - 1], ix[el, c - 1]
            x[no3 - 1] = 0.5 * (x[no1 - 1] + x[no2 - 1])
    idf = np.zeros((nnode, 4), np.int32)
    for n, fl in d["restr"].items():
        idf[n - 1] = fl
    for el in range(numel):
        for (a, b, c) in edges:
            no1, no2, no3 = ix[el, a - 1], ix[el, b - 1], ix[el, c - 1]
            for k in range(3):
                if idf[no1 - 1, k] == 1 and idf[no2 - 1, k] == 1:
                    idf[no3 - 1, k] = 1
    fnno = np.zeros(nnode, np.int32)
    fnno[np.unique(ix[:, :nenv]) - 1] = 1
    return ix, x, idf, fnno, nen, nenv, nnode


def read_history(path):
    rows = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#"):
                continue
            rows.append([float(v) for v in line.split()])
    return np.array(rows)


def read_log(path):
    """Iteration counts and energy norms (x.Kx) of the solver log's PCG lines."""
    its, xkx = [], []
    with open(path) as fh:
        for line in fh:
            m = re.match(r"\s*PCG:\s+it\s+(\d+)\s+energy norm\s+(\S+)", line)
            if m:
                its.append(int(m.group(1)))
                xkx.append(float(m.group(2).replace("D", "E")))
    return np.array(its, np.int32), np.array(xkx)


def read_counts(path):
    out = {}
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if len(t) == 2 and t[0] in ("neq", "nad", "nnode", "numel"):
                out[t[0]] = int(t[1])
    return out


def convert(ref_root, kind, deck, prefix):
    del MISSING[:]
    ddir = os.path.join(ref_root, "output", "poro_mec", "elastico", kind)
    d = parse_deck(os.path.join(ddir, deck))
    ix, x, idf, fnno, nen, nenv, nnode = quadratic_mesh(d)
    numel = d["numel"]
    mats = sorted(d["materials"])
    e = np.zeros((len(mats), 15))
    ie = np.zeros(len(mats), np.int32)
    for k, ma in enumerate(mats):
        old, vals = d["materials"][ma]
        ie[k] = {7: 17, 6: 15}[old]  # old element codes of these decks
        e[k, :len(vals)] = vals
    eload = np.zeros((numel, 7), np.int32)
    for el, fl in d["elmtloads"].items():
        eload[el - 1, :len(fl)] = fl[:7]
    nl = max(d["loads"]) if d["loads"] else 0
    load = np.zeros((nl, 3), np.int32)
    fload = np.zeros((nl, 6, 1))  # (nloads, OR_NFLOAD, maxt=1): constant tables
    for nc, (ty, ncomp, vals) in d["loads"].items():
        load[nc - 1] = (ty, ncomp + 1, 1)
        fload[nc - 1, 0, 0] = 0.0           # time column
        fload[nc - 1, 1:1 + len(vals), 0] = vals
    u0 = np.zeros((nnode, 4))
    for n, p in d["initialpres"].items():
        u0[n - 1, 3] = p
    u0[idf == 1] = 0.0  # boundc: prescribed dofs take f = 0
    hist = {}
    for n in d["print_nodes"]:
        p = os.path.join(ddir, "%s_up_node_%d.txt" % (prefix, n))
        if os.path.exists(p):
            hist[n] = read_history(p)
    # tform_pm outputs of the same nodes: total, effective (stressE) and Biot
    # (stressB) stress, Darcy flux
    extra = {}
    for key, tag in (("hist_stress", "stress"), ("hist_stressE", "stressE"),
                     ("hist_stressB", "stressB"), ("hist_flux", "flux")):
        rows = {}
        for n in d["print_nodes"]:
            pth = os.path.join(ddir, "%s_%s_node_%d.txt" % (prefix, tag, n))
            if os.path.exists(pth):
                rows[n] = read_history(pth)
        if rows and sorted(rows) == sorted(hist):
            extra[key] = np.stack([rows[n] for n in sorted(rows)])
    # the pgeo geometry file of the run (legacy VTK): mesh and input fields
    vtk = {}
    bc = os.path.join(ddir, prefix + "_bc.vtk")
    if os.path.exists(bc):
        sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
        from poromec_gb300.deck import read_vtk
        g = read_vtk(bc)
        vtk["vtk_points"] = g["points"]
        vtk["vtk_cells"] = np.stack(g["cells"])
        vtk["vtk_types"] = g["cell_types"]
        for k, v in g["point_data"].items():
            vtk["vtkp_" + k] = v
        for k, v in g["cell_data"].items():
            vtk["vtkc_" + k] = v
    counts = read_counts(os.path.join(ddir, prefix + "_t_1.txt"))
    its, xkx = read_log(os.path.join(ddir, prefix + "_log_1.txt"))
    tol = d["solver_tol"] if d["solver_tol"] != 0.0 else 2.0 ** -53  # smachn
    hnodes = np.array(sorted(hist), np.int32)
    out = dict(nnode=nnode, nnodev=d["nnodev"], numel=numel, nen=nen, nenv=nenv,
               ix=ix, x=x, id=idf, fnno=fnno, e=e, ie=ie, eload=eload, load=load,
               fload=fload, u0=u0, gravity=np.array(d["gravity"]), dt=d["dt"],
               nsteps=d["nsteps"], maxnlit=d["maxnlit"], solver_tol=tol,
               maxit=d["maxit"], reord=int(d["reord"]), hist_nodes=hnodes,
               hist=np.stack([hist[n] for n in hnodes]) if len(hnodes) else np.zeros(0),
               pcg_iters=its, pcg_xkx=xkx, neq_ref=counts.get("neq", -1), nad_ref=counts.get("nad", -1),
               nnode_ref=counts.get("nnode", -1), complete=int(not MISSING), **extra, **vtk)
    name = os.path.join(HERE, prefix + ".npz")
    np.savez_compressed(name, **out)
    return name, counts, nnode


def check_library_reader(ref_root, kind, deck, prefix):
    """The library's deck reader (pm_deck_read) on the shipped deck must give
    the arrays of this script's restatement bit for bit."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from poromec_gb300.deck import Deck
    fx = np.load(os.path.join(HERE, prefix + ".npz"))
    pb = Deck(os.path.join(ref_root, "output", "poro_mec", "elastico", kind, deck)).problem()
    for k in ("ix", "id", "fnno", "x", "e", "ie", "eload", "load", "fload", "u0"):
        if pb[k].shape != fx[k].shape or not np.array_equal(pb[k], fx[k]):
            raise SystemExit("library deck reader differs on %s: %s" % (deck, k))
    if list(pb["print_nodes"]) != list(fx["hist_nodes"]):
        raise SystemExit("library deck reader differs on %s: setpnode" % deck)
    return True


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("POROMEC_REFERENCE")
    if not ref_root:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT (or set POROMEC_REFERENCE): "
                         "the root of a poroMec checkout holding output/poro_mec/elastico")
    for kind, deck, prefix in CASES:
        name, counts, nnode = convert(ref_root, kind, deck, prefix)
        checked = False
        if not MISSING:
            checked = check_library_reader(ref_root, kind, deck, prefix)
        print("%-28s nnode %6d (log %s) neq %s nad %s  library reader %s" % (
            os.path.basename(name), nnode, counts.get("nnode"), counts.get("neq"),
            counts.get("nad"), "identical" if checked else "skipped (deck incomplete)"))


if __name__ == "__main__":
    main()
