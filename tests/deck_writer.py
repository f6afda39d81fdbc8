"""Decks written from the golden fixtures, in the macro syntax of the
reference's shipped runs (test helper).

A fixture holds the quadratic mesh that the reference builds from a linear
deck.  write_linear_deck writes the linear deck back: vertex coordinates,
hexa8 / tetra4 connectivity, vertex restraints, initial pressures, element
loads and inline type-40 loads, spread over 'insert' files like the shipped
decks, plus the macro program (pcg, gravity, setpnode, maxnlit, dt, pnup,
pnsf, loop / solv / next).  Reading it must give the fixture back.
"""
import os

import numpy as np


def _f(v):
    return repr(float(v)).replace("e", "d")


def write_linear_deck(fx, dirname, name, nsteps=None):
    os.makedirs(dirname, exist_ok=True)
    nen, nenv = int(fx["nen"]), int(fx["nenv"])
    nnodev, numel = int(fx["nnodev"]), int(fx["numel"])
    hexa = nen == 20
    ix = np.asarray(fx["ix"])
    idf = np.asarray(fx["id"])
    x = np.asarray(fx["x"])
    e = np.asarray(fx["e"]).reshape(-1, 15)
    ie = np.asarray(fx["ie"])
    u0 = np.asarray(fx["u0"])

    def put(fname, lines):
        with open(os.path.join(dirname, fname), "w") as fh:
            fh.write("\n".join(lines) + "\n")

    put(name + "_coor.dat", ["coordinates"] +
        ["%8d %s %s %s" % ((i + 1,) + tuple(_f(v) for v in x[i])) for i in range(nnodev)] +
        ["end coordinates", "return"])
    kind = "hexa8" if hexa else "tetra4"
    put(name + "_elem.dat", [kind] +
        [" ".join(str(v) for v in [k + 1] + list(ix[k, :nenv]) + [ix[k, nen]])
         for k in range(numel)] + ["end " + kind, "return"])
    put(name + "_initial.dat", ["initialpres"] +
        ["%d %s" % (i + 1, _f(u0[i, 3])) for i in range(nnodev) if u0[i, 3] != 0.0] +
        ["end initialpres", "return"])
    put("node.dat", [str(len(fx["hist_nodes"]))] + [str(int(n)) for n in fx["hist_nodes"]])
    lines = ["config", "memory 400 reord false", "end config",
             "pcg %d %s" % (int(fx["maxit"]), _f(fx["solver_tol"])),
             "gravity %s" % " ".join(_f(g) for g in fx["gravity"]),
             "mesh",
             "nnode %d numel %d ndf 4 numat %d maxno %d dim 3" % (nnodev, numel, len(ie), nen),
             "materials"]
    old = {17: 7, 15: 6}
    for k in range(len(ie)):
        vals = list(e[k])
        while vals and vals[-1] == 0.0 and len(vals) > 7:
            vals.pop()
        lines.append("%d %d %s" % (k + 1, old[int(ie[k])], " ".join(_f(v) for v in vals)))
    lines += ["end materials", "insert %s_coor.dat" % name, "insert %s_elem.dat" % name,
              "insert %s_initial.dat" % name, "constrainpmec"]
    for i in range(nnodev):
        if idf[i].any():
            lines.append("%d %s" % (i + 1, " ".join(str(int(v)) for v in idf[i])))
    lines.append("end constrainpmec")
    el = np.asarray(fx["eload"])
    lines.append("elmtloads")
    for k in range(numel):
        if el[k].any():
            lines.append("%d %s" % (k + 1, " ".join(str(int(v)) for v in el[k])))
    lines.append("end elmtloads")
    load, fload = np.asarray(fx["load"]), np.asarray(fx["fload"])
    lines.append("loads")
    for i in range(len(load)):
        ty, nparc = int(load[i, 0]), int(load[i, 1])
        vals = [fload[i, k, 0] for k in range(1, nparc)]
        lines.append("%d %d %d %s" % (i + 1, ty, nparc - 1, " ".join(_f(v) for v in vals)))
    lines += ["end loads", "end mesh", "setpnode node.dat", "pgeo",
              "maxnlit %d" % int(fx["maxnlit"]), "dt %s" % _f(fx["dt"]), "pnup", "pnsf",
              "loop %d" % int(nsteps if nsteps is not None else fx["nsteps"]), "solv", "pnup",
              "pnsf", "next", "stop"]
    path = os.path.join(dirname, name + ".dat")
    put(name + ".dat", lines)
    return path
