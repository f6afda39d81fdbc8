"""Seeded synthetic problems for the Biot hot path.

The reference reads its meshes from input decks; there is no public dataset.
These generators build the benchmark workloads (structured hexa20 boxes,
Kuhn-split tetra10 boxes, Gaussian random fields of permeability and
stiffness) directly as the arrays the reference's ``mesh`` macro produces:
ix (numel, nen+1) in the reference's local node order (elmt17_pm /
elmt15_pm node tables, Elmlib03.f), restraint flags id (nnode, 4),
vertex flags fnno, coordinates, per-element materials e (numat, 15), face
loads and load tables in the rload layout (Rdata.f:1487).

Node numbering walks the fine lattice of vertex and mid-edge points in
lexicographic order, so the equation numbering is banded without a
reordering pass.
"""
import numpy as np

PROP = 15
NFLOAD = 6

# local node -> lattice offset (0, 1, 2 along r, s, t) of the reference's
# hexa20 (sfhexa20_m node table, Elmlib.f:1619-1660)
_HEXA20 = [(2, 2, 2), (0, 2, 2), (0, 0, 2), (2, 0, 2), (2, 2, 0), (0, 2, 0), (0, 0, 0),
           (2, 0, 0), (1, 2, 2), (0, 1, 2), (1, 0, 2), (2, 1, 2), (1, 2, 0), (0, 1, 0),
           (1, 0, 0), (2, 1, 0), (2, 2, 1), (0, 2, 1), (0, 0, 1), (2, 0, 1)]
# tetra10 edges (local vertex pair -> local mid-edge node), Adjacency.f:1005
_TETRA10_EDGES = [(0, 1, 4), (0, 2, 5), (0, 3, 6), (1, 2, 7), (2, 3, 8), (3, 1, 9)]


def material_row(E, nu, K_h, M, alpha, rho=0.0, rho_f=1000.0):
    """e(1..7) of the elastic Biot elements: E [MPa], nu, hydraulic
    conductivity K_h [m/s], Biot modulus M [MPa], alpha, rho, rho_f [kg/m^3]."""
    e = np.zeros(PROP)
    e[:7] = [E, nu, K_h, M, alpha, rho, rho_f]
    return e


def conductivity(k_over_mu_si, rho_f=1000.0, g=10.0):
    """K_h [m/s] whose internal mobility K_h/(rho_f 1e-6 |g|) equals k/mu.
    k/mu given in m^2/(Pa s); the elements work in MPa, so the mobility is
    k/mu * 1e6 m^2/(MPa s) (Elmlib03.f:1961-1975)."""
    return np.asarray(k_over_mu_si) * 1.0e6 * rho_f * 1.0e-6 * g


def _lattice_ids(mask):
    ids = np.zeros(mask.shape, np.int64)
    flat = mask.ravel(order="F")  # a fastest, then b, then c
    ids_flat = np.cumsum(flat) * flat
    return ids_flat.reshape(mask.shape, order="F")


def hexa20_box(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0):
    """Structured hexa20 mesh of [0,lx]x[0,ly]x[0,lz]."""
    A, B, C = 2 * nx + 1, 2 * ny + 1, 2 * nz + 1
    a, b, c = np.meshgrid(np.arange(A), np.arange(B), np.arange(C), indexing="ij")
    odd = (a % 2) + (b % 2) + (c % 2)
    mask = odd <= 1
    ids = _lattice_ids(mask)
    nnode = int(mask.sum())
    x = np.zeros((nnode, 3))
    sel = ids[mask] - 1
    x[sel, 0] = a[mask] * (lx / (2 * nx))
    x[sel, 1] = b[mask] * (ly / (2 * ny))
    x[sel, 2] = c[mask] * (lz / (2 * nz))
    fnno = np.zeros(nnode, np.int32)
    fnno[ids[mask & (odd == 0)] - 1] = 1
    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ei, ej, ek = (v.ravel(order="F") for v in (ei, ej, ek))
    numel = nx * ny * nz
    ix = np.zeros((numel, 21), np.int32)
    for k, (oa, ob, oc) in enumerate(_HEXA20):
        ix[:, k] = ids[2 * ei + oa, 2 * ej + ob, 2 * ek + oc]
    ix[:, 20] = 1
    return dict(nnode=nnode, nnodev=int(fnno.sum()), numel=numel, nen=20, nenv=8, ix=ix, x=x,
                fnno=fnno, grid=(nx, ny, nz), elem_ijk=np.stack([ei, ej, ek], 1))


def tetra10_kuhn_box(nx, ny, nz, lx=2.0, ly=2.0, lz=1.0, jitter=0.1, seed=0):
    """Six Kuhn tetrahedra per hex cell; interior vertices jittered uniformly
    by +-jitter of the spacing; mid-edge nodes at the edge midpoints."""
    A, B, C = 2 * nx + 1, 2 * ny + 1, 2 * nz + 1
    a, b, c = np.meshgrid(np.arange(A), np.arange(B), np.arange(C), indexing="ij")
    mask = np.ones((A, B, C), bool)
    ids = _lattice_ids(mask)
    nnode = A * B * C
    h = np.array([lx / nx, ly / ny, lz / nz])
    # vertex positions (jittered inside)
    vi, vj, vk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    pos = np.stack([vi * h[0], vj * h[1], vk * h[2]], -1).astype(float)
    rng = np.random.default_rng(seed)
    interior = (vi > 0) & (vi < nx) & (vj > 0) & (vj < ny) & (vk > 0) & (vk < nz)
    jit = rng.uniform(-jitter, jitter, size=pos.shape) * h
    pos[interior] += jit[interior]
    x = np.zeros((nnode, 3))
    fnno = np.zeros(nnode, np.int32)
    vid = ids[0::2, 0::2, 0::2]
    x[vid.ravel() - 1] = pos.reshape(-1, 3)
    fnno[vid.ravel() - 1] = 1
    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ei, ej, ek = (v.ravel(order="F") for v in (ei, ej, ek))
    tets = []
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    for p in perms:
        v = np.zeros((len(ei), 4, 3), np.int64)
        base = np.stack([ei, ej, ek], 1)
        cur = base.copy()
        v[:, 0] = cur
        for s in range(3):
            cur = cur.copy()
            cur[:, p[s]] += 1
            v[:, s + 1] = cur
        tets.append(v)
    tv = np.concatenate(tets, 0)  # (numel, 4, 3) vertex grid indices
    numel = tv.shape[0]
    lat = 2 * tv  # lattice coordinates
    # orient: reference det = (x1-x4).((x2-x4)x(x3-x4)) > 0
    P = pos[tv[..., 0], tv[..., 1], tv[..., 2]]
    d = np.einsum("ij,ij->i", P[:, 0] - P[:, 3], np.cross(P[:, 1] - P[:, 3], P[:, 2] - P[:, 3]))
    flip = d < 0
    lat[flip, 0], lat[flip, 1] = lat[flip, 1].copy(), lat[flip, 0].copy()
    ix = np.zeros((numel, 11), np.int32)
    for k in range(4):
        ix[:, k] = ids[lat[:, k, 0], lat[:, k, 1], lat[:, k, 2]]
    for (p0, p1, m) in _TETRA10_EDGES:
        mid = (lat[:, p0] + lat[:, p1]) // 2
        ix[:, m] = ids[mid[:, 0], mid[:, 1], mid[:, 2]]
    ix[:, 10] = 1
    # mid-edge coordinates
    for (p0, p1, m) in _TETRA10_EDGES:
        x[ix[:, m] - 1] = 0.5 * (x[ix[:, p0] - 1] + x[ix[:, p1] - 1])
    used = np.zeros(nnode, bool)
    used[ix[:, :10].ravel() - 1] = True
    assert used.all(), "Kuhn lattice left unused nodes"
    return dict(nnode=nnode, nnodev=int(fnno.sum()), numel=numel, nen=10, nenv=4, ix=ix, x=x,
                fnno=fnno, grid=(nx, ny, nz))


def gaussian_random_field(shape, corr_len, spacing, seed=0):
    """Zero-mean, unit-variance stationary Gaussian field with Gaussian
    covariance exp(-r^2/(2 l^2)), sampled on a regular grid by spectral
    filtering of white noise (periodic FFT on a grid padded by 2 l)."""
    pad = [int(np.ceil(2 * corr_len / s)) for s in spacing]
    full = [n + p for n, p in zip(shape, pad)]
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(full)
    k = np.meshgrid(*[2 * np.pi * np.fft.fftfreq(n, d=s) for n, s in zip(full, spacing)],
                    indexing="ij")
    k2 = sum(kk ** 2 for kk in k)
    spec = np.exp(-0.25 * k2 * corr_len ** 2)  # sqrt of the Gaussian spectrum
    f = np.real(np.fft.ifftn(np.fft.fftn(noise) * spec))
    f = f[tuple(slice(0, n) for n in shape)]
    f = (f - f.mean()) / f.std()
    return f


def _faces_top_hexa(mesh):
    """elmtloads rows: face 1 (nodes 1-4, t = +1) of the elements on z = top."""
    nz = mesh["grid"][2]
    eload = np.zeros((mesh["numel"], 7), np.int32)
    top = mesh["elem_ijk"][:, 2] == nz - 1
    eload[top, 0] = 1
    return eload


def _load_table(times, values):
    """One type-40 load (rload layout): load(3) = (40, ncomp+1, ntimes) and
    fload(maxt, NFLOAD) with column 1 the times and 2..4 the vector."""
    times = np.asarray(times, float)
    values = np.asarray(values, float).reshape(len(times), 3)
    load = np.array([[40, 4, len(times)]], np.int32)
    fload = np.zeros((1, NFLOAD, len(times)))
    fload[0, 0] = times
    fload[0, 1:4] = values.T
    return load, fload


def _finish(mesh, idf, e, eload, load, fload, u0, gravity, dt, **kw):
    pb = dict(mesh)
    ne = len(e)
    pb.update(id=idf, ie=np.full(ne, 17 if mesh["nen"] == 20 else 15, np.int32), e=e,
              eload=eload, load=load, fload=fload, u0=u0, gravity=np.asarray(gravity, float),
              dt=float(dt))
    pb.update(kw)
    return pb


def column_problem(nx=2, ny=2, nz=40, lx=1.0, ly=1.0, lz=10.0):
    """1-D consolidation column (structured 2x2x40 hexa20, 1x1x10 m): E = 100
    MPa, nu = 0.3, alpha = 1, M = 1e4 MPa, k/mu = 1e-9 m^2/(Pa s); lateral
    rollers, base fixed in z, drained top (p = 0), undrained base; 1 MPa
    step load on top from t = 0; 20 steps of 10 s; diag-PCG tol 1e-10."""
    m = hexa20_box(nx, ny, nz, lx, ly, lz)
    x = m["x"]
    tol = 1e-9
    idf = np.zeros((m["nnode"], 4), np.int32)
    idf[np.abs(x[:, 0]) < tol, 0] = 1
    idf[np.abs(x[:, 0] - lx) < tol, 0] = 1
    idf[np.abs(x[:, 1]) < tol, 1] = 1
    idf[np.abs(x[:, 1] - ly) < tol, 1] = 1
    idf[np.abs(x[:, 2]) < tol, 2] = 1
    top = np.abs(x[:, 2] - lz) < tol
    idf[top & (m["fnno"] == 1), 3] = 1
    rho_f, g = 1000.0, 10.0
    e = material_row(100.0, 0.3, conductivity(1e-9, rho_f, g), 1.0e4, 1.0, 0.0, rho_f)[None]
    load, fload = _load_table([0.0], [[0.0, 0.0, -1.0]])
    u0 = np.zeros((m["nnode"], 4))
    # hydrostatic initial pressure (the gravity Darcy term then cancels), p = 0 on top
    u0[:, 3] = rho_f * 1e-6 * g * (lz - x[:, 2]) * m["fnno"]
    u0[idf[:, 3] == 1, 3] = 0.0
    return _finish(m, idf, e, _faces_top_hexa(m), load, fload, u0, [0.0, 0.0, -g], 10.0,
                   nsteps=20, solver=1, precond=2, solvtol=1e-10, maxit=50000, maxnlit=2,
                   name="column hexa20 2x2x40")


def cube_problem(n=56, seed=2024, steps=50):
    """Heterogeneous cube: 1x1x1 m, structured n^3 hexa20, log k Gaussian
    random field (mean ln 1e-14 m^2, sigma 1, correlation length 0.1 m) with
    mu = 1e-3 Pa s, E lognormal (median 1 GPa, sigma_ln 0.3), nu = 0.25,
    alpha = 1, M = 1e4 MPa, one material per element; base fixed, drained
    top, top traction ramped to 5 MPa over 10 steps; dt = 100 s."""
    m = hexa20_box(n, n, n, 1.0, 1.0, 1.0)
    x = m["x"]
    tol = 1e-9
    idf = np.zeros((m["nnode"], 4), np.int32)
    base = np.abs(x[:, 2]) < tol
    idf[base, 0:3] = 1
    top = np.abs(x[:, 2] - 1.0) < tol
    idf[top & (m["fnno"] == 1), 3] = 1
    h = 1.0 / n
    logk = np.log(1e-14) + 1.0 * gaussian_random_field((n, n, n), 0.1, (h, h, h), seed)
    logE = np.log(1000.0) + 0.3 * gaussian_random_field((n, n, n), 0.1, (h, h, h), seed + 1)
    ijk = m["elem_ijk"]
    kel = np.exp(logk[ijk[:, 0], ijk[:, 1], ijk[:, 2]])
    Eel = np.exp(logE[ijk[:, 0], ijk[:, 1], ijk[:, 2]])
    rho_f, g, mu = 1000.0, 10.0, 1.0e-3
    e = np.zeros((m["numel"], PROP))
    e[:, 0] = Eel
    e[:, 1] = 0.25
    e[:, 2] = conductivity(kel / mu, rho_f, g)
    e[:, 3] = 1.0e4
    e[:, 4] = 1.0
    e[:, 6] = rho_f
    ix = m["ix"].copy()
    ix[:, 20] = np.arange(1, m["numel"] + 1)
    m["ix"] = ix
    dt = 100.0
    load, fload = _load_table([0.0, 10 * dt], [[0.0, 0.0, 0.0], [0.0, 0.0, -5.0]])
    u0 = np.zeros((m["nnode"], 4))
    u0[:, 3] = rho_f * 1e-6 * g * (1.0 - x[:, 2]) * m["fnno"]
    u0[idf[:, 3] == 1, 3] = 0.0
    return _finish(m, idf, e, _faces_top_hexa(m), load, fload, u0, [0.0, 0.0, -g], dt,
                   nsteps=steps, solver=1, precond=2, solvtol=1e-8, maxit=100000, maxnlit=2,
                   name="heterogeneous cube hexa20 %d^3" % n)


def tetra_problem(n=48, seed=7, steps=30):
    """Unstructured tetra10: n^3 hex cells on a 2x2x1 m box split in 6 Kuhn
    tets, interior vertices jittered +-10 %; two layers at z = 0.5
    (E 500 MPa / 2 GPa, k 1e-13 / 1e-15 m^2, mu = 1e-3 Pa s), alpha = 1,
    M = 1e4 MPa; base fixed, lateral rollers, drained top; point source of
    1e-6 m^3/s at the box centre as a nodal load on its pressure dof
    (pload_pm: b = -dt f); dt = 60 s; MINRES."""
    m = tetra10_kuhn_box(n, n, n, 2.0, 2.0, 1.0, 0.1, seed)
    x = m["x"]
    tol = 1e-9
    idf = np.zeros((m["nnode"], 4), np.int32)
    idf[np.abs(x[:, 2]) < tol, 0:3] = 1
    idf[np.abs(x[:, 0]) < tol, 0] = 1
    idf[np.abs(x[:, 0] - 2.0) < tol, 0] = 1
    idf[np.abs(x[:, 1]) < tol, 1] = 1
    idf[np.abs(x[:, 1] - 2.0) < tol, 1] = 1
    top = np.abs(x[:, 2] - 1.0) < tol
    idf[top & (m["fnno"] == 1), 3] = 1
    rho_f, g, mu = 1000.0, 10.0, 1.0e-3
    lower = material_row(500.0, 0.25, conductivity(1e-13 / mu, rho_f, g), 1.0e4, 1.0, 0.0, rho_f)
    upper = material_row(2000.0, 0.25, conductivity(1e-15 / mu, rho_f, g), 1.0e4, 1.0, 0.0, rho_f)
    e = np.stack([lower, upper])
    ix = m["ix"].copy()
    zc = x[ix[:, :4] - 1, 2].mean(1)
    ix[:, 10] = np.where(zc < 0.5, 1, 2)
    m["ix"] = ix
    centre = np.argmin(np.sum((x - np.array([1.0, 1.0, 0.5])) ** 2, 1) + (1 - m["fnno"]) * 1e9)
    nload = np.zeros((m["nnode"], 4), np.int32)
    nload[centre, 3] = 1
    load = np.array([[1, 1, 1]], np.int32)
    fload = np.zeros((1, NFLOAD, 1))
    fload[0, 0, 0] = 1.0e-6
    u0 = np.zeros((m["nnode"], 4))
    u0[:, 3] = rho_f * 1e-6 * g * (1.0 - x[:, 2]) * m["fnno"]
    u0[idf[:, 3] == 1, 3] = 0.0
    return _finish(m, idf, e, np.zeros((m["numel"], 7), np.int32), load, fload, u0,
                   [0.0, 0.0, -g], 60.0, nload=nload, nsteps=steps, solver=7, precond=2,
                   solvtol=1e-8, maxit=100000, maxnlit=2, name="tetra10 Kuhn %d^3" % n)


def batch_instances(ninst=96, nmin=8, nmax=32, seed=4242):
    """Instances of the batched workload: ninst unit cubes, structured
    hexa20 with an edge count drawn uniformly from nmin..nmax, each with its
    own E (lognormal, median 1 GPa, sigma_ln 0.3) and log k (normal, mean
    ln 1e-14 m^2, sigma 1; mu = 1e-3 Pa s), nu = 0.25, alpha = 1,
    M = 1e4 MPa, and the loading of the consolidation column: lateral
    rollers, base fixed in z, drained top, 1 MPa top load from t = 0,
    hydrostatic initial pressure, dt = 10 s."""
    rng = np.random.default_rng(seed)
    out = []
    rho_f, g, mu = 1000.0, 10.0, 1.0e-3
    for _ in range(ninst):
        n = int(rng.integers(nmin, nmax + 1))
        E = 1000.0 * float(np.exp(0.3 * rng.standard_normal()))
        k = float(np.exp(np.log(1e-14) + rng.standard_normal()))
        m = hexa20_box(n, n, n, 1.0, 1.0, 1.0)
        x = m["x"]
        tol = 1e-9
        idf = np.zeros((m["nnode"], 4), np.int32)
        idf[np.abs(x[:, 0]) < tol, 0] = 1
        idf[np.abs(x[:, 0] - 1.0) < tol, 0] = 1
        idf[np.abs(x[:, 1]) < tol, 1] = 1
        idf[np.abs(x[:, 1] - 1.0) < tol, 1] = 1
        idf[np.abs(x[:, 2]) < tol, 2] = 1
        top = np.abs(x[:, 2] - 1.0) < tol
        idf[top & (m["fnno"] == 1), 3] = 1
        e = material_row(E, 0.25, conductivity(k / mu, rho_f, g), 1.0e4, 1.0, 0.0, rho_f)[None]
        load, fload = _load_table([0.0], [[0.0, 0.0, -1.0]])
        u0 = np.zeros((m["nnode"], 4))
        u0[:, 3] = rho_f * 1e-6 * g * (1.0 - x[:, 2]) * m["fnno"]
        u0[idf[:, 3] == 1, 3] = 0.0
        out.append(_finish(m, idf, e, _faces_top_hexa(m), load, fload, u0, [0.0, 0.0, -g],
                           10.0, nsteps=20, solver=1, precond=2, solvtol=1e-10, maxit=50000,
                           maxnlit=2, name="batch instance hexa20 %d^3" % n, n=n))
    return out


def union_problem(instances):
    """One problem holding independent instances side by side (node ids
    offset, one material per instance, the load table of the first
    instance, which all instances share) with their node ranges in
    inst_node_ptr, for a batched handle."""
    ptr = [0]
    ix, x, fnno, idf, u0, eload, e = [], [], [], [], [], [], []
    for k, pb in enumerate(instances):
        off = ptr[-1]
        a = pb["ix"].copy()
        a[:, :pb["nen"]] += off
        a[:, pb["nen"]] = k + 1
        ix.append(a)
        x.append(pb["x"])
        fnno.append(pb["fnno"])
        idf.append(pb["id"])
        u0.append(pb["u0"])
        eload.append(pb["eload"])
        e.append(np.asarray(pb["e"]).reshape(-1, PROP)[0])
        ptr.append(off + int(pb["nnode"]))
    first = instances[0]
    pb = dict(nnode=ptr[-1], nnodev=int(sum(int(p["nnodev"]) for p in instances)),
              numel=int(sum(int(p["numel"]) for p in instances)), nen=first["nen"],
              nenv=first["nenv"], ix=np.concatenate(ix), x=np.concatenate(x),
              fnno=np.concatenate(fnno), id=np.concatenate(idf), u0=np.concatenate(u0),
              eload=np.concatenate(eload), e=np.stack(e),
              ie=np.full(len(instances), int(first["ie"][0]), np.int32),
              load=first["load"], fload=first["fload"], gravity=first["gravity"],
              dt=first["dt"], inst_node_ptr=np.asarray(ptr, np.int32),
              nsteps=first.get("nsteps"), solver=1, precond=2, solvtol=first.get("solvtol"),
              maxit=first.get("maxit"), maxnlit=first.get("maxnlit"),
              name="batch of %d instances" % len(instances))
    return pb


def partition_instances(edges, world):
    """Instances of a batch split over world ranks, balanced by estimated
    work (nonzeros grow as n^3 for an n^3 cube): largest first, each to the
    rank with the least work so far.  Returns one sorted index list per rank;
    the ranks solve their shares independently (no exchange in the solve)."""
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(edges)), key=lambda k: (-int(edges[k]) ** 3, k)):
        r = min(range(world), key=lambda j: (load[j], j))
        parts[r].append(i)
        load[r] += float(edges[i]) ** 3
    return [sorted(p) for p in parts]
