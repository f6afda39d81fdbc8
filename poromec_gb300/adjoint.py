"""Adjoint gradient of a time-stepped Biot misfit with respect to per-element
material parameters (no counterpart in the reference, which has no
gradient path).

Parameters: theta (numel, 3) = (log E, log c_k, log M) per element, where E
is Young's modulus (material column 1), c_k the hydraulic conductivity
(column 3, proportional to the permeability k, so d/dlog c_k = d/dlog k)
and M the Biot modulus (column 4).  The mesh has one material per element
(numat = numel).

Forward: the implicit Euler steps of the 'solv' macro (Main.f:876-1123) as
the library runs them; for these linear meshes each step solves
    K du_n = F_n - A s_{n-1} - g0,   s_n = s_{n-1} + (du_n, du_n,p)
with s = (u, dp) (the operators in include/poromec_gb300.h).  Misfit, at the
last step N:
    J = sum_s (u_z(N)[s] - tz[s])^2 + w_p sum_s (p(N)[s] - tp[s])^2
over displacement sensors and pressure sensors (node indices).

Reverse sweep (hand-written, not traced): states are checkpointed every c
steps (c ~ sqrt(N)); each segment is recomputed from its checkpoint, then
for n = N..1
    lam_n = K^-1 (mu_n + nu_n)            (one FP64 PCG solve, K symmetric)
    grad += element contractions of lam_n with dK/dtheta, dA/dtheta, dg0/dtheta
    mu_{n-1} = mu_n - [Kuu lam_u ; Kpp_perm lam_p],  nu_{n-1} = nu_n - Kpu lam_u
with mu_N = dJ/du_N, nu_N = 0.  torch.autograd.Function wraps it
(BiotMisfit.apply).  Library calls run on the handle's stream, so torch's
stream is synchronised before each of them.
"""
import math

import numpy as np
import torch

from . import capi


class TimeSteppedMisfit:
    """Misfit J(theta) of a problem dict (poromec_gb300.meshgen layout, one
    material per element) over nsteps steps, and its adjoint gradient."""

    def __init__(self, pb, nsteps, disp_sensors, tz, pres_sensors, tp, w_p=1.0,
                 solvtol=1e-12, maxit=400000, ckpt_every=None):
        if int(len(np.asarray(pb["e"]).reshape(-1, capi.PM_PROP))) != int(pb["numel"]):
            raise ValueError("per-element parameters need one material per element")
        self.pb = pb
        self.nsteps = int(nsteps)
        self.ds, self.tz = np.asarray(disp_sensors), np.asarray(tz, float)
        self.ps, self.tp = np.asarray(pres_sensors), np.asarray(tp, float)
        self.w_p = float(w_p)
        self.solvtol, self.maxit = float(solvtol), int(maxit)
        self.ckpt = int(ckpt_every or max(1, round(math.sqrt(self.nsteps))))
        self.m = capi.from_problem(pb)
        self.base_e = np.array(pb["e"], float).reshape(-1, capi.PM_PROP)
        self.idr = self.m.get_id()
        self.step_kw = dict(maxnlit=2, tol=1e-4, stop_crit=1, solver=1, precond=2,
                            solvtol=self.solvtol, maxit=self.maxit, reassemble=True)
        self.solves = 0

    # ---- parameters and state -------------------------------------------------
    def theta0(self):
        e = self.base_e
        return np.stack([np.log(e[:, 0]), np.log(e[:, 2]), np.log(e[:, 3])], 1)

    def materials(self, theta):
        th = np.asarray(theta, float).reshape(-1, 3)
        e = self.base_e.copy()
        e[:, 0] = np.exp(th[:, 0])
        e[:, 2] = np.exp(th[:, 1])
        e[:, 3] = np.exp(th[:, 2])
        return e

    def _reset(self, state=None, step=0):
        pb = self.pb
        if state is None:
            u0 = pb["u0"]
            self.m.set_state(u=u0, u0=u0, dp=np.zeros(self.m.nnode))
        else:
            self.m.set_state(u=state[0], u0=state[1], dp=state[2])
        self.m.set_env(pb["gravity"], float(pb["dt"]), step * float(pb["dt"]), step)

    def misfit(self, u):
        rz = u[self.ds, 2] - self.tz
        rp = u[self.ps, 3] - self.tp
        return float(np.sum(rz * rz) + self.w_p * np.sum(rp * rp))

    # ---- forward ----------------------------------------------------------------
    def forward(self, theta, keep_checkpoints=True):
        """J(theta); the checkpoints (every ckpt steps, step 0 included) are
        kept for the reverse sweep."""
        self.m.set_materials(self.materials(theta))
        self._reset()
        ck = {0: self.m.get_state()}
        for n in range(1, self.nsteps + 1):
            self.m.step(**self.step_kw)
            self.solves += 1
            if keep_checkpoints and n % self.ckpt == 0 and n < self.nsteps:
                ck[n] = self.m.get_state()
        u, _, _ = self.m.get_state()
        self.checkpoints = ck
        self.u_final = u
        return self.misfit(u)

    # ---- reverse ----------------------------------------------------------------
    def gradient(self):
        """dJ/dtheta (numel, 3) after forward(theta)."""
        dev = torch.device("cuda")
        neq, numel = self.m.neq, int(self.pb["numel"])
        f64 = dict(dtype=torch.float64, device=dev)
        mu = torch.zeros(neq, **f64)
        nu = torch.zeros(neq, **f64)
        grad = torch.zeros(3 * numel, **f64)
        lam = torch.zeros(neq, **f64)
        rhs = torch.zeros(neq, **f64)
        # mu_N = dJ/du_N on the free dofs
        g = np.zeros(neq)
        u = self.u_final
        for s, t in zip(self.ds, self.tz):
            e = self.idr[s, 2]
            if e > 0:
                g[e - 1] += 2.0 * (u[s, 2] - t)
        for s, t in zip(self.ps, self.tp):
            e = self.idr[s, 3]
            if e > 0:
                g[e - 1] += 2.0 * self.w_p * (u[s, 3] - t)
        mu.copy_(torch.from_numpy(g))
        starts = sorted(self.checkpoints)
        bounds = [(k0, (starts[i + 1] if i + 1 < len(starts) else self.nsteps))
                  for i, k0 in enumerate(starts)]
        for k0, k1 in reversed(bounds):
            # recompute the segment's states u_k0 .. u_k1 (nodal, on the device)
            self._reset(self.checkpoints[k0], k0)
            states = [torch.from_numpy(self.checkpoints[k0][0]).to(dev)]
            for n in range(k0 + 1, k1 + 1):
                self.m.step(**self.step_kw)
                self.solves += 1
                states.append(torch.from_numpy(self.m.get_state()[0]).to(dev))
            for n in range(k1, k0, -1):
                un = states[n - k0].contiguous()
                dun = (un - states[n - k0 - 1]).contiguous()
                torch.add(mu, nu, out=rhs)
                torch.cuda.synchronize()
                self.m.solve_dev(rhs.data_ptr(), lam.data_ptr(), solver=1, precond=2,
                                 tol=self.solvtol, maxit=self.maxit)
                self.solves += 1
                self.m.adjoint_grad_dev(lam.data_ptr(), un.data_ptr(), dun.data_ptr(),
                                        grad.data_ptr())
                self.m.adjoint_apply_dev(lam.data_ptr(), mu.data_ptr(), nu.data_ptr())
        torch.cuda.synchronize()
        return grad.view(numel, 3).cpu().numpy()


class BiotMisfit(torch.autograd.Function):
    """J = BiotMisfit.apply(theta, model): theta a (numel, 3) float64 tensor
    of (log E, log c_k, log M); the backward pass runs the adjoint sweep."""

    @staticmethod
    def forward(ctx, theta, model):
        J = model.forward(theta.detach().cpu().numpy())
        ctx.model = model
        return torch.tensor(J, dtype=torch.float64, device=theta.device)

    @staticmethod
    def backward(ctx, gJ):
        g = torch.from_numpy(ctx.model.gradient()).to(gJ.device)
        return gJ * g, None


def sensors_and_targets(pb, n_sensors=100, seed=5, scale_u=1e-3, scale_p=1e-2):
    """Seeded sensors: displacement sensors on the top-surface vertex nodes,
    pressure sensors on vertex nodes whose pressure is free; seeded normal
    target values (standard deviations scale_u m and scale_p MPa)."""
    rng = np.random.default_rng(seed)
    x, fnno, idf = pb["x"], pb["fnno"], pb["id"]
    ztop = x[:, 2].max()
    top = np.where((fnno == 1) & (np.abs(x[:, 2] - ztop) < 1e-9))[0]
    freep = np.where((fnno == 1) & (idf[:, 3] == 0))[0]
    ds = rng.choice(top, size=min(n_sensors, len(top)), replace=False)
    ps = rng.choice(freep, size=min(n_sensors, len(freep)), replace=False)
    tz = rng.standard_normal(len(ds)) * scale_u
    tp = rng.standard_normal(len(ps)) * scale_p
    return ds, tz, ps, tp
