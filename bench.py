"""Benchmark: implicit-Euler Biot steps/s of the heterogeneous hexa20 cube.

Workload (the configuration the headline metric is quoted on; it fits one
GPU): structured 56^3 hexa20 mesh of the unit cube, 731,025 nodes, 2,346,120 free equations
(2.38 M dofs before boundary conditions), log-permeability Gaussian random
field (mean ln 1e-14 m^2, sigma 1, correlation length 0.1 m), lognormal E
(median 1 GPa, sigma_ln 0.3), nu = 0.25, base fixed, drained top, top
traction ramped to 5 MPa over 10 steps of 100 s; seeded synthetic inputs.

One step = the reference's 'solv' macro (Main.f:876-1123): nodal loads,
isw 4 element loop, K re-assembled from the elements (isw 2, as the
reference does every step), residual, diagonal-PCG solve, residual check,
state update, with the reference's nonlinear settings (maxnlit 500,
tol 1e-4, Main.f:269-273; stop_crit 1) and a PCG tolerance of 1e-10, at
which the FP64 steps stay within 1e-8 of an FP64 solve to 1e-12 in u and p.
`value` is steps/s with the state resident in HBM; `e2e` is the same steps
through the C ABI with the nodal state copied from and back to pinned host
buffers every step.  `fp32_refine` is the same timed steps with the matrix
values held as FP32 + an int8 relative correction and the compensated FP32
SpMV inside the FP64 refinement loop (PM_FP32C_REFINE), with its error
against the FP64 steps and, over the first --acc-steps steps, against FP64
solves to 1e-12.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
  python bench.py --spmv-only [--n 32] [--reps 20] [--precision fp64|fp32c]
      (the SpMV alone on an assembled cube: the command the ncu summaries use)

N > 1 runs N independent replicas (one per GPU; a single mesh does not
shard without the halo exchange of the reference's MPI path); the batched
leg shards its instances over the ranks.  Without a torchrun environment,
--gpus N > 1 starts the N local ranks itself.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Biot steps/s at 2M dof: FP64 plain vs FP32+refine at 1e-8 rel; SpMV HBM GB/s"

# PCG iterations per step of the FP64 GPU steps of the 56^3 cube with the
# default step settings (PCG tol 1e-10, maxnlit 500, stop_crit 1), steps
# 1..25, as printed by this bench on a GB300 ('pcg_iterations_warmup_steps'
# then 'pcg_iterations_per_step' of `bench.py --steps 20 --warmup 5`).  The
# reference arm runs before any GPU step and times the CPU's cost of one PCG
# iteration; it multiplies that by these counts for the steps it stands for.
# The oracle takes the same iterations as the GPU within rounding (the
# step-history parity tests hold nlit equal and the mean counts within 3 %).
MEASURED_PCG_ITERS = {
    (56, 1e-10, 500): [3162, 3165, 3094, 3033, 3045, 3048, 3053, 3037, 3036, 3036, 3166, 3278,
                       3165, 3193, 3150, 3193, 3150, 3193, 3180, 3193, 3193, 3193, 3193, 3193,
                       3193],
}


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=56, help="elements per cube edge")
    ap.add_argument("--solvtol", type=float, default=1e-10)
    ap.add_argument("--maxnlit", type=int, default=500,
                    help="nonlinear iterations per step (the reference's default, Main.f:271)")
    ap.add_argument("--acc-steps", type=int, default=2,
                    help="steps over which the FP64 and mixed results are compared with "
                         "FP64 solves to 1e-12")
    ap.add_argument("--ref-iters", type=float, default=0.0,
                    help="reference arm: PCG iterations per step (default: the measured "
                         "GPU FP64 counts of the same steps)")
    ap.add_argument("--pcg-sample", type=int, default=20,
                    help="CPU timing: PCG iterations timed per sample step")
    ap.add_argument("--iters-only", action="store_true",
                    help="print the PCG iterations of steps 1..W+K of the FP64 cube only")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="one step of the same workload only (for the ncu launch list)")
    ap.add_argument("--profile-iters", type=int, default=0,
                    help="with --profile: then a solve of this many PCG iterations between "
                         "cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--workload", default="cube",
                    choices=["cube", "batched", "adjoint", "tetra"],
                    help="batched: only the batch of independent cubes; adjoint: the "
                         "gradient of a 50-step misfit on a 40^3 cube and its finite-"
                         "difference check; tetra: steps on the unstructured tetra10 box, "
                         "FP64 and compensated (its own line)")
    ap.add_argument("--tetra-mixed", action="store_true",
                    help="with --tetra-solver 11, also time rpsqmr on the compensated "
                         "operator: its refinement restarts cost far more iterations than "
                         "they save there")
    ap.add_argument("--tetra-n", type=int, default=48,
                    help="hex cells per edge of the tetra workload (6 tets each)")
    ap.add_argument("--tetra-solver", type=int, default=1, choices=[1, 11],
                    help="Krylov solver of the tetra workload: 1 pcg (with the compensated "
                         "operator and FP64 rpsqmr beside it), 11 rpsqmr")
    ap.add_argument("--fd-dirs", type=int, default=2,
                    help="finite-difference directions of the adjoint workload")
    ap.add_argument("--adj-n", type=int, default=40)
    ap.add_argument("--adj-steps", type=int, default=50)
    ap.add_argument("--batch-inst", type=int, default=96)
    ap.add_argument("--batch-steps", type=int, default=2,
                    help="timed steps of the batch leg in the default run")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-tetra", action="store_true",
                    help="leave out the unstructured tetra10 leg of the default run")
    ap.add_argument("--fp32-plain", action="store_true",
                    help="also time the plain FP32-value refinement (PM_FP32_REFINE)")
    ap.add_argument("--spmv-only", action="store_true",
                    help="time the SpMV alone on the assembled cube of --n")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32c"],
                    help="operator of --spmv-only and --profile")
    return ap.parse_args(argv)


T_START = time.perf_counter()


def log(msg):
    """Progress on stderr (rank 0): seconds since start and what just ended,
    so that a run cut short still shows where its time went."""
    if int(os.environ.get("RANK", "0")) == 0:
        print("[bench %7.1f s] %s" % (time.perf_counter() - T_START, msg), file=sys.stderr,
              flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def relaunch_ranks(args):
    """--gpus N > 1 outside torchrun: start N local ranks of this command
    (one per GPU, rendezvous on 127.0.0.1) and return their exit status."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", str(args.gpus), "--master-addr", "127.0.0.1",
           "--master-port", str(port), "--", os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def step_kwargs(args, solver=1):
    """The 'solv' macro settings of every timed step: the reference's
    nonlinear defaults (maxnlit 500, tol 1e-4; Main.f:269-273) with the
    stop test of the shipped decks (stop_crit 1), diagonal preconditioner,
    re-assembly of K every step."""
    return dict(maxnlit=args.maxnlit, tol=1e-4, stop_crit=1, solver=solver, precond=2,
                solvtol=args.solvtol, maxit=200000, reassemble=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def fp64_peak(torch):
    """GB300's FP64 pipe: 2 DFMA (4 flops) per SM per clock at the measured
    maximum SM clock; there is no measured FP64 peak to use instead."""
    mhz, src = 2070.0, "nominal max SM clock 2070 MHz"
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        if "sm_max_mhz" in d:
            mhz, src = float(d["sm_max_mhz"]), "MEASURED_PEAKS sm_max_mhz"
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return 4.0 * sms * mhz * 1e6 / 1e12, "2 DFMA per SM per clock x %d SMs x %s" % (sms, src)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def spmv_bytes(nad, neq, comp=False):
    """Algorithmic bytes of one CSRD SpMV: each stored lower value and its
    int32 column once, ad, x, y and the int32 row pointer once.  FP64:
    12 nad + 28 neq.  Compensated (values FP32 + int8 = 5 B, x as an FP32
    pair, y FP64): 9 nad + 25 neq."""
    return (9 * nad + 25 * neq) if comp else (12 * nad + 28 * neq)


def profile_traffic(nnz_panel, name="spmv_panel_fp64_cube.md"):
    """DRAM bytes per SpMV launch from the committed ncu summary (bytes per
    panel nonzero measured on a smaller cube, scaled to this launch)."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_panel_nnz:"):
            try:
                return float(line.split(":")[1]) * nnz_panel
            except ValueError:
                return None
    return None


# --------------------------------------------------------------------------
# CPU arm: the oracle (a restatement of the reference's Fortran with its
# OpenMP design: coloured element loop, row-partitioned CSRD SpMV) timed on a
# bounded sample of the same step, on all host cores.
# --------------------------------------------------------------------------
class CpuStep:
    """The work of one 'solv' step of the cube on the host cores, timed on the
    oracle's timing build (-O3, FMA contraction: a release build's speed) with
    the reference's OpenMP design on `threads` threads.  A step is one isw 4
    element pass (rhs), one isw 2 pass assembling K with b -= K du, one isw 2
    residual pass and the PCG solve; every pass covers all elements of the
    mesh.  PCG iterations are timed on the assembled matrix and the step's
    right-hand side; their cost does not depend on the iterate, so the solve
    costs the measured iteration count times the mean iteration time.

    The oracle is built once (its CSRD pattern set-up is not timed)."""

    def __init__(self, pb, threads=None, assemble=False):
        import oracle
        self.oracle = oracle
        self.threads = threads or os.cpu_count()
        t0 = time.perf_counter()
        o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]),
                          int(pb["nen"]), int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"],
                          pb["x"], pb["ie"], pb["e"], timing=True)
        o.set_loads(eload=pb["eload"], load=pb["load"], fload=pb["fload"])
        o.set_env(pb["gravity"], float(pb["dt"]))
        o.set_state(u=pb["u0"], u0=pb["u0"])
        self.o, self.u0 = o, pb["u0"]
        self.numel = int(pb["numel"])
        self.b = np.zeros(o.neq)
        self.du = np.zeros((int(pb["nnode"]), 4))
        if assemble:
            # K and the right-hand side before any timed sample, so that the
            # sampled PCG iterations run on the assembled system
            o.pform(4, False, True, self.u0, self.b, self.threads)
            o.pform(2, True, True, self.du, self.b, self.threads)
        self.setup_s = time.perf_counter() - t0
        self.t_pass = {"isw4": 0.0, "isw2_lhs": 0.0, "isw2_rhs": 0.0}
        self.elements = {"isw4": 0, "isw2_lhs": 0, "isw2_rhs": 0}
        self.t_pcg, self.n_pcg = 0.0, 0
        self.timed_s = 0.0

    def elements_pass(self, e0, e1, record=True):
        """Elements [e0, e1) (0-based) of the three element passes."""
        o, th = self.o, self.threads
        for key, isw, lhs, u in (("isw4", 4, 0, self.u0), ("isw2_lhs", 2, 1, self.du),
                                 ("isw2_rhs", 2, 0, self.du)):
            t0 = time.perf_counter()
            o.pform_range(isw, lhs, 1, u, self.b, th, e0 + 1, e1 + 1)
            dt = time.perf_counter() - t0
            if record:
                self.t_pass[key] += dt
                self.elements[key] += e1 - e0
                self.timed_s += dt

    def pcg(self, n, record=True):
        """n PCG iterations (pcg, Iters.f:299-595) on the handle's matrix."""
        t0 = time.perf_counter()
        try:
            self.o.solve(self.b, tol=1e-300, maxit=n, nthreads=self.threads)
        except self.oracle.OracleError:
            pass  # maxit reached: the sample's iterations are done
        dt = time.perf_counter() - t0
        if record:
            self.t_pcg += dt
            self.n_pcg += n
            self.timed_s += dt

    def step_seconds(self, iters):
        """Seconds of one step with `iters` PCG iterations: the element passes
        scaled from the elements timed (exactly 1 when every element of each
        pass was timed once) plus iters times the mean iteration time."""
        t_el = sum(self.t_pass[k] * self.numel / self.elements[k] for k in self.t_pass)
        return t_el + iters * self.t_pcg / self.n_pcg

    def parts(self, iters):
        d = {"t_" + k: round(self.t_pass[k] * self.numel / self.elements[k], 4)
             for k in self.t_pass}
        d["t_pcg_iter"] = round(self.t_pcg / self.n_pcg, 6)
        d["t_solve"] = round(iters * self.t_pcg / self.n_pcg, 3)
        return d


def cpu_baseline(pb, iters, pcg_sample):
    """The GPU arm's cpu_baseline: one full step's element passes (all
    elements, in the step's order, so the isw 2 pass assembles K) and
    pcg_sample PCG iterations on that matrix, with the solve scaled to the
    GPU FP64 steps' measured mean iteration count."""
    c = CpuStep(pb)
    c.elements_pass(0, c.numel)
    c.pcg(pcg_sample)
    t = c.step_seconds(iters)
    sample = ("one full step of element passes (isw 4, isw 2 lhs+rhs, isw 2 rhs over all %d "
              "elements) and %d PCG iterations on the assembled matrix; the solve is the mean "
              "iteration time x %.1f, the GPU FP64 steps' mean PCG iterations per step; "
              "%d threads; oracle built -O3 with FMA contraction (%.1f s timed, %.1f s set-up)"
              % (c.numel, pcg_sample, iters, c.threads, c.timed_s, c.setup_s))
    return {"value": 1.0 / t, "unit": "steps/s", "cores": c.threads, "kind": "port",
            "sample": sample, "parts_s": c.parts(iters)}


def reference_iters(args):
    """PCG iterations per step for the reference arm's steps warmup+1 ..
    warmup+steps: --ref-iters, else the measured GPU FP64 counts."""
    if args.ref_iters > 0:
        return float(args.ref_iters), "--ref-iters"
    key = (args.n, args.solvtol, args.maxnlit)
    if key not in MEASURED_PCG_ITERS:
        raise SystemExit("no measured PCG iteration count for the %d^3 cube at tol %g, maxnlit "
                         "%d: pass --ref-iters" % key)
    its = MEASURED_PCG_ITERS[key]
    lo = min(args.warmup, len(its) - 1)
    win = its[lo:lo + max(args.steps, 1)]
    return float(np.mean(win)), ("GPU FP64 steps %d..%d of this workload (measured)"
                                 % (lo + 1, lo + len(win)))


def run_reference(args):
    """The reference arm: the reference algorithm's CPU implementation (the
    oracle port) on all host cores, rank 0 only.  Each of the W + K steps times
    args.pcg_sample PCG iterations on the assembled matrix and one K-th slice
    of each of the three element passes, so the K timed steps time every
    element of every pass exactly once; the step time is those passes plus
    the solve at the measured PCG iterations per step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from poromec_gb300 import meshgen
    iters, iters_src = reference_iters(args)
    t_run = time.perf_counter()
    pb = meshgen.cube_problem(args.n)
    c = CpuStep(pb, assemble=True)
    K = max(args.steps, 1)
    bounds = [c.numel * j // K for j in range(K + 1)]
    for k in range(args.warmup):
        # warm-up: the same PCG sample and an element slice, untimed
        c.pcg(args.pcg_sample, record=False)
        c.elements_pass(bounds[k % K], bounds[k % K + 1], record=False)
    for j in range(K):
        c.elements_pass(bounds[j], bounds[j + 1])
        c.pcg(args.pcg_sample)
    t = c.step_seconds(iters)
    v = 1.0 / t
    sample = ("each of the %d timed steps: 1/%d of every element pass (isw 4, isw 2 lhs+rhs, "
              "isw 2 rhs; together each pass over all %d elements once) and %d PCG iterations "
              "on the assembled matrix; the step's solve = the mean iteration time x %.1f "
              "PCG iterations (%s); %d threads; oracle built -O3 with FMA contraction"
              % (K, K, c.numel, args.pcg_sample, iters, iters_src, c.threads))
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * t, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "heterogeneous cube, hexa20 %d^3, PCG tol %g, maxnlit %d, "
                                  "K re-assembled every step" % (args.n, args.solvtol,
                                                                  args.maxnlit),
                      "pcg_iterations_per_step": iters},
           "projected": {"timed_s": round(c.timed_s, 3), "setup_s": round(c.setup_s, 3),
                         "run_s": round(time.perf_counter() - t_run, 3),
                         "note": "ms_per_step is the full step projected from the timed "
                                 "samples: whole element passes plus the PCG iteration time x "
                                 "the iterations per step"},
           "parts_s": c.parts(iters),
           "cpu_baseline": {"value": v, "unit": "steps/s", "cores": c.threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def time_spmv(m, torch, reps):
    """Mean duration (ms) of pm_spmv_dev over reps launches, CUDA events on
    the launching stream, after 5 warm-up launches.  The panel values
    (>= 0.68 GB at n >= 32) exceed L2, so every launch streams them from HBM."""
    x = torch.randn(m.neq, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    s = torch.cuda.Stream()  # a real stream handle (0 would select the library's own)
    for _ in range(5):
        m.spmv_dev(x.data_ptr(), y.data_ptr(), s.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        m.spmv_dev(x.data_ptr(), y.data_ptr(), s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_spmv_only(args):
    import torch
    import poromec_gb300 as pg
    from poromec_gb300 import meshgen
    pb = meshgen.cube_problem(args.n)
    m = pg.from_problem(pb)
    m.pform(2, True, False, np.zeros((m.nnode, 4)), None)
    comp = args.precision == "fp32c"
    shape = None
    if comp:
        m.set_precision(pg.capi.PM_FP32C_REFINE)
        shape = m.tune_spmv()
    ms = time_spmv(m, torch, args.reps)
    B = spmv_bytes(m.nad, m.neq, comp)
    print(json.dumps({"spmv_only": True, "n": args.n, "precision": args.precision,
                      "shape": shape,
                      "neq": m.neq, "nad": m.nad, "nnz_panel": m.nnz_panel, "launch_ms": ms,
                      "algorithmic_bytes": B, "achieved_gbs": B / (ms * 1e-3) / 1e9}),
          flush=True)


def batched_leg(args, steps, warmup):
    """The batched workload: args.batch_inst independent unit cubes, hexa20
    n^3 with n uniform in 8..32, per-instance lognormal E and k, the loading
    of the consolidation column, all stepped by one handle (per-instance
    PCG, shared graph launches) with the compensated FP32 operator in the
    FP64 refinement; value = instance-steps per second."""
    import torch
    import poromec_gb300 as pg
    from poromec_gb300 import meshgen
    rank, world, _ = dist_env()
    t0 = time.perf_counter()
    allinst = meshgen.batch_instances(ninst=args.batch_inst, nmin=8, nmax=32, seed=4242)
    # N > 1: each rank steps its share of the instances (weak scaling, no
    # exchange in the solve); the time is the slowest rank's
    share = meshgen.partition_instances([p["n"] for p in allinst], world)[rank]
    inst = [allinst[i] for i in share]
    pb = meshgen.union_problem(inst)
    m = pg.from_problem(pb)
    m.set_precision(pg.capi.PM_FP32C_REFINE)
    t_setup = time.perf_counter() - t0
    kw = dict(step_kwargs(args), solvtol=float(pb["solvtol"]))
    log("batch set up: %d instances, %d equations (%.1f s)" % (len(inst), m.neq, t_setup))
    for _ in range(warmup):
        m.step(**kw)
        log("batch warm-up step: max PCG iterations %d" % m.batch_iters()[0].max())
    torch.cuda.synchronize()
    its = []
    t0 = time.perf_counter()
    for _ in range(steps):
        m.step(**kw)
        its.append(m.batch_iters()[0].copy())
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([el], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        el = float(t.item())
    it = np.array(its)
    ns = np.array([p["n"] for p in inst])
    out = {"value": len(allinst) * steps / el, "unit": "instance-steps/s",
           "ranks": world, "instances_this_rank": len(inst),
           "ms_per_step": el / steps * 1e3, "instances": len(allinst), "steps": steps,
           "warmup": warmup, "equations": int(m.neq), "nad": int(m.nad),
           "edge_min": int(ns.min()), "edge_max": int(ns.max()),
           "pcg_iterations_max": int(it.max()), "pcg_iterations_mean": float(it.mean()),
           "operator": "compensated FP32 (FP32 + int8 correction) in FP64 refinement",
           "solvtol": float(pb["solvtol"]), "setup_s": t_setup,
           "spmv_shape": m.tune_spmv()}
    m.close()
    return out


def run_batched(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    b = batched_leg(args, args.steps, args.warmup)
    if rank == 0:
        print(json.dumps(dict(metric="batched Biot steps", workload="batched cubes", **b)),
              flush=True)


def run_adjoint(args):
    """Adjoint workload: hexa20 cube of --adj-n^3 elements with per-element
    log E and log k from seeded Gaussian random fields (the heterogeneous
    cube's), --adj-steps steps of 100 s, misfit of the last step's vertical
    displacement at 100 seeded top-surface vertex nodes and pressure at 100
    seeded free-pressure vertex nodes against seeded targets; gradient with
    respect to (log E, log c_k, log M) of every element by the checkpointed
    adjoint sweep (checkpoints every round(sqrt(steps)) steps), FP64 solves
    to 1e-12; checked against central differences (h = 1e-6) along
    --fd-dirs seeded unit directions."""
    import torch
    from poromec_gb300 import adjoint, meshgen
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pb = meshgen.cube_problem(args.adj_n, seed=2024, steps=args.adj_steps)
    ds, tz, ps, tp = adjoint.sensors_and_targets(pb, n_sensors=100, seed=5)
    model = adjoint.TimeSteppedMisfit(pb, args.adj_steps, ds, tz, ps, tp, solvtol=1e-12)
    theta = model.theta0()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J = model.forward(theta)
    t1 = time.perf_counter()
    g = model.gradient()
    t2 = time.perf_counter()
    rng = np.random.default_rng(17)
    gn = float(np.linalg.norm(g))
    fd = []
    h = 1e-6
    # first the steepest direction g / |g| (directional derivative |g|),
    # then seeded random unit directions (derivative ~ |g| / sqrt(parameters),
    # close to the finite-difference noise of the forwards)
    for k in range(args.fd_dirs):
        d = g / gn if k == 0 else rng.standard_normal(theta.shape)
        d = d / np.linalg.norm(d)
        f = (model.forward(theta + h * d, False) - model.forward(theta - h * d, False)) / (2 * h)
        a = float(np.sum(g * d))
        fd.append({"direction": "gradient" if k == 0 else "random", "fd": f, "adjoint": a,
                   "abs_err_over_grad_norm": abs(f - a) / gn,
                   "rel_err": abs(f - a) / max(abs(f), 1e-300)})
    if rank != 0:
        return
    print(json.dumps({
        "metric": "adjoint gradient of a time-stepped Biot misfit", "workload":
        "hexa20 %d^3 cube, %d steps, per-element log E, log k, log M" % (args.adj_n,
                                                                        args.adj_steps),
        "value": (t2 - t0), "unit": "s per gradient (forward + reverse)",
        "higher_is_better": False, "forward_s": t1 - t0, "reverse_s": t2 - t1,
        "parameters": int(3 * pb["numel"]), "equations": int(model.m.neq), "J": J,
        "grad_norm": gn, "checkpoint_every": model.ckpt, "solves": model.solves,
        "fd_step": h, "fd_checks": fd, "data": "synthetic (seeded fields and targets)"}),
        flush=True)


def tetra_leg(args, steps, warmup):
    """Unstructured tetra10 workload: --tetra-n^3 hex cells on a 2 x 2 x 1 m box
    split in 6 Kuhn tets, interior vertices jittered, two layers, a point
    source, dt 60 s, at the cube's PCG tolerance and nonlinear settings.
    Solver (--tetra-solver): pcg (solver 1, default) with the diagonal
    preconditioner, or rpsqmr (solver 11, the reference's default solver).
    Diagonally preconditioned MINRES as the reference implements it (the
    Lanczos alpha taken in absolute value) needs 2e4 iterations per step at
    4^3 and 4e5 at 8^3 on this indefinite system (the oracle shows the same),
    so pcg stands in for it; on this machine pcg takes ~25 % fewer iterations
    than rpsqmr and reaches the same state (the oracle shows that too).  FP64
    steps after warm-up, timed on the device with inputs resident; then the
    same steps from the same state with the compensated operator in FP64
    refinement (PM_FP32C_REFINE: pcg with residual replacement; for rpsqmr
    only with --tetra-mixed, whose refinement restarts its Krylov space and
    at this tolerance costs more iterations than the cheaper product saves);
    with pcg, also FP64 rpsqmr from the same state for comparison."""
    import torch
    import poromec_gb300 as pg
    from poromec_gb300 import meshgen
    pb = meshgen.tetra_problem(args.tetra_n)
    m = pg.from_problem(pb)
    dt = float(pb["dt"])
    kw = step_kwargs(args, solver=args.tetra_solver)
    sname = {1: "pcg", 11: "rpsqmr"}[args.tetra_solver]
    log("tetra set up: %d equations" % m.neq)
    for _ in range(warmup):
        m.step(**kw)
        log("tetra warm-up step: %d iterations" % int(m.timers()[4]))
    snap = m.get_state()

    def restore():
        m.set_state(*snap)
        m.set_env(pb["gravity"], dt, warmup * dt, warmup)

    def timed(skw, what):
        its = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            m.step(**skw)
            its.append(int(m.timers()[4]))
            log("tetra %s step: %d iterations" % (what, its[-1]))
        torch.cuda.synchronize()
        return time.perf_counter() - t0, its

    mixed = qmr = None
    with ClockSampler(0) as clk:
        restore()
        t64, its64 = timed(kw, sname)
        u64, _, _ = m.get_state()
        if args.tetra_solver == 1:
            restore()
            tq, itsq = timed(step_kwargs(args, solver=11), "rpsqmr")
            qmr = {"value": steps / tq, "unit": "steps/s", "ms_per_step": tq / steps * 1e3,
                   "iterations_per_step": itsq}
        if args.tetra_mixed or args.tetra_solver == 1:
            restore()
            m.set_precision(pg.capi.PM_FP32C_REFINE)
            m.step(**kw)  # one-off set-up of the mode (copies, record layout, autotuner)
            restore()
            tc, itsc = timed(kw, sname + " compensated")
            uc, _, _ = m.get_state()
            du = float(np.abs(uc[:, :3] - u64[:, :3]).max() / np.abs(u64[:, :3]).max())
            dp_ = float(np.abs(uc[:, 3] - u64[:, 3]).max() / np.abs(u64[:, 3]).max())
            mixed = {"value": steps / tc, "unit": "steps/s", "speedup_vs_fp64": t64 / tc,
                     "shape": m.tune_spmv(), "iterations_per_step": itsc,
                     "rel_err_vs_fp64_same_tol": {"u": du, "p": dp_}}
    neq, nad = m.neq, m.nad
    m.close()
    out = {"value": steps / t64, "unit": "steps/s", "steps": steps, "warmup": warmup,
           "ms_per_step": t64 / steps * 1e3,
           "workload": "tetra10 Kuhn %d^3 on 2x2x1 m, %d equations, nad %d, %s tol %g, "
                       "K re-assembled every step" % (args.tetra_n, neq, nad, sname,
                                                      kw["solvtol"]),
           "iterations_per_step": its64, "clocks": clk.summary()}
    if mixed:
        out["fp32_refine"] = mixed
    if qmr:
        out["rpsqmr_fp64"] = qmr
    return out


def run_tetra(args):
    t = tetra_leg(args, args.steps, args.warmup)
    out = {"metric": "Biot steps/s, unstructured tetra10 %s: FP64 plain vs FP32+refine"
                     % {1: "pcg", 11: "rpsqmr"}[args.tetra_solver],
           "value": t["value"], "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t["ms_per_step"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded jitter, two layers, point source)",
           "config": {"workload": t["workload"],
                      "iterations_per_step": t["iterations_per_step"]},
           "fp32_refine": t.get("fp32_refine"), "rpsqmr_fp64": t.get("rpsqmr_fp64"),
           "clocks": t["clocks"]}
    print(json.dumps(out), flush=True)


def column_leg(args, steps=20):
    """The reference's CPU-runnable case: the 2 x 2 x 40
    hexa20 consolidation column (4,032 equations before restraints), 1 MPa
    top load from t = 0, 20 implicit Euler steps of 10 s, diagonal PCG to
    1e-10, maxnlit 500, stop_crit 1.  The GPU runs the 20 steps once untimed
    (graph capture and the other one-off set-up), then again from the initial
    state, timed; the CPU oracle (timing build) runs the same 20 steps in full,
    timed, on 1 thread and on all host threads (the faster is reported: on a
    mesh this small the threads cost more than they save).  No projection:
    both sides do the whole run.  The final states are compared."""
    import torch
    import oracle
    import poromec_gb300 as pg
    from poromec_gb300 import meshgen
    pb = meshgen.column_problem()
    kw = dict(step_kwargs(args), solvtol=1e-10)
    m = pg.from_problem(pb)
    for _ in range(steps):
        m.step(**kw)
    m.set_state(u=pb["u0"], u0=pb["u0"], dp=np.zeros(int(pb["nnode"])))
    m.set_env(pb["gravity"], float(pb["dt"]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    its = 0
    for _ in range(steps):
        m.step(**kw)
        its += int(m.timers()[4])
    torch.cuda.synchronize()
    t_gpu = time.perf_counter() - t0
    ug, _, _ = m.get_state()
    m.close()
    best = None
    for th in sorted({1, os.cpu_count()}):
        o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), int(pb["nen"]),
                          int(pb["nenv"]), pb["ix"], pb["id"], pb["fnno"], pb["x"], pb["ie"],
                          pb["e"], timing=True)
        o.set_loads(eload=pb["eload"], load=pb["load"], fload=pb["fload"])
        o.set_env(pb["gravity"], float(pb["dt"]))
        o.set_state(u=pb["u0"], u0=pb["u0"])
        okw = {k: v for k, v in kw.items() if k != "reassemble"}
        t0 = time.perf_counter()
        for _ in range(steps):
            o.step(nthreads=th, **okw)
        t = time.perf_counter() - t0
        uo, _, _ = o.get_state()
        if best is None or t < best[0]:
            best = (t, th, uo)
    t_cpu, th, uo = best
    du = float(np.abs(ug[:, :3] - uo[:, :3]).max() / np.abs(uo[:, :3]).max())
    dp_ = float(np.abs(ug[:, 3] - uo[:, 3]).max() / np.abs(uo[:, 3]).max())
    return {"value": steps / t_gpu, "unit": "steps/s", "steps": steps,
            "workload": "consolidation column, hexa20 2x2x40, %d steps of 10 s, PCG tol 1e-10"
                        % steps,
            "pcg_iterations_per_step": its / steps,
            "cpu_oracle": {"value": steps / t_cpu, "unit": "steps/s", "threads": th,
                           "kind": "port, full run (no projection)"},
            "rel_diff_vs_cpu_oracle": {"u": du, "p": dp_}}


def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import poromec_gb300 as pg
    from poromec_gb300 import meshgen

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    pb = meshgen.cube_problem(args.n)
    m = pg.from_problem(pb)
    log("cube %d^3 set up: %d equations" % (args.n, m.neq))
    step_kw = step_kwargs(args)
    if args.profile:
        if args.precision == "fp32c":
            m.set_precision(pg.capi.PM_FP32C_REFINE)
        info = m.step(**step_kw)
        torch.cuda.synchronize()
        out = {"profile_step": True, "pcg_iterations": int(m.timers()[4]),
               "nlit": info.nlit, "kernels": int(m.timers()[7])}
        if args.profile_iters:
            # a solve of exactly --profile-iters iterations on the step's matrix
            # (tolerance 0, ended by maxit) between cudaProfilerStart/Stop: the
            # in-loop kernels alone for `ncu --profile-from-start off`
            b = np.random.default_rng(1).standard_normal(m.neq)
            torch.cuda.profiler.start()
            try:
                m.solve(b, solver=1, precond=2, tol=0.0, maxit=args.profile_iters)
            except pg.PMError:
                pass
            torch.cuda.synchronize()
            torch.cuda.profiler.stop()
            out["profiled_iterations"] = args.profile_iters
        print(json.dumps(out), flush=True)
        return
    warm_iters = []
    for _ in range(args.warmup):
        info = m.step(**step_kw)
        warm_iters.append(int(m.timers()[4]))
        log("warm-up step %d: %d PCG iterations, nlit %d" % (len(warm_iters), warm_iters[-1],
                                                             info.nlit))
    if args.iters_only:
        # the PCG iterations of every step 1..W+K (the reference arm's table)
        for _ in range(args.steps):
            m.step(**step_kw)
            warm_iters.append(int(m.timers()[4]))
        if rank == 0:
            print(json.dumps({"iters_only": True, "n": args.n, "solvtol": args.solvtol,
                              "maxnlit": args.maxnlit, "pcg_iterations": warm_iters}),
                  flush=True)
        return
    snap = m.get_state()
    t_snap = args.warmup * float(pb["dt"])

    def restore():
        # state and clock of the first timed step (the top load ramps in time)
        m.set_state(*snap)
        m.set_env(pb["gravity"], float(pb["dt"]), t_snap, args.warmup)
    barrier()
    iters, nlits = [], []
    timers = []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            info = m.step(**step_kw)
            timers.append(m.timers())
            iters.append(int(timers[-1][4]))
            nlits.append(info.nlit)
            log("timed step %d: %d PCG iterations, nlit %d" % (len(iters), iters[-1], info.nlit))
        barrier()
        elapsed = time.perf_counter() - t0
    log("timed FP64 steps: %.2f s/step" % (elapsed / args.steps))
    u64, _, _ = m.get_state()
    ms = elapsed / args.steps * 1e3
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * args.steps / elapsed

    # e2e: the same step through the C ABI with the nodal state in pinned host
    # memory, copied in before and out after every step.
    u_h, u0_h, dp_h = [torch.from_numpy(a.copy()).pin_memory().numpy() for a in snap]
    restore()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m.set_state(u_h, u0_h, dp_h)
        m.step(**step_kw)
        u_o, u0_o, dp_o = m.get_state()
        u_h[...], u0_h[...], dp_h[...] = u_o, u0_o, dp_o
    barrier()
    e2e_elapsed = time.perf_counter() - t0
    nbytes = u_h.nbytes + u0_h.nbytes + dp_h.nbytes
    log("e2e steps: %.2f s/step" % (e2e_elapsed / args.steps))

    # Accuracy references (untimed): the first acc steps from the same state
    # in FP64 with PCG at 1e-12 and at the bench's tolerance.
    acc = max(1, min(args.acc_steps, args.steps))
    restore()
    for _ in range(acc):
        m.step(**dict(step_kw, solvtol=1e-12))
    u_ref, _, _ = m.get_state()
    restore()
    for _ in range(acc):
        m.step(**step_kw)
    u64_acc, _, _ = m.get_state()
    log("accuracy references (%d steps at 1e-12 and at the bench tolerance)" % acc)

    def rel_err(a, ref):
        eu = float(np.abs(a[:, :3] - ref[:, :3]).max() / np.abs(ref[:, :3]).max())
        ep = float(np.abs(a[:, 3] - ref[:, 3]).max() / np.abs(ref[:, 3]).max())
        return {"u": eu, "p": ep}

    budget = 2 * max(max(iters), 1)

    def mixed_leg(mode, refine=None):
        """The timed steps again from the same state in another precision
        mode, bounded to twice the FP64 iteration count per solve so that a
        stalled refinement is reported instead of waited for."""
        restore()
        m.set_precision(mode)
        if refine:
            m.set_refine(refine)
        mi = []
        try:
            # the first acc steps untimed from the same state: the one-off
            # set-up of the mode (compensated copies, record layout, SpMV
            # autotuner, graph capture) stays out of the timed steps, as the
            # FP64 set-up does, and their result is compared with the FP64
            # solves to 1e-12
            for _ in range(acc):
                m.step(**dict(step_kw, maxit=budget))
            um_acc, _, _ = m.get_state()
            restore()
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                info = m.step(**dict(step_kw, maxit=budget))
                mi.append((int(m.timers()[4]), info.refine, info.nlit))
                log("mode %d timed step %d: %d PCG iterations, %d replacements, nlit %d"
                    % (mode, len(mi), mi[-1][0], info.refine, info.nlit))
            barrier()
            t_mixed = time.perf_counter() - t0
            um, _, _ = m.get_state()
            out = {"value": world * args.steps / t_mixed, "unit": "steps/s",
                   "speedup_vs_fp64": elapsed / t_mixed,
                   "rel_err_vs_fp64_same_tol": rel_err(um, u64),
                   "rel_err_vs_fp64_1e-12": dict(rel_err(um_acc, u_ref), steps=acc),
                   "pcg_iterations_per_step": [a for a, _, _ in mi],
                   "residual_replacements_per_step": [b for _, b, _ in mi],
                   "nlit_per_step": [c for _, _, c in mi]}
        except pg.PMError as ex:
            torch.cuda.synchronize()
            out = {"value": None, "unit": "steps/s", "status": "no convergence",
                   "detail": str(ex), "steps_completed": len(mi),
                   "iteration_budget_per_solve": budget}
        return out

    mixed = plain32 = None
    if not args.no_mixed:
        mixed = mixed_leg(pg.capi.PM_FP32C_REFINE)
        log("compensated steps: %s steps/s" % mixed.get("value"))
        # the compensated SpMV alone (x split into its FP32 pair included)
        cms = time_spmv(m, torch, 50)
        cB = spmv_bytes(m.nad, m.neq, comp=True)
        ctr = profile_traffic(m.nnz_panel, "spmv_panel_fp32c_cube.md")
        mixed["spmv"] = {"kernel": "k_spmv_cf<0> + k_split_pair", "launch_ms": cms,
                         "shape": m.tune_spmv(),
                         "algorithmic_bytes": cB, "achieved_gbs": cB / (cms * 1e-3) / 1e9,
                         "traffic": ctr}
        mixed["values"] = ("FP32 + int8 relative correction (5 B, 2^-32), compensated FP32 "
                           "products and sums, FP64 vectors and dots")
    if args.fp32_plain:
        plain32 = mixed_leg(pg.capi.PM_FP32_REFINE, 1e-5)
    m.set_precision(pg.capi.PM_FP64)
    fp64_err = dict(rel_err(u64_acc, u_ref), steps=acc)

    # SpMV roofline: the dominant kernel timed alone with CUDA events on the
    # stream it is launched on, 50 launches over the assembled matrix
    spmv_ms = time_spmv(m, torch, 50)
    B = spmv_bytes(m.nad, m.neq)
    achieved = B / (spmv_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    f64_peak, f64_src = fp64_peak(torch)
    f64_achieved = 2.0 * m.nnz_panel / (spmv_ms * 1e-3) / 1e12
    traffic = profile_traffic(m.nnz_panel)
    tm = np.mean(np.array(timers), 0)
    neq, nad, nnz_panel = m.neq, m.nad, m.nnz_panel
    # the legs below run on every rank: the batch shards its instances (with
    # a MAX all-reduce of the time), the tetra box runs as a replica
    batched = tetra = column = None
    if not args.no_batch:
        m.close()  # the batch needs the memory more than the finished cube
        batched = batched_leg(args, args.batch_steps, 1)
        log("batched leg: %.2f instance-steps/s" % batched["value"])
    if not args.no_tetra:
        tetra = tetra_leg(args, 2, 1)
        log("tetra leg: %.3f steps/s" % tetra["value"])
    if rank == 0 and not args.no_cpu:
        column = column_leg(args)
        log("column leg: %.1f steps/s, CPU oracle %.1f" % (column["value"],
                                                            column["cpu_oracle"]["value"]))
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    out = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian random fields, structured mesh)",
        "config": {"workload": "heterogeneous cube, hexa20 %d^3, %d equations, nad %d, "
                               "PCG tol %g, maxnlit %d, stop_crit 1, K re-assembled every "
                               "step" % (args.n, neq, nad, args.solvtol, args.maxnlit),
                   "l2": "inputs larger than L2 (panel values %.2f GB)" % (nnz_panel * 8e-9),
                   "pcg_iterations_per_step": iters,
                   "nlit_per_step": nlits,
                   "pcg_iterations_warmup_steps": warm_iters,
                   "phase_ms": {"pload_isw4": tm[0], "assembly_isw2": tm[1],
                                "residual_isw2": tm[2], "solve": tm[3]},
                   "replicas": world},
        "e2e": {"value": world * args.steps / e2e_elapsed, "unit": "steps/s",
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
        "spmv_gbs": achieved,
        "fp64_rel_err_vs_1e-12": fp64_err,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS hbm_gbs)",
                     "kernel": "k_spmv<double> (node panels)", "launch_ms": spmv_ms,
                     "algorithmic_bytes": B, "traffic": traffic,
                     # the kernel's actual bound: one DFMA per stored panel value
                     "fp64_pipe": {"achieved_tflops": f64_achieved, "peak_tflops": f64_peak,
                                   "frac": f64_achieved / f64_peak, "peak_source": f64_src,
                                   "flops": 2.0 * nnz_panel}},
        "gpu_launches": int(round(args.steps * tm[7])),
        "clocks": clk.summary(),
    }
    if mixed:
        out["fp32_refine"] = mixed
    if plain32:
        out["fp32_plain_refine"] = plain32
    if batched:
        out["batched"] = batched
    if tetra:
        out["tetra"] = tetra
    if column:
        out["column"] = column
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(pb, float(np.mean(iters)), args.pcg_sample)
        log("cpu baseline: %.5f steps/s" % out["cpu_baseline"]["value"])
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_ranks(args))
    if args.spmv_only:
        run_spmv_only(args)
    elif args.workload == "batched" and args.impl != "reference":
        run_batched(args)
    elif args.workload == "adjoint" and args.impl != "reference":
        run_adjoint(args)
    elif args.workload == "tetra" and args.impl != "reference":
        run_tetra(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
