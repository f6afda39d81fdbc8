"""bench.py --impl reference: the CPU implementation of the path (the oracle
port, on the host's cores) prints one JSON line with the keys and meaning of
the GPU arm's line, its own e2e (no host-device copies) and cpu_baseline.
CPU only, on a 12^3 cube with a given PCG iteration count per step."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "2", "--warmup", "1", "--n", "12", "--ref-iters", "700"],
                       capture_output=True, text=True,
                       cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert k in d, k
    assert d["unit"] == "steps/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] == 1
    assert "workload" in d["config"] and "12^3" in d["config"]["workload"]
    assert d["config"]["pcg_iterations_per_step"] == 700
    # the projection is stated: each element pass was timed over all elements
    # once, and the samples took less than the run
    pr = d["projected"]
    assert 0 < pr["timed_s"] <= pr["run_s"]
    parts = d["parts_s"]
    assert abs(d["ms_per_step"] * 1e-3 - (parts["t_isw4"] + parts["t_isw2_lhs"]
                                          + parts["t_isw2_rhs"] + parts["t_solve"])) < 1e-2
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] >= 1 and cb["sample"]


def test_reference_arm_needs_a_measured_iteration_count():
    """Without --ref-iters and without a measured count for the workload the
    arm refuses to guess."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--n", "7"], capture_output=True,
                       text=True, cwd=ROOT, timeout=600)
    assert r.returncode != 0
    assert "--ref-iters" in r.stderr


def test_gpus_n_starts_its_own_ranks():
    """`bench.py --gpus 2` outside torchrun starts two local ranks itself
    (torch.distributed.run on 127.0.0.1); under them the reference arm runs
    on rank 0 only and reports n_gpus 2.  CPU only."""
    env = {k: v for k, v in os.environ.items()
           if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0", "--n", "6",
                        "--ref-iters", "50"], capture_output=True, text=True, cwd=ROOT,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
