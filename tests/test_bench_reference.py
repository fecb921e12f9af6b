"""bench.py's reference arm on the CPU, at a small T: one JSON line with the contract's keys,
the reference's own SPGQPSolver template (oracle/_ref) as the timed implementation where it is
built (the FP64 oracle port otherwise), no host<->device bytes, and the same config dict as the
GPU arm prints for the same arguments."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    sys.path.insert(0, ROOT)
    import bench
    from oracle import pasc_oracle as O
    T = 100_000
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--T", str(T), "--steps", "3",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 3
    assert d["config"] == bench.bench_config(T, 3, 10.0)
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1
    assert cb["kind"] == ("reference" if O.ref_available() else "port")
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    tts = d["time_to_1e-6_rel_obj"]
    assert tts["seconds"] > 0 and tts["spg_it"] >= 1
    if cb["kind"] == "reference":
        assert tts["objective_equals_port_trace"] is True


def test_reference_arm_under_two_ranks():
    """Under torchrun with two ranks rank 0 alone prints the line, both exit 0, and the CPU
    baseline runs on every core of the process's affinity although torchrun sets
    OMP_NUM_THREADS=1 for its workers."""
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29531", "bench.py", "--impl", "reference",
                        "--gpus", "2", "--T", "100000", "--steps", "2", "--warmup", "3"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["impl"] == "reference"
    assert d["cpu_baseline"]["cores"] == len(os.sched_getaffinity(0))


def test_gpu_arm_cpu_baseline_object():
    """The cpu_baseline object the GPU arm adds to its line, built on the CPU at a small T."""
    sys.path.insert(0, ROOT)
    import bench
    from oracle import pasc_oracle as O
    from pasc_inference_gb300 import datagen
    import numpy as np
    T = 50_000
    sig = datagen.signal1d_cfg1(T=T)
    cb = bench.measure_cpu_baseline(sig, np.array([0.0, 1.0, 2.0]), 10.0, T)
    json.dumps(cb)
    assert cb["kind"] == ("reference" if O.ref_available() else "port")
    assert cb["value"] > 0 and cb["cores"] == bench.cpu_cores()
    assert cb["port_all_cores"]["value"] > 0 and cb["one_thread"]["cores"] == 1
    if O.ref_available():
        assert cb["reference_one_thread"]["objective_equals_port"] is True
        assert cb["time_to_1e-6_rel_obj"]["objective_equals_port_trace"] is True
