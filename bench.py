#!/usr/bin/env python
"""SPG iterations/s of the FEM-H1 gamma-step QP on the T = 1e7, K = 3 benchmark signal.

One step = one SPG-QP iteration (SPGQPSolver main loop, src/petscvector/solver/spgqpsolver.cpp:
140-297) over the whole signal: the fused mixed-precision sweep on the GPU.  The workload is
the synthetic 1-D signal of the benchmark configuration (T = 1e7 timesteps, K = 3 levels
{0, 1, 2} in random order per segment, segment lengths U[1e3, 1e5], noise sigma 0.5;
seeded, see pasc_inference_gb300/datagen.py), epssqr = 10, theta fixed at the true levels
as in the reference's own SPG benchmark runs (tssolver_maxit = 1 with theta given), GLL
memory 10.  Every timed step runs the full iteration; stopping tests are off inside the
timed region so that no step is skipped.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Besides the headline line it measures, on rank 0:
  tts        for every epssqr of the sweep {1, 10, 100, 1000}: time to an objective within 1e-6
             relative of the FP64 optimum, for the mixed path and for the plain FP64 GPU path
             on the same problem; the FP64 end point certified by its Frank-Wolfe gap under the
             oracle's operator, and the mixed end point's objective and gamma errors against it.
  e2e        the same metric through the public API with host buffers in page-locked memory
             (pasc_gb300_host_alloc): set_data, set_gamma, permute, set_theta, update_b,
             spgqp_solve (the reference's default stop, |f - f_old| < 1e-9, m 10), get_gamma,
             get_fx; host<->device copies inside the timed region.  FP32 host buffers (the
             mixed path's device format) for the line's value, FP64 host buffers beside it.
  roofline   the sweep kernel's algorithmic bytes (8*K*T + 4*T per iteration: gamma read and
             written in FP32, the data read once) over its CUDA-event time, against the
             measured HBM copy bandwidth.
  cpu_baseline  the reference's own SPGQPSolver template compiled from its headers with a
             host-array backend (oracle/_ref; OpenMP over the vector operations, its sums in the
             oracle's chunk order) on all host cores, and its time to 1e-6 relative objective;
             beside it the FP64 oracle port on all cores (`port_all_cores`) and on one
             (`one_thread`), and the template on one thread (`reference_one_thread`) with a check
             that its objective equals the port's bit for bit.  Where oracle/_ref cannot be built
             the port takes the template's place (kind "port").
  batched    the 256-signal uneven workload (T log-uniform in [1e3, 1e6], K in 2..5, epssqr
             log-uniform in [1, 1000]): every signal's TSSolver (SPG eps 1e-6, m 10; outer loop
             to 1e-6 relative change of L) solved by one batch handle (one CUDA graph launch
             whose conditional nodes loop on the device) and, for comparison, one signal at a
             time with the plain FP64 GPU path and with the single-signal mixed path; the
             batch sweep's HBM throughput with all 256 signals running; and the gamma-step QP
             of every signal at fixed theta by the batch and by the plain FP64 path under the
             same stop rule, objectives compared signal by signal and with the best objective
             any run reached (--no-batched-qp skips it).
  adjoint    derivatives through the converged gamma step at T = 1e6, K = 3 (the benchmark
             signal generator, clean copy kept): dloss/d epssqr of the reconstruction MSE from
             the adjoint, checked against central differences (1e-4 relative) through FP64 GPU
             solves and against the FP64 oracle's gradient (timed: the CPU baseline), then 20
             gradient steps on log epssqr.
  multichannel  T = 1e6 timesteps of n = 128 channels, K = 8 (Markov labels, centroids N(0, I),
             noise 0.8; X in BF16): the TSSolver wall time, and per kernel its device time and
             bytes: the residual on the tensor cores and on the CUDA cores, the theta update,
             the SPG sweep reading the materialised b; the oracle's residual and theta update
             on the host cores for comparison.
"""
from __future__ import annotations

import argparse
import functools
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

METRIC = "SPG iters/s & time to 1e-6 rel obj, T=1e7 K=3 (1 GB300); HBM GB/s vs peak"
UNIT = "SPG iterations/s"
WORKLOAD = "signal1d T=1e7 K=3 levels {0,1,2} sigma=0.5, epssqr=10, theta fixed, GLL m=10"


# ------------------------------------------------------------------------------------------
# replicas: one process per GPU under torchrun.  The SPG path does not shard ("replicas
# only"): ranks exchange nothing on the data path; these helpers only synchronise the timed
# region (barrier) and combine timings (max over ranks) on the host over gloo, so no GPU
# collective is issued.  torch.distributed is used here only, never by the library.
# ------------------------------------------------------------------------------------------
class RankInfo:
    def __init__(self, rank=0, world_size=1, local_rank=0):
        self.rank, self.world_size, self.local_rank = rank, world_size, local_rank
        self.initialised = False


def dist_init(timeout_s: float = 600.0) -> RankInfo:
    """Joins the process group when launched with WORLD_SIZE > 1 (gloo over 127.0.0.1)."""
    info = RankInfo(int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
                    int(os.environ.get("LOCAL_RANK", "0")))
    if info.world_size > 1:
        import datetime

        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29531")
        if not dist.is_initialized():
            dist.init_process_group("gloo", rank=info.rank, world_size=info.world_size,
                                    timeout=datetime.timedelta(seconds=timeout_s))
        info.initialised = True
    return info


def dist_barrier(info: RankInfo) -> None:
    if info.world_size > 1:
        import torch.distributed as dist
        dist.barrier()


def _allreduce(info: RankInfo, value: float, op: str) -> float:
    if info.world_size <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op))
    return float(t.item())


def max_over_ranks(info: RankInfo, value: float) -> float:
    return _allreduce(info, value, "MAX")


def sum_over_ranks(info: RankInfo, value: float) -> float:
    return _allreduce(info, value, "SUM")


def dist_finalize(info: RankInfo) -> None:
    if info.world_size > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--T", type=int, default=10_000_000)
    ap.add_argument("--eps2", type=float, default=10.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tts", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-multichannel", action="store_true")
    ap.add_argument("--no-image", action="store_true")
    ap.add_argument("--no-batched-qp", action="store_true",
                    help="skip the batched gamma-step QP at fixed theta (the plain FP64 path one signal at a "
                         "time takes about two minutes of it)")
    ap.add_argument("--variant", type=int, default=-1, choices=[-1, 0, 1],
                    help="sweep kernel: -1 chosen by timing (default), 0 one timestep per thread, "
                         "1 bulk-copy tiles (pin it when profiling: a profiler distorts the timing)")
    return ap.parse_args()


def bench_config(T, K, eps2):
    """The workload description both arms print (identical dicts for the same arguments)."""
    return {"workload": WORKLOAD, "T": int(T), "K": int(K), "epssqr": float(eps2), "parallelism": "replicas",
            "l2": "inputs larger than L2"}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per sweep launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "spg_sweep_tma_k3_t1e7.md")
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].split()[0])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu), "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_cores():
    """Host cores this process may run on (its CPU affinity): the thread count of every timed
    CPU baseline."""
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


@functools.lru_cache(maxsize=None)
def ref_available() -> bool:
    """Whether the reference's own solver templates are compiled (oracle/_ref: from the reference
    tree, or from the translation unit its recipe left where the tree is absent); built once per
    process."""
    from oracle import pasc_oracle as O
    try:
        return O.build_ref() is not None
    except Exception:
        return False


def cpu_iter_rate(kind, sig, theta, eps2, T, iters, nthreads):
    """SPG iterations/s on the first T timesteps of the signal (every iteration runs) of
    kind "reference", the reference's own SPGQPSolver template compiled from its headers with
    the host-array backend (oracle/_ref), or "port", the FP64 oracle, on nthreads OpenMP
    threads (an explicit count: it overrides OMP_NUM_THREADS, which torchrun sets to 1).
    The solve's set-up (first projection and product) is timed apart and taken off.  Returns
    (iterations/s, seconds, objective after the iterations)."""
    from oracle import pasc_oracle as O
    O.build()
    K = sig.K
    data = sig.data[:T]
    gam = O.permute_blocked_to_interleaved(sig.gamma0[: K * T] if T == sig.T else
                                           sig.gamma0.reshape(K, sig.T)[:, :T].ravel(), T, K)
    b = O.residual_b(data, theta, T, K, nthreads=nthreads)
    coeff = O.A_coeff(eps2, T)

    def solve(maxit):
        if kind == "reference":
            _, it, _, fx = O.ref_spgqp_solve(b, gam, T, K, coeff, nthreads=nthreads, spgqpsolver_maxit=maxit,
                                             spgqpsolver_m=10, spgqpsolver_stop_difff=0)
            return it, fx
        _, r, _ = O.spgqp_solve(b, gam, T, K, coeff, O.spg_opts(maxit=maxit, m=10, stop_difff=0),
                                nthreads=nthreads)
        return r.it, r.fx

    t0 = time.perf_counter()
    solve(0)
    t_init = time.perf_counter() - t0
    t0 = time.perf_counter()
    it, fx = solve(iters)
    dt = max(time.perf_counter() - t0 - t_init, 1e-9)
    return it / dt, dt, fx


def reference_one_thread(sig, theta, eps2, T, iters):
    """The reference's own template on one thread (every sum in index order, as a one-rank
    PETSc host vector sums), with whether its objective equals the port's on one thread bit for
    bit; None where oracle/_ref could not be built."""
    if not ref_available():
        return None
    rate, dt, fx = cpu_iter_rate("reference", sig, theta, eps2, T, iters, 1)
    _, _, fx_port = cpu_iter_rate("port", sig, theta, eps2, T, iters, 1)
    return {"value": rate, "unit": UNIT, "cores": 1, "kind": "reference",
            "sample": f"{iters} SPG iterations of the reference's SPGQPSolver template (oracle/_ref, "
                      f"host-array vectors) on the full T={T} signal ({dt:.1f} s)",
            "objective_equals_port": bool(fx == fx_port)}


def measure_cpu_baseline(sig, theta, eps2, T):
    """The GPU arm's cpu_baseline object: the reference's template on all host cores (the port
    where oracle/_ref is not built), the port on all cores and on one, the template on one, and
    the time to 1e-6 relative objective."""
    kind = "reference" if ref_available() else "port"
    cores = cpu_cores()
    rate, dt, _ = cpu_iter_rate(kind, sig, theta, eps2, T, 5, cores)
    prate, pdt, _ = cpu_iter_rate("port", sig, theta, eps2, T, 5, cores)
    rate1, dt1, _ = cpu_iter_rate("port", sig, theta, eps2, T, 2, 1)
    what = "the reference's SPGQPSolver template (oracle/_ref)" if kind == "reference" else "the FP64 oracle"
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"5 SPG iterations of {what} on the full T={T} signal ({dt:.1f} s, OpenMP)",
            "port_all_cores": {"value": prate, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": f"5 SPG iterations ({pdt:.1f} s)"},
            "one_thread": {"value": rate1, "unit": UNIT, "cores": 1, "kind": "port",
                           "sample": f"2 SPG iterations, same signal ({dt1:.1f} s)"},
            "reference_one_thread": reference_one_thread(sig, theta, eps2, T, 2),
            "time_to_1e-6_rel_obj": cpu_tts(kind, sig, theta, eps2, T)}


def run_reference(args, info):
    """The reference path's CPU implementation on all host cores, rank 0 only: the reference's
    own SPGQPSolver template (oracle/_ref) where it compiled, else the FP64 oracle port."""
    from pasc_inference_gb300 import datagen
    if info.rank != 0:
        return None
    sig = datagen.signal1d_cfg1(T=args.T)
    theta = np.array([0.0, 1.0, 2.0])
    cores = cpu_cores()
    kind = "reference" if ref_available() else "port"
    what = ("the reference's SPGQPSolver template (oracle/_ref, host-array vectors, OpenMP)" if kind == "reference"
            else "the FP64 oracle port (OpenMP)")
    # size the per-step sample so that warmup + steps stay within ~2 minutes
    rate_full, _, _ = cpu_iter_rate(kind, sig, theta, args.eps2, args.T, 1, cores)
    t_full = 1.0 / rate_full
    budget = 120.0 / max(1, args.steps + args.warmup)
    Ts = int(min(args.T, max(100_000, args.T * budget / t_full)))
    steps = args.steps
    if Ts < args.T:
        rate, dt, _ = cpu_iter_rate(kind, sig, theta, args.eps2, Ts, steps, cores)
        value = rate * Ts / args.T
        sample = f"{steps} SPG iterations of {what} on the first {Ts} timesteps, scaled by {Ts}/{args.T}"
    else:
        rate, dt, _ = cpu_iter_rate(kind, sig, theta, args.eps2, args.T, steps, cores)
        value = rate
        sample = f"{steps} SPG iterations of {what} on the full signal"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": bench_config(args.T, 3, args.eps2),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
        "time_to_1e-6_rel_obj": cpu_tts(kind, sig, theta, args.eps2, args.T),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def main():
    args = parse()
    info = dist_init()
    if args.impl == "reference":
        line = run_reference(args, info)
        if line is not None:
            print(json.dumps(line), flush=True)
        dist_finalize(info)
        return

    from pasc_inference_gb300 import PASC_PREC_FP64, PASC_PREC_MIXED, Problem, capi, datagen
    dev = info.local_rank
    sig = datagen.signal1d_cfg1(T=args.T)
    T, K = sig.T, sig.K
    theta = np.array([0.0, 1.0, 2.0])
    B_it = 8.0 * K * T + 4.0 * T  # read x, data; write x (FP32): the sweep's algorithmic bytes

    p = Problem(T, K, args.eps2, precision=PASC_PREC_MIXED, device=dev)
    if args.variant >= 0:
        p.set_sweep_variant(args.variant)
    p.set_data(sig.data)
    p.set_gamma(sig.gamma0)
    p.permute_gamma()
    p.set_theta(theta)
    p.update_b()
    total_steps = args.warmup + args.steps
    opts = capi.spgqp_opts(maxit=10 * total_steps + 100, m=10, stop_difff=0)
    p.spgqp_start(opts)
    variant = p.get_sweep_variant()
    if args.warmup:
        p.spgqp_iterate(args.warmup, poll=False)

    dist_barrier(info)
    sampler = ClockSampler(dev) if info.rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    chunk = 500
    done, ms_total, launches, restarts = 0, 0.0, 0, 0
    t_wall0 = time.perf_counter()
    while done < args.steps:
        n = min(chunk, args.steps - done)
        st = p.spgqp_iterate(n, poll=False)
        ms, nl = p.spgqp_last_iterate()
        if st.status != capi.PASC_SPG_RUNNING:
            # the solve ended inside the chunk (exact stationarity): the chunk is re-run from a
            # fresh start so that every timed step is a full iteration
            restarts += 1
            p.spgqp_start(opts)
            continue
        ms_total += ms
        launches += nl
        done += n
    t_wall = time.perf_counter() - t_wall0
    clocks = sampler.stop() if sampler else None
    dist_barrier(info)
    ms_max = max_over_ranks(info, ms_total)
    value = info.world_size * args.steps / (ms_max / 1000.0)
    ms_per_step = ms_max / args.steps

    peak, peak_kind = measured_peaks()
    achieved = B_it / (ms_per_step / 1000.0) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": profile_traffic(),
                "peak_source": peak_kind,
                "bytes_per_launch": B_it,
                "kernel": "spg_sweep_tma_kernel<3,128,false>" if variant == 1 else "spg_sweep_kernel<3,false>"}

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": info.world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": bench_config(T, K, args.eps2),
        "run": {"wall_s_timed": t_wall, "restarts": restarts,
                "bytes_per_step": "x 120 MB + data 40 MB read, x 120 MB written",
                "sweep_kernel": {0: "one timestep per thread", 1: "bulk-copy tiles, 4 timesteps per thread"}[variant]},
        "gpu_launches": launches,
        "roofline": roofline,
        "clocks": clocks,
    }
    p.close()

    fstar = None
    if info.rank == 0 and not args.no_tts:
        result["time_to_1e-6_rel_obj"] = measure_tts(sig, theta, dev)
        fstar = result["time_to_1e-6_rel_obj"].get(f"epssqr={args.eps2:g}", {}).get("f_star_fp64")
    if info.rank == 0 and not args.no_e2e:
        result["e2e"] = measure_e2e(sig, theta, args.eps2, dev, fstar)
    if info.rank == 0 and not args.no_batched:
        result["batched"] = measure_batched(dev, peak, qp=not args.no_batched_qp)
    if info.rank == 0 and not args.no_multichannel:
        result["multichannel"] = measure_multichannel(dev, peak)
    if info.rank == 0 and not args.no_adjoint:
        result["adjoint"] = measure_adjoint(dev, peak)
    if info.rank == 0 and not args.no_image:
        result["image"] = measure_image(dev, peak)
    if info.rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = measure_cpu_baseline(sig, theta, args.eps2, T)
    if info.rank == 0:
        print(json.dumps(result), flush=True)
    dist_finalize(info)


def measure_e2e(sig, theta, eps2, dev, fstar, steps=6):
    """The public API end to end with host buffers in page-locked memory from the library's
    allocator (pasc_gb300_host_alloc); the copies are inside the timed region.  Each step:
    set_data, set_gamma, permute, set_theta, update_b, spgqp_solve with the reference's default
    stop rule (|f - f_old| < 1e-9, GLL m 10; it ends within 1e-6 relative of the FP64 optimum
    here, checked below), get_gamma, get_fx.  Two forms: FP32 host buffers (the mixed path's
    device format) and FP64 host buffers (the reference's vector type)."""
    from pasc_inference_gb300 import PASC_PREC_MIXED, Problem, capi
    T, K = sig.T, sig.K
    opts = capi.spgqp_opts(m=10, eps=1e-9)
    out = {}
    for form, dt in (("f32_host", np.float32), ("f64_host", np.float64)):
        hb = [capi.host_empty(n, dt) for n in (T, T * K, T * K)]
        data_h, gamma_h, out_h = (h.array for h in hb)
        data_h[:] = sig.data
        gamma_h[:] = sig.gamma0
        with Problem(T, K, eps2, precision=PASC_PREC_MIXED, device=dev) as p:
            its, secs, launches, fx = 0, 0.0, 0, None
            for rep in range(steps + 1):
                t0 = time.perf_counter()
                if dt == np.float32:
                    p.set_data_f32(data_h)
                    p.set_gamma_f32(gamma_h)
                else:
                    p.set_data(data_h)
                    p.set_gamma(gamma_h)
                p.permute_gamma()
                p.set_theta(theta)
                p.update_b()
                st = p.spgqp_solve(opts)
                if dt == np.float32:
                    p.get_gamma_f32_into(out_h)
                else:
                    p.get_gamma_into(out_h)
                fx = p.get_fx()
                dt_s = time.perf_counter() - t0
                if rep > 0:
                    its += st.it
                    secs += dt_s
                    launches += st.kernel_launches
        w = np.dtype(dt).itemsize
        out[form] = {"value": its / secs, "unit": UNIT, "h2d_bytes_per_step": w * T + w * T * K + 8 * K,
                     "d2h_bytes_per_step": w * T * K + 8, "host_buffers": "page-locked (pasc_gb300_host_alloc)",
                     "spg_it_per_step": its / steps, "s_per_step": secs / steps, "fx": fx,
                     "fx_rel_err_vs_fp64_optimum": abs(fx - fstar) / abs(fstar) if fstar else None,
                     "stop": "|f - f_old| < 1e-9 (reference default)", "gpu_launches_per_step": launches / steps}
        for h in hb:
            h.close()
    res = dict(out["f32_host"])
    err = res["fx_rel_err_vs_fp64_optimum"]
    res["time_to_1e-6_rel_obj_s"] = res["s_per_step"] if (err is not None and err <= 1e-6) else None
    res["f64_host"] = out["f64_host"]
    return res


def _fw_gap_rel(x, data, theta, T, K, eps2):
    """Frank-Wolfe gap of x relative to |f(x)|, from the FP64 oracle's operator and residual:
    an upper bound on (f(x) - f*) / |f(x)| for the QP over the simplex product."""
    from oracle import pasc_oracle as orc
    b = orc.residual_b(data, theta, T, K, nthreads=0)
    g = orc.matmult(x, T, K, orc.A_coeff(eps2, T), nthreads=0) - b
    f = 0.5 * (x @ (g + b)) - b @ x
    G, X = g.reshape(T, K), x.reshape(T, K)
    return float(np.sum(np.sum(X * G, axis=1) - G.min(axis=1))) / abs(f)


TTS_PLAN = {1.0: (400, 4000), 10.0: (1600, 4000), 100.0: (2600, 6000), 1000.0: (16000, 25000)}


def measure_tts(sig, theta, dev, eps_list=(1.0, 10.0, 100.0, 1000.0)):
    """Time to an objective within 1e-6 (relative) of the FP64 optimum, for every epssqr of
    the benchmark sweep: the plain FP64 GPU path (the reference's structure) and the mixed
    path from the same gamma0, both run without a stopping test (fixed iteration budgets
    that reach the optimum: TTS_PLAN) and traced every few iterations.  The FP64 end point,
    polished (pasc_gb300_polish), is the optimum, certified by its Frank-Wolfe gap under the
    oracle's FP64 operator; the mixed path's end point is compared with it (objective and
    gamma), before and after its own polish."""
    from pasc_inference_gb300 import PASC_PREC_FP64, PASC_PREC_MIXED, Problem, capi
    T, K = sig.T, sig.K
    out = {}
    for eps2 in eps_list:
        it64, itmx = TTS_PLAN.get(eps2, (4000, 8000))
        traces = {}
        for name, prec, maxit, chunk in (("fp64_plain", PASC_PREC_FP64, it64, 50),
                                         ("mixed_fused", PASC_PREC_MIXED, itmx, 25)):
            with Problem(T, K, eps2, precision=prec, device=dev) as p:
                p.set_data(sig.data)
                p.set_gamma(sig.gamma0)
                p.permute_gamma()
                p.set_theta(theta)
                p.update_b()
                o = capi.spgqp_opts(m=10, maxit=maxit, stop_difff=0)
                t0 = time.perf_counter()
                p.spgqp_start(o)
                tr = []
                while True:
                    st = p.spgqp_iterate(chunk, poll=True)
                    tr.append((time.perf_counter() - t0, st.it, st.fx))
                    if st.status != capi.PASC_SPG_RUNNING:
                        break
                x_end = p.get_gamma()
                t0 = time.perf_counter()
                ps = p.polish()
                t_pol = time.perf_counter() - t0
                traces[name] = (tr, st, x_end, p.get_gamma(), ps, t_pol)
        tr64, st64, x64_end, x64, ps64, _ = traces["fp64_plain"]
        fstar = ps64.fx
        res = {"f_star_fp64": fstar, "fp64_optimum_fw_gap_rel": _fw_gap_rel(x64, sig.data, theta, T, K, eps2),
               "fp64_end_gamma_rel_to_polished": float(np.linalg.norm(x64_end - x64) / np.linalg.norm(x64))}
        for name, (tr, st, x, _, _, _) in traces.items():
            hit = next(((t, it) for t, it, f in tr if abs(f - fstar) <= 1e-6 * abs(fstar)), None)
            res[name] = {"seconds": hit[0] if hit else None, "spg_it": hit[1] if hit else None,
                         "final_rel_err": abs(st.fx - fstar) / abs(fstar), "final_it": st.it,
                         "status": capi.STATUS_NAMES.get(st.status, st.status)}
        _, _, xm, xmp, psm, t_pol = traces["mixed_fused"]
        res["mixed_fused"]["gamma_rel_err_vs_fp64_optimum"] = float(np.linalg.norm(xm - x64) / np.linalg.norm(x64))
        res["mixed_fused"]["labels_equal_frac"] = float(np.mean(np.argmax(xm.reshape(T, K), 1) ==
                                                               np.argmax(x64.reshape(T, K), 1)))
        res["mixed_fused"]["polished"] = {
            "gamma_rel_err_vs_fp64_optimum": float(np.linalg.norm(xmp - x64) / np.linalg.norm(x64)),
            "f_rel_err": abs(psm.fx - fstar) / abs(fstar), "rounds": psm.rounds, "cg_it": psm.cg_it,
            "seconds": t_pol, "device_s": psm.time_s}
        a, b = res["fp64_plain"]["seconds"], res["mixed_fused"]["seconds"]
        res["speedup_vs_fp64_plain"] = (a / b) if (a and b) else None
        out[f"epssqr={eps2:g}"] = res
    return out


def oracle_tts(sig, theta, eps2, T, nthreads=None, maxit=600):
    """The FP64 oracle on the host cores (all of them unless nthreads says otherwise): time to an objective within 1e-6 (relative) of its
    own objective at |f - f_old| < 1e-12 (the reference's SPG loop, traced)."""
    from oracle import pasc_oracle as O
    O.build()
    if nthreads is None:
        nthreads = cpu_cores()
    K = sig.K
    b = O.residual_b(sig.data, theta, T, K, nthreads=nthreads)
    x0 = O.permute_blocked_to_interleaved(sig.gamma0, T, K)
    t0 = time.perf_counter()
    _, r, tr = O.spgqp_solve(b, x0, T, K, O.A_coeff(eps2, T), O.spg_opts(m=10, maxit=maxit, eps=1e-12),
                             trace=True, nthreads=nthreads)
    secs = time.perf_counter() - t0
    f = tr[:, 0]
    fend = f[-1]
    hit = int(np.argmax(np.abs(f - fend) <= 1e-6 * abs(fend)))
    return {"seconds": secs * hit / max(r.it, 1), "spg_it": hit, "f_ref": float(fend), "run_it": int(r.it),
            "run_s": secs, "cores": nthreads, "kind": "port",
            "f_hit": float(f[hit]), "f_ref_rule": "objective of the same run at |f - f_old| < 1e-12"}


def cpu_tts(kind, sig, theta, eps2, T):
    """Time to 1e-6 relative objective on all host cores.  The port's traced run finds the
    iteration that reaches it; for kind "reference" the reference's own template (whose iterates
    equal the port's at the same thread count: its sums follow the same chunks) is then timed
    for exactly that many iterations, and its objective there is checked against the trace."""
    res = oracle_tts(sig, theta, eps2, T)
    if kind != "reference" or res["spg_it"] < 1:
        return res
    from oracle import pasc_oracle as O
    K = sig.K
    b = O.residual_b(sig.data, theta, T, K, nthreads=0)
    x0 = O.permute_blocked_to_interleaved(sig.gamma0, T, K)
    t0 = time.perf_counter()
    _, it, _, fx = O.ref_spgqp_solve(b, x0, T, K, O.A_coeff(eps2, T), nthreads=cpu_cores(), spgqpsolver_maxit=res["spg_it"],
                                     spgqpsolver_m=10, spgqpsolver_stop_difff=0)
    secs = time.perf_counter() - t0
    return {"seconds": secs, "spg_it": int(it), "f_ref": res["f_ref"], "cores": cpu_cores(), "kind": "reference",
            "objective_equals_port_trace": bool(fx == res["f_hit"]), "port": res,
            "f_ref_rule": res["f_ref_rule"]}


def measure_multichannel(dev, peak):
    from pasc_inference_gb300 import PASC_PREC_MIXED, Problem, capi, datagen
    sys.path.insert(0, ROOT)
    from oracle import pasc_oracle as orc
    t0 = time.perf_counter()
    mc = datagen.multichannel()
    t_gen = time.perf_counter() - t0
    T, n, K = mc.T, mc.n, mc.K
    res = {"workload": "multichannel T=1e6 n=128 K=8, Markov labels (stay 0.999), centroids N(0,I), noise 0.8, "
                       "epssqr=50, X in BF16", "T": T, "n": n, "K": K, "datagen_s": t_gen}
    with Problem(T, K, mc.epssqr, precision=PASC_PREC_MIXED, xdim=n, device=dev) as p:
        p.set_data(mc.data)
        p.set_gamma(mc.gamma0)
        p.set_theta(np.zeros(K * n))
        t0 = time.perf_counter()
        st = p.ts_solve(capi.ts_opts(), capi.spgqp_opts(m=10))
        res["tssolver"] = {"wall_s": time.perf_counter() - t0, "L": st.L, "outer_it": st.it_last,
                           "spg_it": st.spg_it_sum, "gpu_launches": st.kernel_launches,
                           "settings": "reference defaults (SPG eps 1e-9, outer |dL| < 1e-6), m 10"}
        kernels = {}
        B_res = 2.0 * T * n + 4.0 * T + 4.0 * T * K  # X (BF16), ||X_t||^2, b written
        for eng, name in ((0, "residual_tcgen05"), (1, "residual_cuda_cores")):
            p.set_residual_engine(eng)
            p.time_model_kernels(2, 3)
            ms = p.time_model_kernels(2, 20)
            kernels[name] = {"us": ms * 1e3, "bytes": B_res, "achieved": B_res / (ms * 1e-3) / 1e9, "unit": "GB/s",
                             "frac": B_res / (ms * 1e-3) / 1e9 / peak,
                             "tflops_useful": 2.0 * T * n * K / (ms * 1e-3) / 1e12}
        p.set_residual_engine(0)
        B_th = 2.0 * T * n + 4.0 * T * K
        p.time_model_kernels(1, 3)
        ms = p.time_model_kernels(1, 20)
        kernels["theta_update"] = {"us": ms * 1e3, "bytes": B_th, "achieved": B_th / (ms * 1e-3) / 1e9, "unit": "GB/s",
                                   "frac": B_th / (ms * 1e-3) / 1e9 / peak}
        p.update_b()
        chosen = p.get_sweep_variant()
        res["tssolver"]["sweep_kernel_chosen"] = chosen
        B_sw = 12.0 * K * T  # x read, b read, x written (FP32)
        for v, name in ((0, "spg_sweep_bmat_thread_per_timestep"), (1, "spg_sweep_bmat_bulk_copy")):
            p.set_sweep_variant(v)
            p.spgqp_start(capi.spgqp_opts(m=10, maxit=100000, stop_difff=0))
            p.spgqp_iterate(20, poll=False)
            p.spgqp_iterate(200, poll=False)
            ms, nl = p.spgqp_last_iterate()
            kernels[name] = {"us": ms / nl * 1e3, "bytes": B_sw, "achieved": B_sw / (ms / nl * 1e-3) / 1e9,
                             "unit": "GB/s", "frac": B_sw / (ms / nl * 1e-3) / 1e9 / peak}
        p.set_sweep_variant(chosen)
        res["kernels"] = kernels
        th = p.get_theta()
        g = p.get_gamma()
    res["peak"] = peak
    # host FP64 oracle: residual (all cores) and theta update (one core)
    t0 = time.perf_counter()
    orc.residual_b(mc.data, th, T, K, xdim=n, nthreads=cpu_cores())
    t_res = time.perf_counter() - t0
    t0 = time.perf_counter()
    orc.theta_update(g, mc.data, T, K, xdim=n)
    t_th = time.perf_counter() - t0
    res["cpu_oracle"] = {"residual_s": t_res, "residual_cores": cpu_cores(), "theta_update_s": t_th,
                         "theta_update_cores": 1}
    return res


def _image_data(w, h, seed=7, sigma=0.4):
    """Background 0, a disc 1, a bar 2, Gaussian noise (a test_image-style input)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    lab = (((xx - w / 3) ** 2 + (yy - h / 2) ** 2) < (min(w, h) / 4) ** 2).astype(np.int8)
    lab[(xx > 0.65 * w) & (xx < 0.9 * w) & (yy > 0.2 * h) & (yy < 0.8 * h)] = 2
    return lab.ravel().astype(np.float64) + sigma * rng.standard_normal(w * h)


def measure_image(dev, peak):
    """Image mode (T = 1, 4-neighbour grid graph): the mixed graph SPG iteration (two kernels)
    on a 4096x4096 image with K = 3, the TSSolver on a 1024x1024 image, and the FP64 oracle's SPG
    iteration on the large image."""
    from pasc_inference_gb300 import PASC_PREC_MIXED, BGMGraphGrid2D, Problem, capi, datagen
    sys.path.insert(0, ROOT)
    from oracle import pasc_oracle as orc
    K, eps2 = 3, 2.0
    w = h = 4096
    R = w * h
    data = _image_data(w, h)
    g = BGMGraphGrid2D(w, h)
    g.process_grid()
    theta = np.array([0.0, 1.0, 2.0])
    B_fused = (8.0 * K + 4.0) * R   # read x, data; write x (FP32): the fused image sweep
    B_graph = (20.0 * K + 4.0) * R  # read x, d, data; write x, d; read d: the general graph sweep
    res = {"workload": f"image {w}x{h} (T=1, 4-neighbour grid graph), K={K}, epssqr={eps2}, disc and bar on 0, "
                       "noise 0.4", "R": R, "K": K}
    for v, name, B_it, kern in ((1, "spg_iteration", B_fused, "image_sweep_kernel<3,false>"),
                                (0, "spg_iteration_general_graph_sweep", B_graph,
                                 "graph_sweep_a_kernel<3,false> + graph_sweep_b_kernel<3,false>")):
        with Problem(1, K, eps2, precision=PASC_PREC_MIXED, device=dev, graph=g) as p:
            p.set_sweep_variant(v)
            p.set_data(data)
            p.set_gamma(datagen.uniform(13, 0, R * K))
            p.set_theta(theta)
            p.update_b()
            p.spgqp_start(capi.spgqp_opts(m=10, maxit=100000, stop_difff=0))
            p.spgqp_iterate(20, poll=False)
            p.spgqp_iterate(300, poll=False)
            ms, nl = p.spgqp_last_iterate()
            it_ms = ms / 300
            ach = B_it / (it_ms * 1e-3) / 1e9
            res[name] = {"it_per_s": 1e3 / it_ms, "us_per_it": it_ms * 1e3, "gpu_launches_per_it": nl / 300,
                         "bytes_per_iteration": B_it, "achieved": ach, "unit": "GB/s", "frac": ach / peak,
                         "kernels": kern}
            if v == 1:
                x = p.get_gamma()
    # the FP64 oracle's SPG iteration on the same image (all cores)
    b = orc.residual_b(data, theta, R, K, bscale=orc.b_coeff(1))
    t0 = time.perf_counter()
    orc.spgqp_solve_graph(b, x, 1, K, orc.A_coeff(eps2, 1), g.ptr, g.idx, orc.spg_opts(maxit=3, eps=0.0, m=10))
    dt = time.perf_counter() - t0
    res["cpu_oracle"] = {"it_per_s": 3 / dt, "sample": "3 SPG iterations of the FP64 oracle (one core)",
                         "cores": 1}
    # TSSolver on a 1024x1024 image with the reference's default stopping rules
    w2 = 1024
    d2 = _image_data(w2, w2, seed=8)
    g2 = BGMGraphGrid2D(w2, w2)
    g2.process_grid()
    with Problem(1, K, eps2, precision=PASC_PREC_MIXED, device=dev, graph=g2) as p:
        p.set_data(d2)
        p.set_gamma(datagen.uniform(13, 0, w2 * w2 * K))
        p.set_theta(np.zeros(K))
        t0 = time.perf_counter()
        st = p.ts_solve(capi.ts_opts(), capi.spgqp_opts(m=10))
        res["tssolver_1024"] = {"wall_s": time.perf_counter() - t0, "L": st.L, "outer_it": st.it_last,
                                "spg_it": st.spg_it_sum, "theta": p.get_theta().tolist()}
    res["peak"] = peak
    return res


def measure_adjoint(dev, peak, eps0=300.0):
    from pasc_inference_gb300 import PASC_PREC_FP64, PASC_PREC_MIXED, Problem, capi, datagen, learn
    sys.path.insert(0, ROOT)
    from oracle import pasc_oracle as orc
    sig = datagen.signal1d_cfg1(T=1_000_000)
    T, K = sig.T, sig.K
    theta = np.array([0.0, 1.0, 2.0])
    # the gradient is taken at the fixed point of each solve: the mixed path runs 20000
    # iterations with no stopping test (its FP32 fixed point), the FP64 path to ||d||^2 < 1e-26
    spg_mixed = capi.spgqp_opts(m=10, maxit=20000, stop_difff=0)
    spg64 = capi.spgqp_opts(m=10, eps=1e-26, maxit=40000, stop_difff=0, stop_normgp=1)

    def loaded(prec, eps2, gamma=None):
        p = Problem(T, K, eps2, precision=prec, device=dev)
        p.set_data(sig.data)
        p.set_theta(theta)
        if gamma is None:
            p.set_gamma(sig.gamma0)
            p.permute_gamma()
        else:
            p.set_gamma(gamma)
        p.update_b()
        return p

    res = {"workload": "signal1d T=1e6 K=3 levels {0,1,2} sigma=0.5 (clean copy kept), theta fixed at the "
                       "levels, loss = MSE(sum_k gamma_k theta_k, clean)", "T": T, "K": K, "epssqr0": eps0}
    # gradient on the mixed path (timed) and its CG throughput
    with loaded(PASC_PREC_MIXED, eps0) as p:
        t0 = time.perf_counter()
        st = p.spgqp_solve(spg_mixed)
        t1 = time.perf_counter()
        pol = p.polish()
        t1p = time.perf_counter()
        loss = p.recon_mse(sig.clean)
        deps, dX, dth, a = p.adjoint()
        t2 = time.perf_counter()
    N = T * K
    # per FP32 CG iteration of the mixed path's refinement: apply (r, p read; p, q written; mask)
    # 16N + 4T, update (d, p, r, q read; d, r written) 24N.  The time per iteration is the whole
    # adjoint's device time over the iterations (setup, FP64 residuals and output included).
    B_cg = 40.0 * N + 4.0 * T
    cg_s = a.time_s / max(a.cg_it, 1)
    res.update({"loss": loss, "dloss_depssqr": deps, "solve_s": t1 - t0, "spg_it": st.it,
                "polish": {"s": t1p - t1, "device_s": pol.time_s, "rounds": pol.rounds, "cg_it": pol.cg_it,
                           "step_rel": pol.step_rel, "face_changes": pol.face_changes},
                "adjoint_s": t2 - t1p, "adjoint_device_s": a.time_s, "cg_it": a.cg_it,
                "free_dims": a.free_dims,
                "cg_iteration": {"us": cg_s * 1e6, "bytes": B_cg, "achieved": B_cg / cg_s / 1e9, "unit": "GB/s",
                                 "peak": peak, "frac": B_cg / cg_s / 1e9 / peak}})
    # FP64 GPU: gradient and central differences
    with loaded(PASC_PREC_FP64, eps0) as p:
        p.spgqp_solve(spg64)
        p.polish()
        x0 = p.get_gamma()
        p.recon_mse(sig.clean)
        deps64, _, _, _ = p.adjoint()
        h = 1e-4
        lo = []
        for e in (eps0 * (1 + h), eps0 * (1 - h)):
            p.set_epssqr(e)
            p.set_gamma(x0)
            p.update_b()
            p.spgqp_solve(spg64)
            p.polish()
            lo.append(p.recon_mse(sig.clean))
    fd = (lo[0] - lo[1]) / (2 * h * eps0)
    # FP64 oracle on the host: solve (the reference's stop rule, |f - f_old| < 1e-12) + adjoint,
    # timed as the CPU baseline of the gradient
    t0 = time.perf_counter()
    b = orc.residual_b(sig.data, theta, T, K, nthreads=cpu_cores())
    xo, _, _ = orc.spgqp_solve(b, orc.permute_blocked_to_interleaved(sig.gamma0, T, K), T, K,
                               orc.A_coeff(eps0, T), orc.spg_opts(m=10, eps=1e-12, maxit=20000),
                               nthreads=cpu_cores())
    _, dgo, _ = orc.recon_mse(xo, theta, sig.clean, T, K)
    orc.adjoint(xo, sig.data, theta, dgo, T, K, eps0)
    t_cpu = time.perf_counter() - t0
    # the oracle's adjoint at the FP64 optimum (the FP64 GPU solve above, ||d||^2 < 1e-26, polished)
    _, dgo, _ = orc.recon_mse(x0, theta, sig.clean, T, K)
    deps_o = orc.adjoint(x0, sig.data, theta, dgo, T, K, eps0, cg_tol=1e-12)[0]
    res["checks"] = {"fd_central_h1e-4_fp64": fd, "adjoint_fp64": deps64, "oracle_fp64_at_fixed_point": deps_o,
                     "rel_mixed_vs_fd": abs(deps - fd) / abs(fd), "rel_fp64_vs_fd": abs(deps64 - fd) / abs(fd),
                     "rel_mixed_vs_oracle": abs(deps - deps_o) / abs(deps_o),
                     "mixed_solve": "20000 SPG iterations, no stopping test (FP32 fixed point), then "
                                    "pasc_gb300_polish (FP64 face-Newton rounds to the optimum)"}
    res["cpu_baseline_gradient_s"] = t_cpu
    res["cpu_baseline_cores"] = cpu_cores()
    # 20 gradient steps on log epssqr
    with loaded(PASC_PREC_MIXED, eps0) as p:
        t0 = time.perf_counter()
        rec = learn.descend_log_epssqr(p, sig.clean, steps=20, spg=spg_mixed)
        t_gd = time.perf_counter() - t0
    res["descent"] = {"steps": 20, "wall_s": t_gd, "loss_first": rec[0]["loss"], "loss_last": rec[-1]["loss"],
                      "epssqr_last": rec[-1]["epssqr"],
                      "epssqr": [r["epssqr"] for r in rec], "loss": [r["loss"] for r in rec]}
    return res


def measure_batched(dev, peak, qp=True):
    """The 256-signal uneven workload through one batch handle: the sweep's HBM throughput with
    every signal running, the TSSolver of every signal (device-driven loop; and the host-driven
    loop for comparison) against one signal at a time on the plain FP64 GPU path and on the
    single-signal mixed path, and the gamma-step QP at fixed theta (batch vs plain FP64 one at a
    time, the same stop rule; and the batch alone driven much further, to find how far each
    stop leaves every signal from its optimum)."""
    from pasc_inference_gb300 import PASC_PREC_FP64, PASC_PREC_MIXED, Batch, Problem, capi, datagen
    inst = datagen.batched()
    n = len(inst)
    ts = capi.ts_opts(eps=1e-6, relative=1)
    spg = capi.spgqp_opts(m=10, eps=1e-6)

    def load_batch(theta0, device_loop=True):
        bt = Batch([s.T for s in inst], [s.K for s in inst], [s.epssqr for s in inst], device=dev)
        bt.set_loop(device_loop, 4)
        for i, s in enumerate(inst):
            bt.set_data(i, s.data)
            bt.set_gamma(i, s.gamma0)
            bt.set_theta(i, theta0(s))
        return bt

    # sweep throughput with every signal running (stopping tests off; work items sized for that)
    B_sweep = float(sum((8 * s.K + 4) * s.T for s in inst))
    with load_batch(lambda s: np.linspace(0.0, 4.0, s.K)) as bt:
        bt.spgqp_solve(capi.spgqp_opts(maxit=20, stop_difff=0))
        seg_tiles, item_tiles = bt.get_segment_tiles()
        for i, s in enumerate(inst):
            bt.set_gamma(i, s.gamma0)
        st = bt.spgqp_solve(capi.spgqp_opts(maxit=200, stop_difff=0))
        running = sum(1 for x in st if x.status == capi.PASC_SPG_MAXIT)
        sweep_s = st[0].time_s / (200 + 1)
    gbs = B_sweep / sweep_s / 1e9

    walls, L_b = {True: [], False: []}, None
    for device_loop in (True, True, False):
        with load_batch(lambda s: np.zeros(s.K), device_loop) as bt:
            t0 = time.perf_counter()
            st = bt.ts_solve(ts, spg)
            walls[device_loop].append(time.perf_counter() - t0)
            if device_loop:
                L_b = np.array([x.L for x in st])
                spg_it_b = int(sum(x.spg_it_sum for x in st))
                launches_b = st[0].kernel_launches
    seq = {}
    for name, prec in (("fp64_plain", PASC_PREC_FP64), ("mixed_single", PASC_PREC_MIXED)):
        tot, its, Ls = 0.0, 0, []
        for s in inst:
            with Problem(s.T, s.K, s.epssqr, precision=prec, device=dev) as p:
                p.set_data(s.data)
                p.set_gamma(s.gamma0)
                p.set_theta(np.zeros(s.K))
                t0 = time.perf_counter()
                r = p.ts_solve(ts, spg)
                tot += time.perf_counter() - t0
                its += r.spg_it_sum
                Ls.append(r.L)
        seq[name] = (tot, its, np.array(Ls))
    wall_b = min(walls[True])
    rel = np.abs(L_b - seq["fp64_plain"][2]) / np.abs(seq["fp64_plain"][2])
    # The alternating loop starts from random gamma: its first theta step gives nearly equal
    # levels, and rounding-level differences in the first gamma steps decide which local
    # minimum a signal ends in, so L is compared here only as a distribution.
    res_qp = measure_batched_qp(inst, load_batch, dev) if qp else None
    return {
        "workload": "256 signals, T log-U[1e3,1e6], K U{2..5}, epssqr log-U[1,1000], sorted levels U[0,4], "
                    "segments U[T/50,T/5], sigma U[0.2,1]; TSSolver SPG eps 1e-6 m 10, outer 1e-6 relative",
        "signals": n, "timesteps": int(sum(s.T for s in inst)),
        "work_items": {"segment_tiles": seg_tiles, "item_tiles_all_running": item_tiles,
                       "sizing": "items of 4..32 tiles, about 4 per resident block, resized at every "
                                 "rebuild of the work list"},
        "batch_s": wall_b, "batch_host_loop_s": min(walls[False]), "batch_spg_it_sum": spg_it_b,
        "batch_gpu_launches": launches_b, "batch_loop": "one CUDA graph launch (conditional WHILE nodes)",
        "fp64_plain_sequential_s": seq["fp64_plain"][0], "fp64_plain_spg_it_sum": int(seq["fp64_plain"][1]),
        "mixed_single_sequential_s": seq["mixed_single"][0],
        "mixed_single_spg_it_sum": int(seq["mixed_single"][1]),
        "speedup_vs_fp64_plain_sequential": seq["fp64_plain"][0] / wall_b,
        "speedup_vs_mixed_single_sequential": seq["mixed_single"][0] / wall_b,
        "L_rel_diff_vs_fp64_random_start": {"median": float(np.median(rel)), "max": float(np.max(rel)),
                                            "frac_within_1e-6": float(np.mean(rel <= 1e-6)),
                                            "frac_within_1e-4": float(np.mean(rel <= 1e-4))},
        "qp_fixed_theta": res_qp,
        "sweep_all_running": {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                              "us_per_sweep": sweep_s * 1e6, "bytes_per_sweep": B_sweep,
                              "signals_running_at_end": running},
    }


def _dist(f, fbest):
    r = (np.asarray(f) - fbest) / np.abs(fbest)
    return {"median": float(np.median(r)), "max": float(np.max(r)), "frac_within_1e-6": float(np.mean(r <= 1e-6)),
            "frac_within_1e-5": float(np.mean(r <= 1e-5))}


def measure_batched_qp(inst, load_batch, dev):
    """The gamma-step QP of every batched signal at fixed theta (its sorted true levels) from
    the same random start, a convex problem: the batch and the plain FP64 path one signal at a
    time under the same stop rule (the reference's default, |f - f_old| < 1e-9, GLL m 10, maxit
    20000), and the batch again with |f - f_old| < 1e-14 and maxit 200000.  f_best per signal is
    the lowest objective any of the three runs reached; each run's distance from it (relative)
    shows where its stop left the signals, and the two paths under the same rule are compared
    signal by signal."""
    from pasc_inference_gb300 import PASC_PREC_FP64, Problem, capi
    qp_spg = capi.spgqp_opts(m=10, eps=1e-9, maxit=20000)
    tight = capi.spgqp_opts(m=10, eps=1e-14, maxit=200000)
    runs = {}
    for name, o in (("batch", qp_spg), ("batch_tight", tight)):
        walls = []
        for rep in range(2 if name == "batch" else 1):
            with load_batch(lambda s: s.levels) as bt:
                t0 = time.perf_counter()
                qst = bt.spgqp_solve(o)
                walls.append(time.perf_counter() - t0)
        runs[name] = (min(walls), np.array([x.fx for x in qst]), int(sum(x.it for x in qst)),
                      int(sum(1 for x in qst if x.status == capi.PASC_SPG_CONVERGED)))
    q64_s, q64_it, f_64, conv64 = 0.0, 0, [], 0
    for s in inst:
        with Problem(s.T, s.K, s.epssqr, precision=PASC_PREC_FP64, device=dev) as p:
            p.set_data(s.data)
            p.set_gamma(s.gamma0)
            p.set_theta(s.levels)
            p.update_b()
            t0 = time.perf_counter()
            r = p.spgqp_solve(qp_spg)
            q64_s += time.perf_counter() - t0
            q64_it += r.it
            conv64 += r.status == capi.PASC_SPG_CONVERGED
            f_64.append(r.fx)
    f_64 = np.array(f_64)
    fbest = np.minimum(np.minimum(runs["batch"][1], runs["batch_tight"][1]), f_64)
    qrel = np.abs(runs["batch"][1] - f_64) / np.abs(f_64)
    return {"theta": "sorted true levels of each signal, fixed",
            "stop": "|f - f_old| < 1e-9, GLL m 10, maxit 20000 (both paths)",
            "batch_s": runs["batch"][0], "batch_spg_it_sum": runs["batch"][2], "batch_converged": runs["batch"][3],
            "fp64_plain_sequential_s": q64_s, "fp64_plain_spg_it_sum": q64_it, "fp64_converged": int(conv64),
            "speedup_vs_fp64_plain_sequential": q64_s / runs["batch"][0],
            "f_rel_diff_batch_vs_fp64_same_rule": {"median": float(np.median(qrel)), "max": float(np.max(qrel)),
                                                    "frac_within_1e-6": float(np.mean(qrel <= 1e-6)),
                                                    "frac_batch_lower": float(np.mean(runs["batch"][1] < f_64))},
            "distance_from_f_best": {"batch": _dist(runs["batch"][1], fbest), "fp64_plain": _dist(f_64, fbest),
                                     "batch_tight": _dist(runs["batch_tight"][1], fbest)},
            "batch_tight": {"stop": "|f - f_old| < 1e-14, maxit 200000", "s": runs["batch_tight"][0],
                            "spg_it_sum": runs["batch_tight"][2], "converged": runs["batch_tight"][3]}}


if __name__ == "__main__":
    main()
