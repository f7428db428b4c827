#!/usr/bin/env python3
"""Benchmark of the NuFI hot path on GB300: backtraced point-steps/s.

A step is one whole simulation of the workload (default: 1D1V two-stream
instability, 256 x 1024 quadrature, dt = 1/16, T = 50, i.e. 801 time steps
and 8.40e10 backtraced point-steps): every time step traces all points back
through all earlier substeps, reduces rho, and runs the Poisson + spline
solve that appends the next coefficient slab.  The headline is the
FP32-split form; the FP64 plain form runs beside it for the error gate
(max_n |W_split - W_fp64| / max_n |W_fp64| <= 1e-6) and its own rate.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own
GPU (the path is not split across GPUs); value is the total point-steps of
all ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "backtraced point-steps/s FP32-split vs FP64 at ≤1e-6 rel. energy error"
UNIT = "point-steps/s"
# Algorithmic work per point-step (one drift + one field evaluation + one
# kick, order 4, all field components from one gather): 1D 30, 2D 136,
# 3D 460 flop.
FLOP_PER_POINT_STEP = {1: 30, 2: 136, 3: 460}
# Shared-memory bytes the FP32-split trace loads per point-step: the 1D
# per-cell table entry (one float4), the 4x4 / 4x4x4 FP32 slab window.
SMEM_BYTES_PER_POINT_STEP = {1: 16, 2: 64, 3: 256}
GATE = 1e-6


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks + throttle reasons, sampled every `interval_ms`;
    each line is stamped on arrival, and stop(t0, t1) keeps the samples
    inside the timed window [t0, t1] (time.monotonic())."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu: int, interval_ms: int = 50):
        self.gpu = gpu
        self.interval_ms = interval_ms
        self.proc = None
        self.lines = []  # (arrival time, line)
        self.thread = None

    def start(self, ready_timeout: float = 3.0):
        """Start sampling and wait (at most ready_timeout s) for the first
        sample, so that sampling covers a timed region started next."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", str(self.interval_ms), "-i", str(self.gpu)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        t_end = time.monotonic() + ready_timeout
        while not self.lines and time.monotonic() < t_end and self.proc.poll() is None:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def stop(self, t0: float | None = None, t1: float | None = None):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        inside = [ln for t, ln in self.lines if (t0 is None or t >= t0) and (t1 is None or t <= t1)]
        in_window = bool(inside)
        if not inside:  # a window shorter than the interval: the samples around it
            inside = [ln for _, ln in self.lines]
        sm, smax, reasons = [], [], set()
        for ln in inside:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(self.NAMES, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "in_timed_window": in_window}


def aggregate_replicas(total_ms: float, steps: int, point_steps: int, ws: int, device: str = "cuda"):
    """Replicas on ws ranks (one GPU each, the same workload): the slowest
    rank's time per step and the whole-job rate ws * point_steps / time.
    With ws > 1 the max is taken over the process group."""
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(total_ms)], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / steps
    return ms_per_step, ws * point_steps / (ms_per_step * 1e-3)


def measure_peaks():
    """FP32 / FP64 FMA throughput (TFLOP/s) and shared-memory load bandwidth
    (GB/s) of this GPU, from probes/peaks.cu (best of 3 each)."""
    import ctypes
    lib = ctypes.CDLL(str(ROOT / "numericalflowiteration_gb300" / "libnufi_probes.so"))
    lib.nufi_probe_fma_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.nufi_probe_smem_bw.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    out = {}
    for name, fp64, iters in (("fp32", 0, 4096), ("fp64", 1, 128)):
        best = 0.0
        for _ in range(3):
            t = ctypes.c_double()
            ms = ctypes.c_double()
            if lib.nufi_probe_fma_peak(fp64, iters, ctypes.byref(t), ctypes.byref(ms)) == 0:
                best = max(best, t.value)
        out[name] = best
    best = 0.0
    for _ in range(3):
        g = ctypes.c_double()
        ms = ctypes.c_double()
        if lib.nufi_probe_smem_bw(2048, ctypes.byref(g), ctypes.byref(ms)) == 0:
            best = max(best, g.value)
    out["smem_gbs"] = best
    return out


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu
    summary (profiles/traffic.json), or None."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        return json.loads(p.read_text()).get(f"{kernel}@{workload}")
    except (ValueError, OSError):
        return None


def golden_energy(workload: str, nt: int):
    """The reference's own energy history of the whole workload, from the
    committed golden fixture tests/golden/<workload>.npz (written by
    tests/golden/make_golden.py with the reference's code): (in-order,
    compensated) arrays of W_0..W_Nt, or None where no such fixture exists."""
    p = ROOT / "tests" / "golden" / f"{workload}.npz"
    if not p.exists():
        return None
    g = np.load(p)
    if int(g["n_last"]) != nt:
        return None
    return np.asarray(g["energy"]), np.asarray(g["energy_comp"])


def energy_errors_vs_oracle(e_split, e64, gold):
    """Errors of the FP32-split and FP64 energy histories against the
    reference's (compensated rho sums; the in-order one beside it)."""
    ref_inorder, ref_comp = gold

    def errs(e, ref):
        d = np.abs(np.asarray(e) - ref)
        return {"max_normalised": float(np.max(d) / np.max(np.abs(ref))),
                "pointwise_max": float(np.max(d / np.abs(ref)))}

    return {"oracle": "reference energy history W_0..W_Nt (tests/golden, the reference's own code, "
                      "compensated rho sums)",
            "fp32split": errs(e_split, ref_comp), "fp64": errs(e64, ref_comp),
            "fp64_vs_inorder_reference": errs(e64, ref_inorder),
            "reference_summation_floor": float(np.max(np.abs(ref_inorder - ref_comp)) / np.max(np.abs(ref_comp))),
            "gating_measure": "max_normalised"}


def parse_windows(spec: str, nt: int):
    """'0:10,200:10,...' -> [(first step, count), ...]; a first step below
    0 counts from the end (-10:10 = the last 10 steps)."""
    out = []
    for part in spec.split(","):
        a, b = part.split(":")
        n0, cnt = int(a), int(b)
        if n0 < 0:
            n0 = nt + 1 + n0
        n0 = max(0, min(n0, nt))
        out.append((n0, max(1, min(cnt, nt + 1 - n0))))
    return out


def cpu_windows(cfg, windows, threads: int):
    """The CPU loop of the reference (oracle port: per step rho over all
    points, then the field solve) timed step by step in the given windows
    of the workload, and the whole run's time extrapolated from them.

    Step n costs t(n) = c0 + c1 n: c0 (f0 at every point, the rho sums,
    the solve) and c1 (one backward substep of every point) are fitted by
    least squares to the timed steps; the whole run is then
    sum_{n=0..Nt} t(n) = (Nt+1) c0 + c1 Nt(Nt+1)/2.  The first window
    starts at step 0 and computes real slabs; a later window at n0 runs on
    a history whose slab k is real slab k mod (len of the first window):
    a step's work depends only on n, not on the field values."""
    from oracle import oracle
    oracle.build()
    oracle.set_summation(0)
    windows = sorted(windows)
    if windows[0][0] != 0:
        windows = [(0, 1)] + windows
    st = cfg.stride_t
    hist = np.zeros((cfg.Nt + 1) * st)
    ns, ts = [], []
    real = 0
    for i, (n0, cnt) in enumerate(windows):
        if i > 0:
            h = hist.copy()
            for k in range(real, n0 + cnt):
                h[k * st:(k + 1) * st] = hist[(k % real) * st:(k % real + 1) * st]
        else:
            h = hist
        for n in range(n0, n0 + cnt):
            t0 = time.perf_counter()
            oracle.run(cfg, n, n, coeffs=h, keep_rho=False, nthreads=threads)
            ts.append(time.perf_counter() - t0)
            ns.append(n)
        if i == 0:
            real = n0 + cnt
    A = np.stack([np.ones(len(ns)), np.asarray(ns, dtype=np.float64)], axis=1)
    t_arr = np.asarray(ts)
    (c0, c1), *_ = np.linalg.lstsq(A, t_arr, rcond=None)
    if c0 < 0:  # both costs are non-negative: refit with c0 = 0
        c0, c1 = 0.0, float(np.dot(A[:, 1], t_arr) / np.dot(A[:, 1], A[:, 1]))
    pred = A @ np.array([c0, c1])
    resid = float(np.sqrt(np.mean((pred - np.asarray(ts)) ** 2)) / np.mean(ts))
    nt = cfg.Nt
    full_s = (nt + 1) * c0 + c1 * nt * (nt + 1) / 2
    ps = cfg.point_steps()
    timed_ps = sum(cfg.n_points * n for n in ns)
    return {"value": ps / full_s, "unit": UNIT, "cores": threads, "kind": "port",
            "full_run_s_extrapolated": full_s, "fit_c0_s": float(c0), "fit_c1_s": float(c1),
            "fit_rel_rms_residual": resid, "timed_s": float(sum(ts)), "same_config": True,
            "sample": (f"{len(ns)} steps of the workload in windows "
                       + ",".join(f"{a}..{a + c - 1}" for a, c in windows)
                       + f" ({timed_ps:.3e} point-steps, {sum(ts):.1f} s, OpenMP over spatial nodes); "
                       "per-step time fitted as c0 + c1 n and summed over all steps 0..Nt")}


def run_reference(args, cfg):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    windows = parse_windows(args.cpu_windows, cfg.Nt)
    vals, fits = [], []
    for k in range(args.warmup + args.steps):
        r = cpu_windows(cfg.replace(precision="fp64"), windows, threads)
        if k >= args.warmup:
            vals.append(r["value"])
            fits.append(r)
    value = statistics.median(vals)
    fit = fits[vals.index(value)] if value in vals else fits[-1]
    ps = cfg.point_steps()
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * ps / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic initial condition)",
            "config": {"workload": args.workload, "Nx": cfg.Nx[0], "Nv": cfg.Nv[0], "Nt": cfg.Nt, "dt": cfg.dt,
                       "point_steps_per_step": ps, "threads": threads, "same_config": True,
                       "sample_windows": args.cpu_windows},
            "cpu_baseline": {**fit, "value": value},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def e2e_c_loop(cfg, device: int, repeats: int, ws: int, ps: int):
    """End to end through the C ABI with host buffers: the reference
    drivers' loop (compute_rho, download_rho, field solve of the host rho,
    upload_phi) as a compiled C++ caller runs it (numericalflowiteration_gb300/
    e2e_loop.cpp), the median of `repeats` whole runs after one untimed run."""
    import tempfile
    exe = ROOT / "numericalflowiteration_gb300" / "e2e_loop"
    with tempfile.TemporaryDirectory() as td:
        cf = Path(td) / "cfg.bin"
        cf.write_bytes(cfg.to_bytes())
        r = subprocess.run([str(exe), str(cf), str(repeats), str(device)], capture_output=True, text=True,
                           timeout=1800)
    if r.returncode != 0:
        raise RuntimeError(f"e2e_loop failed ({r.returncode}): {r.stderr[-2000:]}")
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return {"value": ws * ps / d["seconds"], "unit": UNIT, "ms_per_step": d["seconds"] * 1e3,
            "h2d_bytes_per_step": d["h2d_bytes"], "d2h_bytes_per_step": d["d2h_bytes"], "repeats": repeats,
            "path": "C ABI with host buffers, the reference drivers' loop compiled as a C++ caller "
                    "(compute_rho, download_rho, field_solve, upload_phi per time step)",
            "call_us_per_time_step": d.get("call_us_per_step")}


def e2e_python_loop(nufi, cfg, device: int, repeats: int, ws: int, ps: int):
    """The same loop through the Python binding (ctypes), for comparison."""
    import torch
    sim2 = nufi.Simulation(cfg, device=device)
    rho = np.zeros(cfg.n_spatial)
    coeffs = np.zeros((cfg.Nt + 1) * cfg.stride_t)
    times = []
    for rep in range(1 + repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for n in range(cfg.Nt + 1):
            rho[:] = 0
            sim2.compute_rho(n)
            sim2.download_rho(rho)
            slab, _ = sim2.field_solve(rho)
            coeffs[n * cfg.stride_t:(n + 1) * cfg.stride_t] = slab
            sim2.upload_phi(n, coeffs)
        torch.cuda.synchronize()
        if rep > 0:
            times.append(time.perf_counter() - t0)
    sim2.close()
    s = statistics.median(times)
    return {"value": ws * ps / s, "ms_per_step": s * 1e3}


def run_ours(args, cfg):
    import torch
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300 import build

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    build.build()
    nufi.load()

    cfg_split = cfg.replace(precision="fp32split")
    sim = nufi.Simulation(cfg_split, device=local)
    ext = torch.cuda.ExternalStream(sim.stream, device=torch.device("cuda", local))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        sim.run(energy=False)
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = sim.launches
    times = []
    t_start = time.monotonic()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            e0.record()
        sim.run(energy=False)
        with torch.cuda.stream(ext):
            e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    t_end = time.monotonic()
    barrier()
    clocks = sampler.stop(t_start, t_end)
    launches = sim.launches - launches0
    ps = cfg.point_steps()
    ms_per_step, value = aggregate_replicas(sum(times), args.steps, ps, ws, device="cuda")
    e_split = sim.energy()

    # FP64 plain form: same workload, for the error gate and its own rate.
    fp64 = None
    if not args.no_fp64:
        sim64 = nufi.Simulation(cfg.replace(precision="fp64"), device=local)
        ext64 = torch.cuda.ExternalStream(sim64.stream, device=torch.device("cuda", local))
        sim64.run(energy=False)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext64):
            e0.record()
        sim64.run(energy=False)
        with torch.cuda.stream(ext64):
            e1.record()
        e1.synchronize()
        ms64 = e0.elapsed_time(e1)
        e64 = sim64.energy()
        sim64.close()
        err_max = float(np.max(np.abs(e_split - e64)) / np.max(np.abs(e64)))
        err_pt = float(np.max(np.abs(e_split - e64) / np.abs(e64)))
        fp64 = {"value": ps / (ms64 * 1e-3), "ms_per_step": ms64, "speedup_split_vs_fp64": ms64 / ms_per_step,
                "energy_err_max_normalised": err_max, "energy_err_pointwise_max": err_pt,
                "gate": GATE, "gate_passed": err_max <= GATE,
                "gating_measure": "max_n |dW_n| / max_n |W_n| (normalised); the pointwise max_n |dW_n|/|W_n| "
                                  "is reported beside it"}
        gold = golden_energy(args.workload, cfg.Nt)
        if gold is not None:
            fp64["err_vs_oracle"] = energy_errors_vs_oracle(e_split, e64, gold)
            fp64["gate_passed_vs_oracle"] = fp64["err_vs_oracle"]["fp32split"]["max_normalised"] <= GATE

    # Per-step trace launches: CUDA events around compute_rho(n) on the
    # handle's stream at several n (trace + rho reduction).
    ns = [cfg.Nt // 4, cfg.Nt // 2, (3 * cfg.Nt) // 4, cfg.Nt]
    kt, kps = 0.0, 0
    for n in ns:
        for rep in range(2):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(ext):
                e0.record()
            sim.compute_rho(n)
            with torch.cuda.stream(ext):
                e1.record()
            e1.synchronize()
            if rep == 1:
                kt += e0.elapsed_time(e1)
                kps += cfg.n_points * n
    kernel_rate = kps / (kt * 1e-3)
    peaks = measure_peaks()
    flop = FLOP_PER_POINT_STEP[cfg.dim]
    desc = sim.describe()
    # The dominant kernel of the timed region: with the whole-run kernel one
    # launch is one timed step (all Nt+1 time steps), so its launch duration
    # is ms_per_step; otherwise the per-step trace launches above.
    if desc["persistent"]["ok"]:
        kname, krate, launch_ms = desc["run"], ps / (ms_per_step * 1e-3), ms_per_step
    else:
        kname, krate, launch_ms = desc["trace"], kernel_rate, kt / len(ns)
    achieved = krate * flop / 1e12
    smem_bytes = SMEM_BYTES_PER_POINT_STEP[cfg.dim]
    roofline = {"bound": "fp32", "achieved": achieved, "peak": peaks["fp32"], "unit": "TFLOP/s",
                "frac": achieved / peaks["fp32"] if peaks["fp32"] else None,
                "traffic": profiled_traffic(kname, args.workload),
                "kernel": kname, "launch_ms": launch_ms, "point_steps_per_s": krate,
                "flop_per_point_step": flop,
                "peak_source": "measured live in this run: FP32 FMA chains (probes/peaks.cu); "
                               "MEASURED_PEAKS.json holds no SIMT peak",
                "smem_cobound": {"bytes_per_point_step": smem_bytes, "achieved_gbs": krate * smem_bytes / 1e9,
                                 "peak_gbs": peaks["smem_gbs"],
                                 "frac": krate * smem_bytes / 1e9 / peaks["smem_gbs"] if peaks["smem_gbs"] else None},
                "per_step_trace": {"kernel": desc["trace"], "point_steps_per_s": kernel_rate},
                "fp64_fma_peak_tflops": peaks["fp64"],
                "traffic_source": "profiles/traffic.json (ncu dram__bytes_read.sum + dram__bytes_write.sum per launch)"}

    # End to end through the reference-facing calls with host buffers, the
    # loop of bin/test_nufi_gpu_1d.cpp:241-252: compute_rho -> download_rho
    # -> field solve (host rho in, host slab out) -> upload_phi, per step.
    e2e = None
    if not args.no_e2e:
        e2e = e2e_c_loop(cfg_split, local, max(2, args.steps), ws, ps)
        e2e["python_loop"] = e2e_python_loop(nufi, cfg_split, local, max(1, args.steps // 2), ws, ps)

    batch = None
    if rank == 0 and ws == 1 and not args.no_batch:
        batch = batch_leg(nufi, local, max(2, min(3, args.steps)))

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_windows(cfg.replace(precision="fp64"), parse_windows(args.cpu_windows, cfg.Nt),
                          os.cpu_count() or 1)
    sim.close()

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (analytic initial condition)",
                "config": {"workload": args.workload, "Nx": cfg.Nx[0], "Nv": cfg.Nv[0], "Nt": cfg.Nt, "dt": cfg.dt,
                           "point_steps_per_step": ps, "precision": "fp32-split (FP64 rho/solve)",
                           "l2": "flushed between timed steps (256 MB write)",
                           "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
                "fp64_plain": fp64, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "batch": batch,
                "gpu_launches": launches, "clocks": clocks}
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_batch(args):
    """The batched configuration: seeded bump-on-tail instances of uneven
    sizes (Nx in {64,128,256}, Nv in {256,512,1024}, T = 20).  Times the
    batched FP32-split forward, the batched FP64 forward and the FP64
    adjoint (gradient of int |E|^2 dt for all instances), CUDA events on the
    batch stream; prints one JSON line."""
    import torch
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300 import build
    from numericalflowiteration_gb300.config import batched_bump_on_tail
    build.build()
    nufi.load()
    cfgs = batched_bump_on_tail(count=args.instances)
    ps = sum(c.point_steps() for c in cfgs)

    def timed(b, fn, reps):
        ext = torch.cuda.ExternalStream(b.stream)
        out = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(ext):
                e0.record()
            fn()
            with torch.cuda.stream(ext):
                e1.record()
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return min(out)

    res = {"instances": len(cfgs), "point_steps": ps}
    with nufi.Batch([c.replace(precision="fp32split") for c in cfgs]) as b:
        b.forward()
        ms = timed(b, b.forward, max(1, args.steps))
        b.backward()
        msb = timed(b, b.backward, max(1, args.steps))
        G_split = b.backward()
        res["split_forward"] = {"ms": ms, "point_steps_per_s": ps / (ms * 1e-3), "autotune": b.describe()["autotune"]}
        res["split_backward"] = {"ms": msb, "cost_vs_forward": msb / ms,
                                 "note": "FP32-split adjoint: characteristics recomputed from per-chunk "
                                         "checkpoints, fixed-point table adjoints"}
    if not args.no_fp64:
        with nufi.Batch(cfgs) as b:
            msf = timed(b, b.forward, 1)
            J = b.forward()
            msb = timed(b, b.backward, 1)
            G = b.backward()
            res["fp64_forward"] = {"ms": msf, "point_steps_per_s": ps / (msf * 1e-3)}
            res["fp64_backward"] = {"ms": msb, "cost_vs_forward": msb / msf,
                                    "autotune": b.describe()["autotune"]["chosen"]}
            res["J_first"] = float(J[0])
            res["grad_first"] = [float(v) for v in G[0]]
            rel = np.abs(G_split - G) / np.maximum(np.abs(G), 1e-300)
            res["split_vs_fp64_grad_rel_max"] = float(np.max(rel))
            res["split_vs_fp64_grad_rel_median"] = float(np.median(rel))
            # relative to each instance's largest component (the tests' measure;
            # a component near zero makes its own relative error meaningless)
            inst = np.max(np.abs(G_split - G), axis=1) / np.max(np.abs(G), axis=1)
            res["split_vs_fp64_grad_rel_to_instance_max"] = float(np.max(inst))
            w = np.unravel_index(int(np.argmax(rel)), rel.shape)
            res["split_vs_fp64_worst_component"] = {"instance": int(w[0]), "component": int(w[1]),
                                                    "split": float(G_split[w]), "fp64": float(G[w])}
    line = {"metric": "batched bump-on-tail: forward point-steps/s and adjoint cost", "config": {
        "workload": f"batched_bump_on_tail_{len(cfgs)}", "seed": 20261203, "Nt": 320, "dt": 1 / 16}, **res}
    print(json.dumps(line), flush=True)
    return 0


def batch_leg(nufi, device: int, reps: int, instances: int = 256, fd_instances: int = 4, fd_h: float = 1e-6):
    """The batched workload (seeded bump-on-tail instances of uneven sizes,
    Nx in {64,128,256}, Nv in {256,512,1024}, T = 20) in the FP32-split
    form: forward and adjoint (gradient of J = int |E|^2 dt with respect to
    alpha, k, u_b, sigma_b of every instance) timed with CUDA events on the
    batch stream, clocks sampled over the timed calls, and the gradient of
    `fd_instances` evenly spaced instances checked against central
    differences of the FP64 forward (single-instance runs, h = fd_h
    relative to each parameter's scale of 1)."""
    import torch
    from numericalflowiteration_gb300.config import batched_bump_on_tail
    cfgs = batched_bump_on_tail(count=instances)
    ps = sum(c.point_steps() for c in cfgs)

    def timed(b, fn):
        ext = torch.cuda.ExternalStream(b.stream, device=torch.device("cuda", device))
        out = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(ext):
                e0.record()
            fn()
            with torch.cuda.stream(ext):
                e1.record()
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return statistics.median(out)

    with nufi.Batch([c.replace(precision="fp32split") for c in cfgs], device=device) as b:
        b.forward()
        b.backward()  # warm-up of both graphs
        torch.cuda.synchronize()
        sampler = ClockSampler(device)
        sampler.start()
        t0 = time.monotonic()
        ms_f = timed(b, b.forward)
        ms_b = timed(b, b.backward)
        t1 = time.monotonic()
        clocks = sampler.stop(t0, t1)
        G = b.backward()
        desc = b.describe()
        chosen = dict(desc["autotune"]["chosen"], forward_launch=desc["forward_launch"],
                      forward_timing=desc["autotune"].get("forward"))
    # central differences of the FP64 forward on sampled instances
    pick = [int(round(i * (instances - 1) / max(1, fd_instances - 1))) for i in range(fd_instances)]
    fd_err = []
    for i in pick:
        c = cfgs[i]
        fd = np.zeros(4)
        for k in range(4):
            pp = list(c.f0_params)
            pp[k] += fd_h
            with nufi.Simulation(c.replace(f0_params=list(pp)), device=device) as s:
                jp = s.forward()
            pp[k] -= 2 * fd_h
            with nufi.Simulation(c.replace(f0_params=list(pp)), device=device) as s:
                jm = s.forward()
            fd[k] = (jp - jm) / (2 * fd_h)
        fd_err.append(float(np.max(np.abs(G[i] - fd)) / np.max(np.abs(fd))))
    return {"workload": f"batched_bump_on_tail_{instances}", "instances": instances, "point_steps": ps,
            "precision": "fp32-split (FP64 rho/solve; FP64 sums of the table adjoints)",
            "forward_ms": ms_f, "forward_point_steps_per_s": ps / (ms_f * 1e-3), "backward_ms": ms_b,
            "backward_cost_vs_forward": ms_b / ms_f, "target_cost_vs_forward": 3.0,
            "grad_vs_central_differences": {"instances": pick, "h": fd_h,
                                            "max_err_rel_to_instance_max": max(fd_err), "per_instance": fd_err,
                                            "tolerance": 1e-5},
            "autotune_chosen": chosen, "timed_reps": reps, "clocks": clocks}


def profile_case(args, cfg):
    """One run of steps 0..nt in one precision; prints the chosen kernels."""
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300 import build
    build.build()
    nufi.load()
    nt = cfg.Nt if args.nt is None else args.nt
    c = cfg.replace(precision=args.precision, Nt=nt)
    with nufi.Simulation(c) as sim:
        e = sim.run()
        print(json.dumps({"workload": args.workload, "precision": args.precision, "nt": nt,
                          "energy_last": float(e[-1]), "kernels": sim.describe()}), flush=True)
    return 0


def main(argv=None):
    from numericalflowiteration_gb300.config import WORKLOADS
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="two_stream_1d_256x1024_T50", choices=sorted(WORKLOADS))
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="leave out the batched forward/adjoint leg")
    ap.add_argument("--cpu-windows", default="0:12,200:6,400:6,600:4,-4:4",
                    help="CPU baseline and reference arm: timed step windows first:count (negative first: "
                         "from the end); the whole run is extrapolated from them")
    ap.add_argument("--profile-case", action="store_true",
                    help="run steps 0..--nt of the workload once in --precision and exit (a small case for ncu)")
    ap.add_argument("--precision", default="fp32split", choices=["fp32split", "fp64"])
    ap.add_argument("--nt", type=int, default=None, help="with --profile-case: last step")
    ap.add_argument("--batch", action="store_true", help="time the batched bump-on-tail configuration and exit")
    ap.add_argument("--instances", type=int, default=256, help="with --batch: number of instances")
    args = ap.parse_args(argv)
    cfg = WORKLOADS[args.workload]()
    if args.profile_case:
        return profile_case(args, cfg)
    if args.batch:
        return run_batch(args)
    if args.impl == "reference":
        return run_reference(args, cfg)
    return run_ours(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
