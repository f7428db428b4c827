"""The reference's own GPU kernels, launched beside the new ones: TEST INFRASTRUCTURE.

oracle/ref/Makefile compiles the reference's nufi/cuda_kernel.cu (where it
lies, unchanged; the configured f0 supplied as explicit specialisations of
config_t<real>::f0, see ref_gpu.cu) into oracle/_ref/nufi_ref_gpu.cubin,
device code only, plus the names of its entry functions and the byte layout
of its by-value config arguments.  This module loads the cubin through the
CUDA driver API (ctypes on libcuda, inside torch's context) and launches
nufi::dim{1,2,3}::cuda_eval_rho<real, order> exactly as the reference's
cuda_kernel::compute_rho does (nufi/cuda_kernel.cu:112-132, 289-311,
486-510: rho zeroed, 64-thread blocks, one thread per quadrature point in
the reference's q order, one atomicAdd each).

It is used by tests/test_gpu_reference_kernel.py (the reference's GPU rho
against the new FP64 path) and, as a script, to time the reference's GPU
path beside the new kernels on the same GPU:

    python oracle/ref/ref_gpu.py [--workload two_stream_1d_256x1024_T50]

Nothing in the product path imports it.
"""
from __future__ import annotations

import ctypes
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
REF_DIR = ROOT / "oracle" / "_ref"
BLOCK = 64  # nufi/cuda_kernel.cu:124, 301, 497

SPACE = ("x", "y", "z")
VEL = ("u", "v", "w")


class RefGpuUnavailable(RuntimeError):
    pass


def available() -> bool:
    return all((REF_DIR / f).exists() for f in ("nufi_ref_gpu.cubin", "nufi_ref_gpu.entries", "ref_gpu_layout.json"))


class RefGpu:
    """The reference's cuda_eval_rho<real, order> (dim 1, 2, 3), launched on
    torch's current CUDA context and stream."""

    def __init__(self):
        if not available():
            raise RefGpuUnavailable("oracle/_ref holds no reference GPU build (make -C oracle/ref gpu)")
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # the runtime's primary context, current on this thread
        self.torch = torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.layout = json.loads((REF_DIR / "ref_gpu_layout.json").read_text())
        self.entries = (REF_DIR / "nufi_ref_gpu.entries").read_text().split()
        self._check(self.cu.cuInit(0), "cuInit")
        ctx = ctypes.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RefGpuUnavailable("no current CUDA context")
        self.module = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.module), str(REF_DIR / "nufi_ref_gpu.cubin").encode()),
                    "cuModuleLoad")
        self.funcs = {}

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed (CUresult {rc})")

    def _func(self, dim: int, real: str, order: int):
        key = (dim, real, order)
        if key not in self.funcs:
            tag = {"float": "If", "double": "Id"}[real]
            prefix = f"_ZN4nufi4dim{dim}13cuda_eval_rho{tag}Lm{order}E"
            name = next((e for e in self.entries if e.startswith(prefix)), None)
            if name is None:
                raise RefGpuUnavailable(f"dim{dim}::cuda_eval_rho<{real},{order}> not in the cubin")
            f = ctypes.c_void_p()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.module, name.encode()), "cuModuleGetFunction")
            self.funcs[key] = f
        return self.funcs[key]

    def set_f0(self, kind: int, params) -> None:
        """The configured f0 (kind, alpha, k, u_b, sigma_b ...) into the
        cubin's __constant__ nufi_ref_f0 (nufi_f0_params layout)."""
        lay = self.layout["nufi_f0_params"]
        buf = bytearray(lay["size"])
        buf[lay["kind"]:lay["kind"] + 4] = int(kind).to_bytes(4, "little", signed=True)
        p = np.zeros(8, dtype=np.float64)
        p[:len(params)] = params
        buf[lay["p"]:lay["p"] + 64] = p.tobytes()
        dptr = ctypes.c_uint64()
        size = ctypes.c_size_t()
        self._check(self.cu.cuModuleGetGlobal_v2(ctypes.byref(dptr), ctypes.byref(size), self.module, b"nufi_ref_f0"),
                    "cuModuleGetGlobal")
        if size.value != len(buf):
            raise RuntimeError(f"nufi_ref_f0 is {size.value} bytes, layout says {len(buf)}")
        src = (ctypes.c_char * len(buf)).from_buffer(buf)
        self._check(self.cu.cuMemcpyHtoD_v2(dptr, src, ctypes.c_size_t(len(buf))), "cuMemcpyHtoD")

    def pack_conf(self, real: str, cfg) -> bytes:
        """dim{D}::config_t<real> by value for a Config, the derived fields
        computed in `real` as the reference's constructors do
        (nufi/config.hpp:53-67, 116-135, 195-219)."""
        D = cfg.dim
        lay = self.layout[f"dim{D}::config_t<{real}>"]
        R = np.float32 if real == "float" else np.float64
        f = {"dt": R(cfg.dt)}
        ints = {"Nt": cfg.Nt}
        for a in range(D):
            s, v = SPACE[a], VEL[a]
            ints["N" + s] = cfg.Nx[a]
            ints["N" + v] = cfg.Nv[a]
            f[s + "_min"], f[s + "_max"] = R(cfg.x_min[a]), R(cfg.x_max[a])
            f[v + "_min"], f[v + "_max"] = R(cfg.v_min[a]), R(cfg.v_max[a])
            L = R(f[s + "_max"] - f[s + "_min"])
            f["L" + s], f["L" + s + "_inv"] = L, R(R(1) / L)
            d = R(L / R(cfg.Nx[a]))
            f["d" + s], f["d" + s + "_inv"] = d, R(R(1) / d)
            f["d" + v] = R(R(f[v + "_max"] - f[v + "_min"]) / R(cfg.Nv[a]))
        off = lay["fields"]
        if set(off) != set(f) | set(ints):
            raise RuntimeError(f"config_t layout fields {sorted(off)} do not match {sorted(set(f) | set(ints))}")
        buf = bytearray(lay["size"])
        for name, v in ints.items():
            buf[off[name]:off[name] + 8] = int(v).to_bytes(8, "little")
        for name, v in f.items():
            b = np.array([v], dtype=R).tobytes()
            buf[off[name]:off[name] + len(b)] = b
        return bytes(buf)

    def eval_rho(self, real: str, cfg, n: int, coeffs, conf: bytes, rho, q_begin: int = 0, q_end: int | None = None,
                 stream=None) -> None:
        """rho = 0, then dim{D}::cuda_eval_rho<real, order> over q in
        [q_begin, q_end) (cuda_kernel::compute_rho).  coeffs and rho are torch
        tensors of the real type; the sizes are checked here so that every
        access of the kernel stays inside them."""
        torch = self.torch
        dt = torch.float32 if real == "float" else torch.float64
        Nq, Ns = cfg.n_points, cfg.n_spatial
        q_end = Nq if q_end is None else q_end
        if not (0 <= n <= cfg.Nt and 0 <= q_begin <= q_end <= Nq):
            raise ValueError("step or point range out of range")
        if coeffs.dtype != dt or rho.dtype != dt or not coeffs.is_cuda or not rho.is_cuda:
            raise TypeError("coeffs and rho must be CUDA tensors of the kernel's real type")
        # slabs 0..n-1 are read; a window at the wrap edge may reach past its
        # slab by less than one slab
        if coeffs.numel() < (cfg.Nt + 2) * cfg.stride_t or rho.numel() < Ns:
            raise ValueError("coeffs or rho too small")
        if len(conf) != self.layout[f"dim{cfg.dim}::config_t<{real}>"]["size"]:
            raise ValueError("config of the wrong size")
        rho[:Ns].zero_()
        if q_end == q_begin:
            return
        N = q_end - q_begin
        nblocks = 1 + (N - 1) // BLOCK
        if nblocks >= 2 ** 31:
            raise ValueError("too many blocks")
        a_n = ctypes.c_size_t(n)
        a_c = ctypes.c_void_p(coeffs.data_ptr())
        a_conf = (ctypes.c_char * len(conf)).from_buffer_copy(conf)
        a_rho = ctypes.c_void_p(rho.data_ptr())
        a_qb = ctypes.c_size_t(q_begin)
        a_qe = ctypes.c_size_t(q_end)
        params = (ctypes.c_void_p * 6)(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in
                                         (a_n, a_c, a_conf, a_rho, a_qb, a_qe)])
        st = ctypes.c_void_p(stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        self._check(self.cu.cuLaunchKernel(self._func(cfg.dim, real, cfg.order), ctypes.c_uint(nblocks),
                                           ctypes.c_uint(1), ctypes.c_uint(1), ctypes.c_uint(BLOCK), ctypes.c_uint(1),
                                           ctypes.c_uint(1), ctypes.c_uint(0), st, params, None), "cuLaunchKernel")


def device_history(cfg, hist: np.ndarray, real: str):
    """The FP64 coefficient history as a CUDA tensor of `real`, padded by one
    slab (a window at the wrap edge may read past its slab)."""
    import torch
    dt = torch.float32 if real == "float" else torch.float64
    t = torch.zeros((cfg.Nt + 2) * cfg.stride_t, dtype=dt, device="cuda")
    t[:hist.size] = torch.from_numpy(np.ascontiguousarray(hist)).to(device="cuda", dtype=dt)
    return t


# Steps timed per dimension and precision: every step where that is quick,
# a spread of steps where the reference's kernel is slow (the rate is flat
# in n beyond the first few steps).
def timed_steps(cfg, real: str):
    Nt = cfg.Nt
    if cfg.dim == 1:
        return list(range(0, Nt + 1)) if real == "float" else list(range(8, Nt + 1, 8))
    if cfg.dim == 2:
        return list(range(4, Nt + 1, 4)) if real == "float" else list(range(16, Nt + 1, 16))
    return [Nt // 5, 2 * Nt // 5, 3 * Nt // 5, 4 * Nt // 5, Nt] if real == "float" else [Nt // 4, Nt // 2]


def main(argv=None) -> int:
    """Times the reference's GPU path (cuda_eval_rho<float,4> and <double,4>,
    one launch per step as its drivers do) on a workload's coefficient
    history (from the new FP32-split run), beside the new per-step kernels
    on the same history, and checks the reference's rho against the new
    FP64 rho at a few steps."""
    import argparse
    import torch
    sys.path.insert(0, str(ROOT))
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300.config import WORKLOADS, _F0_NAMES

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="two_stream_1d_256x1024_T50", choices=sorted(WORKLOADS))
    ap.add_argument("--profile-step", type=int, default=None,
                    help="only launch the reference's cuda_eval_rho<double,4> and the new FP64 trace once each at "
                         "this step, for a profiler")
    args = ap.parse_args(argv)
    nufi.load()
    cfg = WORKLOADS[args.workload]().replace(precision="fp64")
    Nq, Ns, Nt = cfg.n_points, cfg.n_spatial, cfg.Nt
    ref = RefGpu()
    ref.set_f0(_F0_NAMES[cfg.f0], cfg.f0_params)
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        sim.run()
        hist = sim.history()
    if args.profile_step is not None:
        n = args.profile_step
        coeffs = device_history(cfg, hist, "double")
        rho = torch.zeros(Ns, dtype=coeffs.dtype, device="cuda")
        ref.eval_rho("double", cfg, n, coeffs, ref.pack_conf("double", cfg), rho)
        torch.cuda.synchronize()
        with nufi.Simulation(cfg) as sim:
            for k in range(n):
                sim.upload_phi(k, hist)
            sim.compute_rho(n)
            sim.synchronize()
        print(json.dumps({"profile_step": n, "point_steps_per_launch": Nq * n}), flush=True)
        return 0

    check_steps = sorted({1, 2, Nt // 2, Nt})
    rho_new = {}
    with nufi.Simulation(cfg) as sim:
        for k in range(Nt + 1):
            sim.upload_phi(k, hist)
        for n in check_steps:
            sim.compute_rho(n)
            rho_new[n] = sim.download_rho(np.zeros(Ns))
    stream = torch.cuda.current_stream()

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    out = {"workload": args.workload, "dim": cfg.dim, "Nq": Nq, "Nt": Nt, "order": cfg.order,
           "path": f"reference nufi/cuda_kernel.cu built for sm_103a: dim{cfg.dim}::cuda_eval_rho<real,4>, "
                   "64-thread blocks, one FP atomicAdd per point, rho zeroed per step (cuda_kernel::compute_rho)",
           "history": "from the new FP32-split run of the workload"}
    for real in ("double", "float"):
        coeffs = device_history(cfg, hist, real)
        rho = torch.zeros(Ns, dtype=coeffs.dtype, device="cuda")
        conf = ref.pack_conf(real, cfg)
        errs = {}
        for n in check_steps:
            ref.eval_rho(real, cfg, n, coeffs, conf, rho)
            r = rho.double().cpu().numpy()
            errs[n] = float(np.max(np.abs(r - rho_new[n])) / max(np.max(np.abs(rho_new[n])), 1e-300))
        steps = timed_steps(cfg, real)
        ref.eval_rho(real, cfg, steps[0], coeffs, conf, rho)  # warm-up
        ms = timed(lambda: [ref.eval_rho(real, cfg, n, coeffs, conf, rho) for n in steps])
        ps = Nq * sum(steps)
        out[f"reference_{real}"] = {"point_steps_per_s": ps / (ms * 1e-3), "ms": ms, "steps_timed": len(steps),
                                    "point_steps": ps, "rho_rel_err_vs_new_fp64": errs}
    # the new per-step kernels on the same history (drop-in compute_rho)
    for prec, real in (("fp32split", "float"), ("fp64", "double")):
        with nufi.Simulation(cfg.replace(precision=prec)) as sim:
            for n in range(Nt + 1):
                sim.upload_phi(n, hist)
            steps = timed_steps(cfg, real)
            ext = torch.cuda.ExternalStream(sim.stream)
            sim.compute_rho(steps[0])
            sim.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(ext):
                e0.record()
            for n in steps:
                sim.compute_rho(n)
            with torch.cuda.stream(ext):
                e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            ps = Nq * sum(steps)
            out[f"new_{prec}_per_step"] = {"point_steps_per_s": ps / (ms * 1e-3), "ms": ms, "steps_timed": len(steps)}
    out["speedup_new_split_vs_reference_float"] = (out["new_fp32split_per_step"]["point_steps_per_s"] /
                                                   out["reference_float"]["point_steps_per_s"])
    out["speedup_new_fp64_vs_reference_double"] = (out["new_fp64_per_step"]["point_steps_per_s"] /
                                                   out["reference_double"]["point_steps_per_s"])
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
