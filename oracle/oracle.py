"""ctypes binding of the CPU oracle (liboracle.so, built from nufi_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke()
and by bench.py's CPU-baseline leg, always as the oracle that the CUDA
path is compared with.  The product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

_lib = None


def _elf_matches_host(path: Path) -> bool:
    import platform
    want = {"x86_64": 62, "amd64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine().lower())
    try:
        head = path.read_bytes()[:20]
    except OSError:
        return False
    return len(head) == 20 and head[:4] == b"\x7fELF" and (want is None or int.from_bytes(head[18:20], "little") == want)


def build(force: bool = False) -> Path:
    """Compile liboracle.so with the local C compiler (gcc, OpenMP)."""
    srcs = [HERE / "nufi_oracle.c", HERE / "nufi_f0.h"]
    stale = (force or not LIB_PATH.exists() or not _elf_matches_host(LIB_PATH)
             or any(LIB_PATH.stat().st_mtime < s.stat().st_mtime for s in srcs))
    if stale:
        subprocess.run(["make", "-s", "-B", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.oracle_rho.argtypes = [P, i64, P, i64, i64, P, ctypes.c_int]
        L.oracle_eval.argtypes = [P, i64, P, i64, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_metrics.argtypes = [P, i64, P, i64, i64, P, ctypes.c_int, ctypes.c_int]
        L.oracle_field_solve.argtypes = [P, P, P, P]
        L.oracle_poisson.argtypes = [P, P, P]
        L.oracle_interpolate.argtypes = [P, P, P]
        L.oracle_eval_field.argtypes = [P, P, i64, P, P, P]
        L.oracle_run.argtypes = [P, i64, i64, P, P, P, ctypes.c_int]
        L.oracle_sizes.argtypes = [P, P, P, P]
        L.oracle_set_summation.argtypes = [ctypes.c_int]
        L.oracle_objective_tangent.argtypes = [P, i64, P, P, ctypes.c_int]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _cfg(cfg):
    c = cfg.to_c()
    return c, ctypes.cast(ctypes.pointer(c), ctypes.c_void_p)


def _check(st: int, what: str):
    if st != 0:
        raise RuntimeError(f"oracle {what} failed with status {st}")


def set_summation(mode: int):
    """0: in-order double sum over velocity (the reference's CPU loop);
    1: compensated sum (the exact sum of the same f~ values to ~1 ulp)."""
    lib().oracle_set_summation(int(mode))


def threads() -> int:
    return int(os.environ.get("NUFI_ORACLE_THREADS", os.cpu_count() or 1))


def run(cfg, n0: int = 0, n1: int | None = None, coeffs: np.ndarray | None = None, keep_rho: bool = True,
        nthreads: int | None = None):
    """Steps n0..n1 of the reference loop.  Returns (energy, rho_hist, coeffs)."""
    n1 = cfg.Nt if n1 is None else n1
    c, p = _cfg(cfg)
    if coeffs is None:
        coeffs = np.zeros((cfg.Nt + 1) * cfg.stride_t)
    energy = np.zeros(n1 - n0 + 1)
    rho = np.zeros((n1 - n0 + 1) * cfg.n_spatial) if keep_rho else None
    st = lib().oracle_run(p, n0, n1, _ptr(coeffs), _ptr(energy), _ptr(rho) if keep_rho else None,
                          nthreads or threads())
    _check(st, "run")
    return energy, (rho.reshape(n1 - n0 + 1, cfg.n_spatial) if keep_rho else None), coeffs


def objective(cfg, n1: int | None = None, nthreads=None) -> float:
    """J = 2 dt sum_{n<=n1} W_n of the reference loop (oracle_run)."""
    n1 = cfg.Nt if n1 is None else n1
    energy, _, _ = run(cfg, 0, n1, keep_rho=False, nthreads=nthreads)
    return 2.0 * cfg.dt * float(np.sum(energy))


def objective_tangent(cfg, n1: int | None = None, nthreads=None):
    """(J, dJ/d(alpha, k, u_b, sigma_b)) by forward-mode differentiation of
    the 1D loop in FP64 (oracle_objective_tangent)."""
    n1 = cfg.Nt if n1 is None else n1
    c, p = _cfg(cfg)
    J = np.zeros(1)
    dJ = np.zeros(4)
    _check(lib().oracle_objective_tangent(p, n1, _ptr(J), _ptr(dJ), nthreads or threads()), "objective_tangent")
    return float(J[0]), dJ


def rho(cfg, n: int, coeffs: np.ndarray, q_begin: int = 0, q_end: int | None = None, nthreads=None):
    q_end = cfg.n_points if q_end is None else q_end
    c, p = _cfg(cfg)
    out = np.zeros(cfg.n_spatial)
    _check(lib().oracle_rho(p, n, _ptr(coeffs), q_begin, q_end, _ptr(out), nthreads or threads()), "rho")
    return out


def field_solve(cfg, rho_in: np.ndarray):
    c, p = _cfg(cfg)
    r = np.ascontiguousarray(rho_in, dtype=np.float64)
    slab = np.zeros(cfg.stride_t)
    e = np.zeros(1)
    _check(lib().oracle_field_solve(p, _ptr(r), _ptr(slab), _ptr(e)), "field_solve")
    return slab, float(e[0])


def poisson(cfg, data: np.ndarray):
    c, p = _cfg(cfg)
    d = np.ascontiguousarray(data, dtype=np.float64).copy()
    e = np.zeros(1)
    _check(lib().oracle_poisson(p, _ptr(d), _ptr(e)), "poisson")
    return d, float(e[0])


def interpolate(cfg, values: np.ndarray):
    c, p = _cfg(cfg)
    v = np.ascontiguousarray(values, dtype=np.float64)
    slab = np.zeros(cfg.stride_t)
    _check(lib().oracle_interpolate(p, _ptr(v), _ptr(slab)), "interpolate")
    return slab


def eval_points(cfg, n: int, coeffs: np.ndarray, pts: np.ndarray, mode: int = 0, feet: bool = False,
                nthreads=None):
    """f~ (mode 0) or f (mode 1) at points (npts, 2*dim); feet written back if asked."""
    c, p = _cfg(cfg)
    pts = np.ascontiguousarray(pts, dtype=np.float64).copy()
    out = np.zeros(pts.shape[0])
    _check(lib().oracle_eval(p, n, _ptr(coeffs), pts.shape[0], _ptr(pts), _ptr(out), mode, int(feet),
                             nthreads or threads()), "eval")
    return (out, pts) if feet else out


def metrics(cfg, n: int, coeffs: np.ndarray, q_begin=0, q_end=None, weight3d_full=False, nthreads=None):
    q_end = cfg.n_points if q_end is None else q_end
    c, p = _cfg(cfg)
    m = np.zeros(4)
    _check(lib().oracle_metrics(p, n, _ptr(coeffs), q_begin, q_end, _ptr(m), int(weight3d_full),
                                nthreads or threads()), "metrics")
    return m


def eval_field(cfg, slab: np.ndarray, pts: np.ndarray, deriv=(0, 0, 0)):
    c, p = _cfg(cfg)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    d = (ctypes.c_int * 3)(*deriv)
    out = np.zeros(pts.shape[0])
    _check(lib().oracle_eval_field(p, _ptr(np.ascontiguousarray(slab)), pts.shape[0], _ptr(pts),
                                   ctypes.cast(d, ctypes.c_void_p), _ptr(out)), "eval_field")
    return out
