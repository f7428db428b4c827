"""ctypes binding of libnufi_gb300.so (include/nufi_gb300.h).

``Simulation`` mirrors the reference's per-device object
``nufi::dimN::cuda_kernel<real,order>`` (nufi/cuda_kernel.hpp:33-56): the
drop-in calls compute_rho / download_rho / upload_phi, plus the
device-resident step / run / field_solve of this library.  Failures raise
the exception type the reference raises for the same condition:
``IndexError`` where it throws std::range_error, ``RuntimeError`` for CUDA
errors (nufi::cuda::exception), ``ValueError`` for invalid arguments and
``NotImplementedError`` for configurations the library does not cover.

There is no fallback: if the CUDA library is missing or cannot load,
``load()`` raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from .config import Config, NufiConfigC

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libnufi_gb300.so"

OK, ERR_INVALID, ERR_RANGE, ERR_CUDA, ERR_UNSUPPORTED, ERR_DEVICE = range(6)

# Every exported function of include/nufi_gb300.h with its C signature.
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
SIGNATURES = {
    "nufi_last_error": (ctypes.c_char_p, [_P]),
    "nufi_create": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_P)]),
    "nufi_create_ex": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.POINTER(_P)]),
    "nufi_plan_ex": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]),
    "nufi_batch_create_ex": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_int, _P]),
    "nufi_destroy": (ctypes.c_int, [_P]),
    "nufi_compute_rho": (ctypes.c_int, [_P, _I64, _I64, _I64]),
    "nufi_download_rho": (ctypes.c_int, [_P, _P]),
    "nufi_download_rho_f32": (ctypes.c_int, [_P, _P]),
    "nufi_upload_phi": (ctypes.c_int, [_P, _I64, _P]),
    "nufi_upload_phi_f32": (ctypes.c_int, [_P, _I64, _P]),
    "nufi_compute_metrics": (ctypes.c_int, [_P, _I64, _I64, _I64]),
    "nufi_describe": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "nufi_plan": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]),
    "nufi_solve_kernels": (ctypes.c_int, [_P, _P, _I64, _P]),
    "nufi_forward": (ctypes.c_int, [_P, _I64, _P]),
    "nufi_eval_points": (ctypes.c_int, [_P, _I64, ctypes.c_int, _I64, _P, _P, _P]),
    "nufi_save_history": (ctypes.c_int, [_P, _I64, ctypes.c_char_p]),
    "nufi_load_history": (ctypes.c_int, [_P, ctypes.c_char_p, _P]),
    "nufi_objective": (ctypes.c_int, [_P, _I64, _P]),
    "nufi_backward": (ctypes.c_int, [_P, _I64, _P]),
    "nufi_batch_create": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int, _P]),
    "nufi_batch_destroy": (ctypes.c_int, [_P]),
    "nufi_batch_last_error": (ctypes.c_char_p, [_P]),
    "nufi_batch_forward": (ctypes.c_int, [_P, _P]),
    "nufi_batch_backward": (ctypes.c_int, [_P, _P]),
    "nufi_batch_energy": (ctypes.c_int, [_P, ctypes.c_int32, _P]),
    "nufi_batch_stream": (ctypes.c_int, [_P, _P]),
    "nufi_batch_describe": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "nufi_download_metrics": (ctypes.c_int, [_P, _P]),
    "nufi_set_metrics_grid": (ctypes.c_int, [_P, _P]),
    "nufi_step": (ctypes.c_int, [_P, _I64, _P]),
    "nufi_run": (ctypes.c_int, [_P, _I64, _I64, _P]),
    "nufi_download_history": (ctypes.c_int, [_P, _I64, _I64, _P]),
    "nufi_download_energy": (ctypes.c_int, [_P, _I64, _I64, _P]),
    "nufi_field_solve": (ctypes.c_int, [_P, _P, _P, _P]),
    "nufi_synchronize": (ctypes.c_int, [_P]),
    "nufi_sizes": (ctypes.c_int, [_P, _P, _P, _P]),
    "nufi_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "nufi_launch_count": (ctypes.c_int, [_P, _P]),
    "nufi_compute_rho_noalloc": (ctypes.c_int, [_P, _I64, _P, _I64, _I64, _I64, _P, _P]),
}

_lib = None


class NufiError(RuntimeError):
    pass


class NufiOptionsC(ctypes.Structure):
    """Byte-for-byte layout of ``struct nufi_options`` (launch options; every
    field's 0 is the default)."""

    _fields_ = [
        ("split_global_loads", ctypes.c_int32),
        ("split_plain_kick", ctypes.c_int32),
        ("no_persistent", ctypes.c_int32),
        ("split_ctas_per_sm", ctypes.c_int32),
        ("split_threads_per_node", ctypes.c_int32),
        ("batch_no_autotune", ctypes.c_int32),
        ("batch_adjoint_ppt", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 9),
    ]


def options(opts: dict | None):
    """A nufi_options struct from {field: value} (None: all defaults)."""
    o = NufiOptionsC()
    for k, v in (opts or {}).items():
        if k == "reserved" or k not in dict(NufiOptionsC._fields_):
            raise ValueError(f"unknown option {k!r}")
        setattr(o, k, int(v))
    return o


def load(path: Path | None = None):
    """Load the CUDA library (raises if it is absent: there is no CPU path)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m numericalflowiteration_gb300.build`")
    L = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _host_buffer(a: np.ndarray, n: int, what: str):
    """The C ABI takes bare pointers: the array must be contiguous and hold
    at least n values, or the library would read or write past it."""
    if not isinstance(a, np.ndarray) or not a.flags.c_contiguous:
        raise TypeError(f"{what} must be a C-contiguous numpy array")
    if a.size < n:
        raise ValueError(f"{what} holds {a.size} values, the call needs {n}")


def _raise(code: int, msg: str):
    if code == ERR_RANGE:
        raise IndexError(msg)
    if code == ERR_INVALID:
        raise ValueError(msg)
    if code == ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise NufiError(f"[{code}] {msg}")


def plan(cfg, sms: int = 152, opts: dict | None = None) -> dict:
    """The launch plan a Simulation of cfg (with launch options `opts`)
    would choose on a device with `sms` multiprocessors (nufi_plan_ex),
    without touching CUDA."""
    import json
    lib = load()
    c = cfg.to_c()
    o = options(opts)
    buf = ctypes.create_string_buffer(4096)
    st = lib.nufi_plan_ex(ctypes.byref(c), ctypes.byref(o), int(sms), buf, len(buf))
    if st:
        _raise(st, lib.nufi_last_error(None).decode())
    return json.loads(buf.value.decode())


def solve_kernels(cfg) -> np.ndarray:
    """The field solve's circulant kernels for cfg (nufi_solve_kernels), as
    an (nconv, Ns) array, computed on the host."""
    lib = load()
    c = cfg.to_c()
    n = ctypes.c_int32()
    st = lib.nufi_solve_kernels(ctypes.byref(c), None, 0, ctypes.byref(n))
    if st == 0:
        out = np.zeros((n.value, cfg.n_spatial))
        st = lib.nufi_solve_kernels(ctypes.byref(c), _ptr(out), out.size, ctypes.byref(n))
    if st:
        _raise(st, lib.nufi_last_error(None).decode())
    return out


class Simulation:
    """One configuration on one GPU (one CUDA stream).  `opts`: launch
    options (nufi_options fields, e.g. {"no_persistent": 1}); None keeps
    the defaults."""

    def __init__(self, cfg: Config, device: int = 0, opts: dict | None = None):
        self.cfg = cfg
        self._lib = load()
        self._c = cfg.to_c()
        self._o = options(opts)
        h = ctypes.c_void_p()
        st = self._lib.nufi_create_ex(ctypes.byref(self._c), ctypes.byref(self._o), device, ctypes.byref(h))
        if st:
            _raise(st, self._lib.nufi_last_error(None).decode())
        self._h = h
        self.stride_t = cfg.stride_t
        self.n_spatial = cfg.n_spatial
        self.n_points = cfg.n_points
        self._metrics_points = cfg.n_points

    # -- plumbing ---------------------------------------------------------
    def _check(self, st: int):
        if st:
            _raise(st, self._lib.nufi_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.nufi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._check(self._lib.nufi_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    @property
    def launches(self) -> int:
        c = np.zeros(1, dtype=np.int64)
        self._check(self._lib.nufi_launch_count(self._h, _ptr(c)))
        return int(c[0])

    # -- drop-in calls (cuda_kernel / cuda_scheduler) ----------------------
    def compute_rho(self, n: int, q_begin: int = 0, q_end: int | None = None):
        q_end = self.n_points if q_end is None else q_end
        self._check(self._lib.nufi_compute_rho(self._h, n, q_begin, q_end))

    # -- phase-space sampling, history files -------------------------------
    EVAL_FTILDA, EVAL_F, EVAL_PHASE_FLOW = 0, 1, 2

    def eval_points(self, n: int, pts: np.ndarray, mode: int = 1, feet: bool = False):
        """f (mode 1), f~ (mode 0) or the 1D phase flow (mode 2) at points
        pts[i] = (x.., v..); returns f (or None for mode 2) and, if asked,
        the final (x.., v..)."""
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        if pts.ndim != 2 or pts.shape[1] != 2 * self.cfg.dim:
            raise ValueError(f"pts must have shape (npts, {2 * self.cfg.dim})")
        npts = pts.shape[0]
        f = np.zeros(npts) if mode != 2 else None
        ft = np.zeros_like(pts) if (feet or mode == 2) else None
        self._check(self._lib.nufi_eval_points(self._h, n, mode, npts, _ptr(pts), _ptr(f) if f is not None else None,
                                               _ptr(ft) if ft is not None else None))
        return (f, ft) if (feet or mode == 2) else f

    def save_history(self, path: str, n1: int | None = None):
        n1 = self.cfg.Nt if n1 is None else n1
        self._check(self._lib.nufi_save_history(self._h, n1, str(path).encode()))

    def load_history(self, path: str) -> int:
        n = ctypes.c_int64()
        self._check(self._lib.nufi_load_history(self._h, str(path).encode(), ctypes.byref(n)))
        return n.value

    # -- gradient of J = 2 dt sum_n W_n (no reference counterpart) ----------
    def forward(self, n1: int | None = None) -> float:
        """Steps 0..n1 and J = 2 dt sum_{n<=n1} W_n."""
        n1 = self.cfg.Nt if n1 is None else n1
        J = ctypes.c_double()
        self._check(self._lib.nufi_forward(self._h, n1, ctypes.byref(J)))
        return J.value

    def objective(self, n1: int | None = None) -> float:
        n1 = self.cfg.Nt if n1 is None else n1
        J = ctypes.c_double()
        self._check(self._lib.nufi_objective(self._h, n1, ctypes.byref(J)))
        return J.value

    def backward(self, n1: int | None = None) -> np.ndarray:
        """dJ/d(alpha, k, u_b, sigma_b) by the adjoint of the forward run."""
        n1 = self.cfg.Nt if n1 is None else n1
        g = np.zeros(4)
        self._check(self._lib.nufi_backward(self._h, n1, _ptr(g)))
        return g

    def describe(self) -> dict:
        """Kernels and launch shapes this handle chose."""
        import json
        buf = ctypes.create_string_buffer(4096)
        self._check(self._lib.nufi_describe(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def compute_metrics(self, n: int, q_begin: int = 0, q_end: int | None = None):
        """L1 norm, sum w f^2, kinetic energy and entropy of f(n) (eval_f),
        over the metrics grid's points (by default all of them)."""
        q_end = self._metrics_points if q_end is None else q_end
        self._check(self._lib.nufi_compute_metrics(self._h, n, q_begin, q_end))

    def set_metrics_grid(self, metrics_cfg=None):
        """The metrics points on another grid (the reference's conf_metrics):
        its Nx, Nv and domain; None returns to the rho grid."""
        if metrics_cfg is None:
            self._check(self._lib.nufi_set_metrics_grid(self._h, None))
            self._metrics_points = self.n_points
            return
        c = metrics_cfg.to_c()
        self._check(self._lib.nufi_set_metrics_grid(self._h, ctypes.byref(c)))
        self._metrics_points = metrics_cfg.n_points

    def download_metrics(self, metrics: np.ndarray | None = None) -> np.ndarray:
        """metrics += device sums (4 doubles); a new zeroed array if None."""
        m = np.zeros(4) if metrics is None else metrics
        if m.dtype != np.float64 or m.shape != (4,) or not m.flags.c_contiguous:
            raise TypeError("metrics must be a contiguous float64 array of 4")
        self._check(self._lib.nufi_download_metrics(self._h, _ptr(m)))
        return m

    def download_rho(self, rho: np.ndarray) -> np.ndarray:
        """rho += device rho (the caller zeroes it first, as the reference's drivers do)."""
        _host_buffer(rho, self.n_spatial, "rho")
        if rho.dtype == np.float64:
            self._check(self._lib.nufi_download_rho(self._h, _ptr(rho)))
        elif rho.dtype == np.float32:
            self._check(self._lib.nufi_download_rho_f32(self._h, _ptr(rho)))
        else:
            raise TypeError("rho must be float64 or float32")
        return rho

    def upload_phi(self, n: int, coeffs: np.ndarray):
        """Slab n from the history base `coeffs` (slab n at n * stride_t)."""
        if 0 <= n <= self.cfg.Nt:  # other n: the library's range error, before any read
            _host_buffer(coeffs, (n + 1) * self.stride_t, "coeffs")
        if coeffs.dtype == np.float64:
            self._check(self._lib.nufi_upload_phi(self._h, n, _ptr(coeffs)))
        elif coeffs.dtype == np.float32:
            self._check(self._lib.nufi_upload_phi_f32(self._h, n, _ptr(coeffs)))
        else:
            raise TypeError("coeffs must be float64 or float32")

    # -- device-resident stepping ----------------------------------------
    def step(self, n: int) -> float:
        e = np.zeros(1)
        self._check(self._lib.nufi_step(self._h, n, _ptr(e)))
        return float(e[0])

    def step_async(self, n: int):
        self._check(self._lib.nufi_step(self._h, n, None))

    def run(self, n0: int = 0, n1: int | None = None, energy: bool = True):
        n1 = self.cfg.Nt if n1 is None else n1
        if energy:
            e = np.zeros(n1 - n0 + 1)
            self._check(self._lib.nufi_run(self._h, n0, n1, _ptr(e)))
            return e
        self._check(self._lib.nufi_run(self._h, n0, n1, None))
        return None

    def history(self, n0: int = 0, n1: int | None = None, out: np.ndarray | None = None) -> np.ndarray:
        n1 = self.cfg.Nt if n1 is None else n1
        if out is None:
            out = np.zeros((self.cfg.Nt + 1) * self.stride_t)
        if out.dtype != np.float64:
            raise TypeError("out must be float64")
        if 0 <= n0 <= n1 <= self.cfg.Nt:  # other ranges: the library's range error, before any write
            _host_buffer(out, (n1 + 1) * self.stride_t, "out")
        self._check(self._lib.nufi_download_history(self._h, n0, n1, _ptr(out)))
        return out

    def energy(self, n0: int = 0, n1: int | None = None) -> np.ndarray:
        n1 = self.cfg.Nt if n1 is None else n1
        e = np.zeros(n1 - n0 + 1)
        self._check(self._lib.nufi_download_energy(self._h, n0, n1, _ptr(e)))
        return e

    def field_solve(self, rho: np.ndarray):
        r = np.ascontiguousarray(rho, dtype=np.float64)
        _host_buffer(r, self.n_spatial, "rho")
        slab = np.zeros(self.stride_t)
        e = np.zeros(1)
        self._check(self._lib.nufi_field_solve(self._h, _ptr(r), _ptr(slab), _ptr(e)))
        return slab, float(e[0])

    def synchronize(self):
        self._check(self._lib.nufi_synchronize(self._h))


class Batch:
    """Many 1D instances advanced together (nufi_batch_*): one graph launch
    for the whole forward, one for the whole adjoint."""

    def __init__(self, cfgs, device: int = 0, opts: dict | None = None):
        self.cfgs = list(cfgs)
        self._lib = load()
        arr = (NufiConfigC * len(self.cfgs))(*[c.to_c() for c in self.cfgs])
        self._arr = arr
        self._o = options(opts)
        h = ctypes.c_void_p()
        st = self._lib.nufi_batch_create_ex(arr, len(self.cfgs), ctypes.byref(self._o), device, ctypes.byref(h))
        if st:
            _raise(st, self._lib.nufi_batch_last_error(None).decode())
        self._h = h

    def _check(self, st: int):
        if st:
            _raise(st, self._lib.nufi_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.nufi_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.cfgs)

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._check(self._lib.nufi_batch_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def forward(self) -> np.ndarray:
        """All steps of every instance; J_i = 2 dt sum_n W_n."""
        J = np.zeros(len(self.cfgs))
        self._check(self._lib.nufi_batch_forward(self._h, _ptr(J)))
        return J

    def backward(self) -> np.ndarray:
        """dJ_i/d(alpha, k, u_b, sigma_b), shape (count, 4)."""
        g = np.zeros((len(self.cfgs), 4))
        self._check(self._lib.nufi_batch_backward(self._h, _ptr(g)))
        return g

    def energy(self, i: int) -> np.ndarray:
        e = np.zeros(self.cfgs[i].Nt + 1)
        self._check(self._lib.nufi_batch_energy(self._h, i, _ptr(e)))
        return e

    def describe(self) -> dict:
        import json
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self._lib.nufi_batch_describe(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())
