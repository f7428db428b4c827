"""ctypes mirror of ``nufi_config`` (include/nufi_gb300.h) and the named
workloads of the NuFI hot path.

The reference keeps its configuration as compile-time ``config_t`` structs
whose constructors derive the grid quantities (nufi/config.hpp:55-70,
117-138, 196-219) and whose ``f0`` is hard-coded; here every field is a
runtime value and f0 is chosen by kind + parameters.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Sequence

PREC_FP64 = 0
PREC_FP32_SPLIT = 1

F0_LANDAU = 0
F0_TWO_STREAM = 1
F0_BUMP_ON_TAIL = 2

_PREC_NAMES = {"fp64": PREC_FP64, "fp32split": PREC_FP32_SPLIT, "fp32-split": PREC_FP32_SPLIT}
_F0_NAMES = {"landau": F0_LANDAU, "two_stream": F0_TWO_STREAM, "bump_on_tail": F0_BUMP_ON_TAIL}


class NufiConfigC(ctypes.Structure):
    """Byte-for-byte layout of ``struct nufi_config``."""

    _fields_ = [
        ("dim", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("f0_kind", ctypes.c_int32),
        ("Nx", ctypes.c_int64 * 3),
        ("Nv", ctypes.c_int64 * 3),
        ("Nt", ctypes.c_int64),
        ("dt", ctypes.c_double),
        ("x_min", ctypes.c_double * 3),
        ("x_max", ctypes.c_double * 3),
        ("v_min", ctypes.c_double * 3),
        ("v_max", ctypes.c_double * 3),
        ("f0_params", ctypes.c_double * 8),
    ]


@dataclass
class Config:
    """One NuFI run: grid, domain, time stepping, f0 and precision."""

    dim: int
    Nx: Sequence[int]
    Nv: Sequence[int]
    Nt: int
    dt: float
    x_min: Sequence[float]
    x_max: Sequence[float]
    v_min: Sequence[float]
    v_max: Sequence[float]
    f0: str = "landau"
    f0_params: Sequence[float] = field(default_factory=lambda: [0.01, 0.5])
    order: int = 4
    precision: str = "fp64"

    def replace(self, **kw) -> "Config":
        d = dict(self.__dict__)
        d.update(kw)
        return Config(**d)

    # -- derived sizes ---------------------------------------------------
    @property
    def n_spatial(self) -> int:
        return int(math.prod(self.Nx[: self.dim]))

    @property
    def n_velocity(self) -> int:
        return int(math.prod(self.Nv[: self.dim]))

    @property
    def n_points(self) -> int:
        return self.n_spatial * self.n_velocity

    @property
    def stride_t(self) -> int:
        return int(math.prod(n + self.order - 1 for n in self.Nx[: self.dim]))

    def point_steps(self, n0: int = 0, n1: int | None = None) -> int:
        """Backtraced point-steps of steps n0..n1: sum_n Nq * n."""
        n1 = self.Nt if n1 is None else n1
        return self.n_points * (n1 * (n1 + 1) // 2 - (n0 - 1) * n0 // 2)

    def to_c(self) -> NufiConfigC:
        c = NufiConfigC()
        c.dim = self.dim
        c.order = self.order
        c.precision = _PREC_NAMES[self.precision] if isinstance(self.precision, str) else int(self.precision)
        c.f0_kind = _F0_NAMES[self.f0] if isinstance(self.f0, str) else int(self.f0)
        for a in range(3):
            inside = a < self.dim
            c.Nx[a] = int(self.Nx[a]) if inside else 1
            c.Nv[a] = int(self.Nv[a]) if inside else 1
            c.x_min[a] = float(self.x_min[a]) if inside else 0.0
            c.x_max[a] = float(self.x_max[a]) if inside else 1.0
            c.v_min[a] = float(self.v_min[a]) if inside else 0.0
            c.v_max[a] = float(self.v_max[a]) if inside else 1.0
        c.Nt = int(self.Nt)
        c.dt = float(self.dt)
        for i in range(8):
            c.f0_params[i] = float(self.f0_params[i]) if i < len(self.f0_params) else 0.0
        return c

    def to_bytes(self) -> bytes:
        return bytes(self.to_c())

    @staticmethod
    def from_c(c: NufiConfigC) -> "Config":
        d = int(c.dim)
        inv_prec = {PREC_FP64: "fp64", PREC_FP32_SPLIT: "fp32split"}
        inv_f0 = {v: k for k, v in _F0_NAMES.items()}
        return Config(d, [int(c.Nx[a]) for a in range(d)], [int(c.Nv[a]) for a in range(d)], int(c.Nt),
                      float(c.dt), [float(c.x_min[a]) for a in range(d)], [float(c.x_max[a]) for a in range(d)],
                      [float(c.v_min[a]) for a in range(d)], [float(c.v_max[a]) for a in range(d)],
                      inv_f0[int(c.f0_kind)], [float(c.f0_params[i]) for i in range(8)], int(c.order),
                      inv_prec[int(c.precision)])

    @staticmethod
    def from_bytes(b: bytes) -> "Config":
        return Config.from_c(NufiConfigC.from_buffer_copy(bytes(b)))


FOUR_PI = 4.0 * math.pi


def landau_1d(Nx=64, Nv=256, Nt=480, dt=1.0 / 16, alpha=0.01, k=0.5, **kw) -> Config:
    """1D1V weak Landau damping: f0 = (1 + a cos kx) exp(-v^2/2)/sqrt(2 pi),
    x in [0, 4 pi), v in [-10, 10]; defaults are the 64 x 256, T = 30 run."""
    return Config(1, [Nx], [Nv], Nt, dt, [0.0], [FOUR_PI], [-10.0], [10.0], "landau", [alpha, k], **kw)


def two_stream_1d(Nx=256, Nv=1024, Nt=800, dt=1.0 / 16, alpha=0.001, k=0.5, **kw) -> Config:
    """1D1V two-stream instability: f0 = (1 + a cos kx) v^2 exp(-v^2/2)/sqrt(2 pi),
    x in [0, 4 pi), v in [-10, 10]; defaults are the 256 x 1024, T = 50 run."""
    return Config(1, [Nx], [Nv], Nt, dt, [0.0], [FOUR_PI], [-10.0], [10.0], "two_stream", [alpha, k], **kw)


def bump_on_tail_1d(Nx=64, Nv=256, Nt=320, dt=1.0 / 16, alpha=0.03, k=0.4, u_b=4.5, sigma_b=0.5,
                    v_lim=10.0, **kw) -> Config:
    """1D1V bump-on-tail: f0 = (1 + a cos kx)[0.9 N(v;0,1) + 0.1 N(v;u_b,s_b)],
    x in [0, 2 pi / k), v in [-v_lim, v_lim]."""
    L = 2.0 * math.pi / k
    return Config(1, [Nx], [Nv], Nt, dt, [0.0], [L], [-v_lim], [v_lim], "bump_on_tail",
                  [alpha, k, u_b, sigma_b], **kw)


def bump_on_tail_3d(Nx=8, Nv=8, Nt=50, dt=0.1, alpha=0.03, k=0.3, u_b=4.5, sigma_b=0.5, v_min=-9.0, v_max=0.0,
                    **kw) -> Config:
    """3D3V bump-on-tail, the reference's compiled-in 3D configuration
    (nufi/config.hpp: 8^3 x 8^3, dt = 0.1, T = 5, x in [0, 20 pi / 3)^3,
    v in [-9, 0]^3): f0 = (1 + a sum_d cos k x_d)[0.9 N(u;0,1) +
    0.1 N(u;u_b,s_b)] N(v;0,1) N(w;0,1).  FP64 form only."""
    L = 2.0 * math.pi / k
    return Config(3, [Nx] * 3, [Nv] * 3, Nt, dt, [0.0] * 3, [L] * 3, [v_min] * 3, [v_max] * 3, "bump_on_tail",
                  [alpha, k, u_b, sigma_b], **kw)


def landau_2d(Nx=32, Nv=64, Nt=160, dt=1.0 / 8, alpha=0.01, k=0.5, **kw) -> Config:
    """2D2V weak Landau damping: x in [0, 4 pi)^2, v in [-8, 8]^2; defaults
    are the 32^2 x 64^2, T = 20 run (4.2M points)."""
    return Config(2, [Nx, Nx], [Nv, Nv], Nt, dt, [0.0, 0.0], [FOUR_PI] * 2, [-8.0] * 2, [8.0] * 2,
                  "landau", [alpha, k], **kw)


def landau_3d(Nx=16, Nv=32, Nt=100, dt=0.1, alpha=0.01, k=0.5, **kw) -> Config:
    """3D3V weak Landau damping: x in [0, 4 pi)^3, v in [-6, 6]^3; defaults
    are the 16^3 x 32^3, T = 10 run (134M points per step)."""
    return Config(3, [Nx] * 3, [Nv] * 3, Nt, dt, [0.0] * 3, [FOUR_PI] * 3, [-6.0] * 3, [6.0] * 3,
                  "landau", [alpha, k], **kw)


def batched_bump_on_tail(count=256, seed=20261203, Nt=320, dt=1.0 / 16, nx=(64, 128, 256), nv=(256, 512, 1024),
                         precision="fp64", **kw):
    """The batched adjoint configuration: `count` bump-on-tail instances
    with seeded uniform alpha in [0.01, 0.05], k in [0.3, 0.5], u_b in
    [4, 5], sigma_b in [0.4, 0.6] and grid sizes drawn from nx x nv
    (dt = 1/16, T = 20)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        a = float(rng.uniform(0.01, 0.05))
        k = float(rng.uniform(0.3, 0.5))
        ub = float(rng.uniform(4.0, 5.0))
        sb = float(rng.uniform(0.4, 0.6))
        Nx = int(rng.choice(nx))
        Nv = int(rng.choice(nv))
        out.append(bump_on_tail_1d(Nx=Nx, Nv=Nv, Nt=Nt, dt=dt, alpha=a, k=k, u_b=ub, sigma_b=sb,
                                   precision=precision, **kw))
    return out


WORKLOADS = {
    "landau_1d_64x256_T30": landau_1d,
    "two_stream_1d_256x1024_T50": two_stream_1d,
    "landau_2d_32x64_T20": landau_2d,
    "landau_3d_16x32_T10": landau_3d,
}
