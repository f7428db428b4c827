"""(CPU) The field solve's circulant kernels (nufi_solve_kernels: the
host-side long-double DFTs nufi_create uploads) applied in numpy to the
reference's own field-solve cases: the spline slab and W against the
reference's DHT Poisson + LSMR collocation (tests/golden/solve_*.npz,
from nufi/poisson.cpp and nufi/fields.hpp), including orders 3 and 5,
where the collocation symbol vanishes at the Nyquist mode and the
minimum-norm solution drops it.  The 1D FP32-split rows K A, K B, K C
against their definition from c."""
import numpy as np
import pytest

from conftest import golden, rel_max

from numericalflowiteration_gb300 import _lib, solve_kernels


@pytest.fixture(scope="module", autouse=True)
def lib():
    from numericalflowiteration_gb300 import build
    build.build()
    return _lib.load()


def circ(G, r, shape):
    """out[i] = sum_j G[i - j] r[j], periodic per axis (x fastest)."""
    Gs, rs = G.reshape(shape[::-1]), r.reshape(shape[::-1])
    return np.real(np.fft.ifftn(np.fft.fftn(Gs) * np.fft.fftn(rs))).ravel()


@pytest.mark.parametrize("name", ["solve_1d_64", "solve_1d_256", "solve_2d_32", "solve_3d_16",
                                  "solve_1d_64_order3", "solve_1d_64_order5", "solve_2d_256", "solve_3d_32"])
def test_kernels_reproduce_the_reference_solve(name):
    cfg, g = golden(name)
    G = solve_kernels(cfg)
    assert G.shape == (2, cfg.n_spatial)
    rho = g["rho"] - np.mean(g["rho"])
    shape = list(cfg.Nx)
    c = circ(G[0], rho, shape)
    phi = circ(G[1], rho, shape)
    pad = [(0, cfg.order - 1)] * cfg.dim
    slab = np.pad(c.reshape(shape[::-1]), pad, mode="wrap").ravel()
    assert rel_max(slab, g["slab"]) <= 1e-12
    L = np.prod([b - a for a, b in zip(cfg.x_min, cfg.x_max)])
    W = L / (2 * cfg.n_spatial) * np.dot(rho, phi)
    assert abs(W - float(g["energy"])) <= 1e-12 * abs(float(g["energy"]))
    # the kernels sum to zero (the mean mode is dropped)
    assert abs(G[0].sum()) <= 1e-12 * np.abs(G[0]).max() * cfg.n_spatial


@pytest.mark.parametrize("name", ["solve_1d_64", "solve_1d_256"])
def test_split_rows_are_the_cell_quadratic(name):
    """K A_i = K/2 (c[i+2] - c[i]), K B_i = K (c[i] - 2 c[i+1] + c[i+2]),
    K C_i = K/2 (-c[i] + 3 c[i+1] - 3 c[i+2] + c[i+3]), K = -dt^2/dx^2:
    the kick of one substep over cell i as a quadratic in the cell
    coordinate, from the order-4 spline derivative."""
    cfg, g = golden(name)
    G = solve_kernels(cfg.replace(precision="fp32split"))
    assert G.shape == (5, cfg.n_spatial)
    assert np.array_equal(G[:2], solve_kernels(cfg))
    rho = g["rho"] - np.mean(g["rho"])
    shape = list(cfg.Nx)
    c = circ(G[0], rho, shape)
    s = [np.roll(c, -m) for m in range(4)]
    dx = (cfg.x_max[0] - cfg.x_min[0]) / cfg.Nx[0]
    K = -cfg.dt ** 2 / dx ** 2
    want = [K / 2 * (s[2] - s[0]), K * (s[0] - 2 * s[1] + s[2]), K / 2 * (-s[0] + 3 * s[1] - 3 * s[2] + s[3])]
    for r, w in zip(G[2:], want):
        assert rel_max(circ(r, rho, shape), w) <= 1e-11


def test_kernel_errors():
    from numericalflowiteration_gb300.config import landau_1d
    with pytest.raises(NotImplementedError):
        solve_kernels(landau_1d(Nx=20000, Nv=8, Nt=2))  # above 16384 nodes with an axis above 4096
