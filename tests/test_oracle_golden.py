"""The CPU oracle against golden vectors produced by the reference's own
code (tests/golden/make_golden.py runs oracle/_ref/ref_driver, built from
nufi/rho.hpp, fields.hpp, splines.hpp, lsmr.tpp and poisson.cpp).

Tolerances: rho(0) involves only f0 and the point convention and must be
bit-identical; later steps go through the field solve, where the reference
iterates LSMR to machine precision and the oracle solves directly, so they
agree to ~1e-14 and the tests use 1e-12 (max |d| / max |ref|).  Energy
histories are compared the same way, normalised by their maximum (with
alpha = 1e-3 the energy is a difference of O(1) terms and pointwise
relative errors near its minima say nothing about the solver).
"""
import numpy as np
import pytest

from conftest import energy_tol, golden, golden_manifest, rel_max

RUN_CASES_FAST = [
    "small_landau_1d_16x32",
    "small_landau_2d_8x8",
    "small_landau_3d_4x4",
    "order3_landau_1d_32x64",
    "order5_landau_1d_32x64",
    "landau_1d_64x256_T30",
    "bump_on_tail_1d_64x256_T20",
    "two_stream_1d_256x1024_n40",
    "landau_3d_8x8_T2",
    "landau_2d_16x16_T20",
    "ordernd3_landau_2d_8x8",
    "ordernd5_landau_2d_8x8",
    "ordernd3_landau_3d_4x4",
    "ordernd5_landau_3d_4x4",
    "orderhi6_landau_1d_32x64",
    "orderhi7_landau_1d_32x64",
    "orderhi8_landau_1d_32x64",
    "orderhi6_landau_2d_8x8",
    "params_bump_lo_1d_64x256_n60",
    "params_bump_hi_1d_128x512_n40",
    "params_landau_k03_1d_64x256_n60",
]

# Long two-stream run: chaotic after saturation, so agreement is looser
# once the instability has saturated (see test below).
TWO_STREAM_LONG = "two_stream_1d_64x256_T50"


@pytest.mark.parametrize("name", RUN_CASES_FAST)
def test_oracle_run_matches_reference(name, oracle_mod):
    cfg, g = golden(name)
    n_last = int(g["n_last"])
    oracle_mod.set_summation(0)
    energy, rho, coeffs = oracle_mod.run(cfg, 0, n_last)
    assert rel_max(energy, g["energy"]) <= energy_tol(g)
    for i, n in enumerate(g["rho_steps"]):
        assert rel_max(rho[n], g["rho"][i]) <= 1e-12, f"rho step {n}"
    assert np.array_equal(rho[0], g["rho"][0]), "rho(0) must be bit-identical (f0 + point convention)"
    st = cfg.stride_t
    for i, n in enumerate(g["slab_steps"]):
        assert rel_max(coeffs[n * st:(n + 1) * st], g["slabs"][i]) <= 1e-11, f"slab {n}"


def test_oracle_two_stream_long(oracle_mod):
    """Linear phase to the alpha = 1e-3 summation floor (energy_tol); through
    saturation the two codes stay within 1e-9 of the peak energy (rounding
    differences are amplified by the instability, as between any two FP64
    implementations)."""
    cfg, g = golden(TWO_STREAM_LONG)
    energy, rho, _ = oracle_mod.run(cfg, 0, int(g["n_last"]), keep_rho=True)
    e_ref = g["energy"]
    assert rel_max(energy[:200], e_ref[:200]) <= max(2e-12, energy_tol(g))
    assert rel_max(energy, e_ref) <= 1e-9
    assert np.array_equal(rho[0], g["rho"][0])


@pytest.mark.parametrize("name", ["small_landau_1d_16x32", "two_stream_1d_256x1024_n40", "landau_3d_8x8_T2"])
def test_compensated_oracle_matches_compensated_reference(name, oracle_mod):
    """Both sides summing rho compensated: only the field-solve methods
    differ (LSMR vs direct), so the histories agree to 1e-12."""
    cfg, g = golden(name)
    oracle_mod.set_summation(1)
    try:
        energy, rho, _ = oracle_mod.run(cfg, 0, int(g["n_last"]))
    finally:
        oracle_mod.set_summation(0)
    assert rel_max(energy, g["energy_comp"]) <= 1e-12
    for i, n in enumerate(g["rho_steps"]):
        assert rel_max(rho[n], g["rho_comp"][i]) <= 1e-12


@pytest.mark.parametrize("name", ["solve_1d_64", "solve_1d_256", "solve_2d_32", "solve_3d_16",
                                  "solve_1d_64_order3", "solve_1d_64_order5", "solve_2d_256", "solve_3d_32"])
def test_oracle_field_solve_matches_reference(name, oracle_mod):
    cfg, g = golden(name)
    slab, e = oracle_mod.field_solve(cfg, g["rho"])
    assert rel_max(slab, g["slab"]) <= 1e-12
    assert abs(e - float(g["energy"])) <= 1e-13 * abs(float(g["energy"]))


def test_oracle_poisson_known_answer(oracle_mod):
    """bin/test_poisson.cpp:36-119: rho = cos2z + sin8y + cos42x on 128x64x32
    over [0, 2pi)^3; the reference prints a relative l1 error of ~4e-15."""
    from numericalflowiteration_gb300.config import Config
    cfg = Config(3, [128, 64, 32], [1, 1, 1], 0, 1.0, [0.0] * 3, [2 * np.pi] * 3, [0.0] * 3, [1.0] * 3)
    dx = 2 * np.pi / np.array([128, 64, 32])
    z, y, x = np.meshgrid(np.arange(32) * dx[2], np.arange(64) * dx[1], np.arange(128) * dx[0], indexing="ij")
    rho = np.cos(2 * z) + np.sin(8 * y) + np.cos(42 * x)
    phi = np.cos(2 * z) / 4 + np.sin(8 * y) / 64 + np.cos(42 * x) / (42 * 42)
    out, _ = oracle_mod.poisson(cfg, rho.ravel())
    err = np.sum(np.abs(out - phi.ravel())) / np.sum(np.abs(phi))
    ref = golden_manifest()["kat"]["test_poisson_rel_l1"]["double"]
    assert err < 1e-13 and ref < 1e-13


def test_oracle_fields_known_answer(oracle_mod):
    """bin/test_fields.cpp:129-190: interpolate sin3x + sin3y on 128x128 and
    evaluate back at the nodes (the reference's max error is ~1.6e-14)."""
    from numericalflowiteration_gb300.config import Config
    cfg = Config(2, [128, 128], [1, 1], 0, 1.0, [0.0, -np.pi], [4 * np.pi, np.pi], [0.0] * 2, [1.0] * 2)
    dx, dy = 4 * np.pi / 128, 2 * np.pi / 128
    j, i = np.meshgrid(np.arange(128), np.arange(128), indexing="ij")
    x, y = i * dx, -np.pi + j * dy
    vals = np.sin(3 * x) + np.sin(3 * y)
    slab = oracle_mod.interpolate(cfg, vals.ravel())
    pts = np.stack([x.ravel(), y.ravel()], axis=1)
    back = oracle_mod.eval_field(cfg, slab, pts)
    err = np.max(np.abs(back - vals.ravel()))
    ref = golden_manifest()["kat"]["test_fields_2d"]["max_node_error_2d"]
    assert err < 1e-12 and ref < 1e-12


def test_oracle_spline_known_answers(oracle_mod):
    """nufi/splines.hpp:39-110 on a 1D grid with dx = 1: at a node the
    order-4 window weights are N4(0) = [1/6, 2/3, 1/6, 0]; at the cell
    midpoint the coefficients e1 = [0, 1, 0, 0] give eval<4,0>(0.5) =
    0.47916666666666663 and eval<4,1>(0.5) = -0.625 (values the reference's
    own functions print)."""
    from numericalflowiteration_gb300.config import Config
    N = 16
    cfg = Config(1, [N], [1], 0, 1.0, [0.0], [float(N)], [0.0], [1.0])
    i = 5
    node = np.array([[float(i)]])
    weights = []
    for j in range(4):
        slab = np.zeros(N + 3)
        slab[i + j] = 1.0
        weights.append(oracle_mod.eval_field(cfg, slab, node)[0])
    assert weights == [0.16666666666666666, 0.66666666666666663, 0.16666666666666666, 0.0]
    slab = np.zeros(N + 3)
    slab[i + 1] = 1.0
    mid = np.array([[i + 0.5]])
    assert oracle_mod.eval_field(cfg, slab, mid)[0] == 0.47916666666666663
    assert oracle_mod.eval_field(cfg, slab, mid, deriv=(1, 0, 0))[0] == -0.625


@pytest.mark.parametrize("case", ["landau_1d", "two_stream_1d", "landau_2d", "landau_3d"])
def test_oracle_initial_energy_known_answer(case, oracle_mod):
    """The field energy at t = 0 of f0 = (1 + a sum_i cos k x_i) g(v) with
    unit-mass g: E_i = (a/k) sin k x_i, so 1/2 int |E|^2 = 1/2 d (a/k)^2
    L^(d-1) L/2.  The velocity midpoint sum of g is exact to rounding on
    [-10, 10] and [-8, 8]; on [-6, 6]^3 the truncated Gaussian's missing
    mass (2e-9 per axis) sets the 3D tolerance."""
    from numericalflowiteration_gb300 import config
    cfg, tol = {"landau_1d": (config.landau_1d(Nt=1), 1e-12),
                "two_stream_1d": (config.two_stream_1d(Nx=64, Nv=256, Nt=1), 1e-12),
                "landau_2d": (config.landau_2d(Nx=16, Nv=32, Nt=1), 1e-12),
                "landau_3d": (config.landau_3d(Nx=8, Nv=16, Nt=1), 2e-8)}[case]
    a, k = cfg.f0_params[0], cfg.f0_params[1]
    L = cfg.x_max[0] - cfg.x_min[0]
    d = cfg.dim
    expect = 0.5 * d * (a / k) ** 2 * L ** (d - 1) * L / 2
    energy, _, _ = oracle_mod.run(cfg, 0, 0)
    assert abs(energy[0] - expect) <= tol * expect, (energy[0], expect)


def _ref_driver():
    from conftest import ROOT
    drv = ROOT / "oracle" / "_ref" / "ref_driver"
    if not drv.exists():
        pytest.skip("no reference build in oracle/_ref")
    return drv


@pytest.mark.parametrize("dim,order", [(1, o) for o in range(3, 9)] + [(2, o) for o in (3, 4, 5, 6)] +
                         [(3, o) for o in (3, 4, 5)])
def test_oracle_rho_bit_identical_to_reference_build(dim, order, oracle_mod, tmp_path):
    """rho of the oracle and of the reference's own eval_ftilda (its headers
    compiled by oracle/ref/Makefile, `ref_driver rho`) on the same seeded
    random history, every spline order each dimension takes: equal to the
    last bit (the same operations in the same order, -ffp-contract=off)."""
    import subprocess
    from numericalflowiteration_gb300.config import landau_1d, landau_2d, landau_3d
    drv = _ref_driver()
    cfg = {1: lambda: landau_1d(Nx=32, Nv=64, Nt=9, order=order),
           2: lambda: landau_2d(Nx=8, Nv=8, Nt=5, order=order),
           3: lambda: landau_3d(Nx=4, Nv=4, Nt=4, order=order)}[dim]()
    rng = np.random.default_rng(100 + 10 * dim + order)
    hist = 1e-2 * rng.standard_normal((cfg.Nt + 1) * cfg.stride_t)
    p = tmp_path / "c"
    p.with_suffix(".cfg").write_bytes(cfg.to_bytes())
    hist.tofile(str(p) + ".hist")
    oracle_mod.set_summation(0)
    for n in (1, cfg.Nt):
        subprocess.run([str(drv), "rho", str(p.with_suffix(".cfg")), str(p) + ".hist", str(n), str(p), "1"],
                       check=True, capture_output=True)
        ref = np.fromfile(str(p) + ".rho")
        got = oracle_mod.rho(cfg, n, hist)
        assert np.array_equal(got, ref), (n, float(np.max(np.abs(got - ref))))


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_f0_kinds_bit_identical_to_the_references_compiled_f0(dim, oracle_mod, tmp_path):
    """The reference hard-codes one f0 per dimension (nufi/config.hpp: 1D
    u^2 M two-stream with alpha = 0.01, k = 0.5; 2D Landau with alpha = k =
    0.5; 3D bump-on-tail with alpha = 0.03, k = 0.3, u_b = 4.5, sigma_b =
    0.5).  `ref_driver_native` keeps those compiled-in functions; the f0
    kinds with these parameters must give its rho to the last bit: at step 0
    (f0 alone at the grid points) and after traced steps."""
    import subprocess
    from conftest import ROOT
    from numericalflowiteration_gb300.config import bump_on_tail_3d, landau_2d, two_stream_1d
    drv = ROOT / "oracle" / "_ref" / "ref_driver_native"
    if not drv.exists():
        pytest.skip("no reference build in oracle/_ref")
    cfg = {1: lambda: two_stream_1d(Nx=32, Nv=64, Nt=9, alpha=0.01, k=0.5),
           2: lambda: landau_2d(Nx=8, Nv=8, Nt=5, alpha=0.5, k=0.5),
           3: lambda: bump_on_tail_3d(Nx=4, Nv=6, Nt=4)}[dim]()
    rng = np.random.default_rng(300 + dim)
    hist = 1e-2 * rng.standard_normal((cfg.Nt + 1) * cfg.stride_t)
    p = tmp_path / "c"
    p.with_suffix(".cfg").write_bytes(cfg.to_bytes())
    hist.tofile(str(p) + ".hist")
    oracle_mod.set_summation(0)
    for n in (0, 1, cfg.Nt):
        subprocess.run([str(drv), "rho", str(p.with_suffix(".cfg")), str(p) + ".hist", str(n), str(p), "1"],
                       check=True, capture_output=True)
        ref = np.fromfile(str(p) + ".rho")
        got = oracle_mod.rho(cfg, n, hist)
        assert np.any(ref != 0) and np.array_equal(got, ref), (n, float(np.max(np.abs(got - ref))))


@pytest.mark.parametrize("dim,order", [(1, 4), (1, 6), (1, 3), (2, 4), (2, 5), (3, 4), (3, 3)])
def test_oracle_points_bit_identical_to_reference_build(dim, order, oracle_mod, tmp_path):
    """eval_ftilda and eval_f at arbitrary points (the sampling path), and
    in 1D eval_phase_flow (the eval_f trajectory only when n > 1, then
    x - L floor(x / L), nufi/rho.hpp:98-131), of the oracle and of the
    reference's own functions (`ref_driver points`), on a seeded random
    history and points partly outside the domain: equal to the last bit."""
    import subprocess
    from numericalflowiteration_gb300.config import landau_1d, landau_2d, landau_3d
    drv = _ref_driver()
    cfg = {1: lambda: landau_1d(Nx=32, Nv=64, Nt=9, order=order),
           2: lambda: landau_2d(Nx=8, Nv=8, Nt=5, order=order),
           3: lambda: landau_3d(Nx=4, Nv=4, Nt=4, order=order)}[dim]()
    rng = np.random.default_rng(200 + 10 * dim + order)
    hist = 1e-2 * rng.standard_normal((cfg.Nt + 1) * cfg.stride_t)
    lo = np.array(list(cfg.x_min[:dim]) + list(cfg.v_min[:dim]))
    hi = np.array(list(cfg.x_max[:dim]) + list(cfg.v_max[:dim]))
    span = hi - lo
    pts = lo - 0.5 * span + 2.0 * span * rng.random((300, 2 * dim))
    p = tmp_path / "c"
    p.with_suffix(".cfg").write_bytes(cfg.to_bytes())
    hist.tofile(str(p) + ".hist")
    pts.tofile(str(p) + ".in")

    def ref(n, mode):
        subprocess.run([str(drv), "points", str(p.with_suffix(".cfg")), str(p) + ".hist", str(n), str(mode),
                        str(p) + ".in", str(p)], check=True, capture_output=True)
        return np.fromfile(str(p) + ".f"), np.fromfile(str(p) + ".pts").reshape(pts.shape)

    for n in (0, 1, 2, cfg.Nt):
        for mode in (0, 1):
            got = oracle_mod.eval_points(cfg, n, hist, pts, mode=mode)
            want, _ = ref(n, mode)
            assert np.array_equal(got, want), (n, mode, float(np.max(np.abs(got - want))))
        if dim == 1:
            _, flow = ref(n, 2)
            feet = oracle_mod.eval_points(cfg, n, hist, pts, mode=1, feet=True)[1] if n > 1 else pts.copy()
            L = cfg.x_max[0] - cfg.x_min[0]
            feet[:, 0] = feet[:, 0] - L * np.floor(feet[:, 0] * (1.0 / L))
            assert np.array_equal(feet, flow), n


def test_oracle_q_range_partition(oracle_mod):
    """rho over a split q range adds up to rho over the whole range, as the
    reference's multi-device split relies on (nufi/cuda_scheduler.hpp:88-118)."""
    cfg, g = golden("small_landau_1d_16x32")
    coeffs = np.zeros((cfg.Nt + 1) * cfg.stride_t)
    st = cfg.stride_t
    for i, n in enumerate(g["slab_steps"]):
        coeffs[n * st:(n + 1) * st] = g["slabs"][i]
    n = 7
    full = oracle_mod.rho(cfg, n, coeffs)
    cuts = [0, 37, 200, cfg.n_points]
    parts = sum(oracle_mod.rho(cfg, n, coeffs, a, b) for a, b in zip(cuts[:-1], cuts[1:]))
    assert rel_max(parts, full) <= 1e-14
    assert rel_max(full, g["rho"][n]) <= 1e-12


METRICS_CASES = ["metrics_small_landau_1d_16x32", "metrics_landau_1d_64x256_T30", "metrics_two_stream_1d_64x256_T50",
                 "metrics_bump_on_tail_1d_64x256_n80", "metrics_order5_landau_1d_32x64",
                 "metrics_small_landau_2d_8x8", "metrics_landau_2d_16x16_n40", "metrics_small_landau_3d_4x4",
                 "metrics_landau_3d_8x8_T2"]


@pytest.mark.parametrize("name", METRICS_CASES)
def test_oracle_metrics_match_reference(name, oracle_mod):
    """eval_f metrics (L1, sum f^2, kinetic energy, entropy) of the oracle on
    the reference's own history against the reference's eval_f metrics:
    both sum per node in q order and then over the nodes in order, so they
    agree to the last bit."""
    cfg, g = golden(name)
    hist = np.ascontiguousarray(g["slabs"].reshape(-1))
    for n, ref in zip(g["steps"], g["metrics"]):
        got = oracle_mod.metrics(cfg, int(n), hist)
        assert np.array_equal(got, ref), (int(n), got, ref)


@pytest.mark.parametrize("f0", ["landau", "two_stream", "bump_on_tail"])
def test_oracle_forward_mode_matches_central_differences(f0, oracle_mod):
    """The FP64 forward-mode derivative of J = 2 dt sum W_n (the check of the
    GPU adjoint) against central differences (h = 1e-6) of the oracle's own
    loop, per component to 1e-5 relative."""
    from numericalflowiteration_gb300.config import bump_on_tail_1d, landau_1d, two_stream_1d
    cfg = {"landau": landau_1d(Nx=16, Nv=32, Nt=10), "two_stream": two_stream_1d(Nx=16, Nv=64, Nt=10),
           "bump_on_tail": bump_on_tail_1d(Nx=16, Nv=64, Nt=12)}[f0]
    J, dJ = oracle_mod.objective_tangent(cfg)
    assert J == pytest.approx(oracle_mod.objective(cfg), rel=1e-13)
    h = 1e-6
    for i in range(4 if f0 == "bump_on_tail" else 2):
        Js = []
        for sgn in (1, -1):
            pp = list(cfg.f0_params)
            pp[i] += sgn * h
            Js.append(oracle_mod.objective(cfg.replace(f0_params=pp)))
        fd = (Js[0] - Js[1]) / (2 * h)
        assert abs(dJ[i] - fd) <= 1e-5 * abs(fd), (i, dJ[i], fd)
    if f0 != "bump_on_tail":
        assert dJ[2] == 0 and dJ[3] == 0
