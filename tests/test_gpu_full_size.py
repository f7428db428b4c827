"""GPU parity at the benchmark configurations' own sizes, over their whole
runs, against the reference's own results (tests/golden/make_golden.py
--full: the reference's eval_ftilda / poisson / interpolate loop, built from
its sources).

Measures: max |d| / max |ref| (rel_max) for energy histories, rho and
slabs.  FP64 plain: 1e-12 against the reference run with compensated rho
sums, and within the case's FP64 summation floor (conftest.energy_tol)
against its in-order sums.  FP32-split: the metric's gate, max_n |dW_n| /
max_n |W_n| <= 1e-6 against the reference's energy history; its pointwise
max_n |dW_n| / |W_n| is checked to a looser bound (the energy passes near
zero between its oscillations, where a relative error means little).
"""
import numpy as np
import pytest

from conftest import energy_tol, golden, rel_max

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nufi():
    import numericalflowiteration_gb300 as m
    from numericalflowiteration_gb300 import build
    build.build()
    m.load()
    return m


def _check_run(cfg, g, e, hist, rho_last, tol_comp=1e-12):
    n_last = int(g["n_last"])
    assert rel_max(e, g["energy_comp"][:n_last + 1]) <= tol_comp
    assert rel_max(e, g["energy"][:n_last + 1]) <= max(tol_comp, energy_tol(g))
    st = cfg.stride_t
    for i, n in enumerate(g["slab_steps"]):
        assert rel_max(hist[n * st:(n + 1) * st], g["slabs_comp"][i]) <= 1e-11, f"slab {n}"
    assert rel_max(rho_last, g["rho_comp"][list(g["rho_steps"]).index(n_last)]) <= 1e-12


def test_fp64_two_stream_256x1024_whole_run(nufi):
    """The bench workload (two-stream 256 x 1024, T = 50, all 801 steps) in
    FP64 against the reference's run of the same configuration."""
    cfg, g = golden("two_stream_1d_256x1024_T50")
    with nufi.Simulation(cfg) as sim:
        e = sim.run()
        hist = sim.history()
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
    _check_run(cfg, g, e, hist, rho)


def test_split_two_stream_256x1024_whole_run_within_gate(nufi):
    """The bench's headline form (the FP32-split whole-run kernel) over all
    801 steps against the reference's energy history: the metric's gate."""
    cfg, g = golden("two_stream_1d_256x1024_T50")
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        e = sim.run()
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
    assert rel_max(e, g["energy_comp"]) <= 1e-6
    assert float(np.max(np.abs(e - g["energy_comp"]) / np.abs(g["energy_comp"]))) <= 1e-3
    assert rel_max(rho, g["rho_comp"][-1]) <= 1e-6


def test_split_dropin_two_stream_256x1024_later_steps(nufi):
    """The per-step split trace (the drop-in compute_rho) at late steps on
    the FP64 history (itself pinned to the reference's by the test above):
    rho within the split form's accuracy of the reference's rho."""
    cfg, g = golden("two_stream_1d_256x1024_T50")
    with nufi.Simulation(cfg) as ref:
        ref.run()
        coeffs = ref.history()
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        for n in range(cfg.Nt + 1):
            sim.upload_phi(n, coeffs)
        for n in (400, 600, 800):
            sim.compute_rho(n)
            got = sim.download_rho(np.zeros(cfg.n_spatial))
            assert rel_max(got, g["rho_comp"][list(g["rho_steps"]).index(n)]) <= 1e-6, n


def test_fp64_landau_2d_32x64_whole_run(nufi):
    """The 2D workload (Landau 32^2 x 64^2, T = 20, all 161 steps) in FP64
    against the reference's run of the same configuration."""
    cfg, g = golden("landau_2d_32x64_T20")
    with nufi.Simulation(cfg) as sim:
        e = sim.run()
        hist = sim.history()
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
    _check_run(cfg, g, e, hist, rho)


def test_split_landau_2d_32x64_whole_run_within_gate(nufi):
    """The 2D FP32-split run over all 161 steps against the reference's
    energy history and its last rho: the metric's gate."""
    cfg, g = golden("landau_2d_32x64_T20")
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        e = sim.run()
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
    assert rel_max(e, g["energy_comp"]) <= 1e-6
    assert rel_max(rho, g["rho_comp"][-1]) <= 1e-6


def test_fp64_landau_3d_16x32_first_steps(nufi):
    """The 3D workload at its own size (16^3 x 32^3: 134M points per step)
    over its first 10 steps, FP64, against the reference's run."""
    cfg, g = golden("landau_3d_16x32_n10")
    n_last = int(g["n_last"])
    with nufi.Simulation(cfg) as sim:
        e = sim.run(0, n_last)
        hist = sim.history()
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
    _check_run(cfg, g, e, hist, rho)


def test_split_landau_3d_16x32_first_steps_within_gate(nufi):
    cfg, g = golden("landau_3d_16x32_n10")
    n_last = int(g["n_last"])
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        e = sim.run(0, n_last)
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
    assert rel_max(e, g["energy_comp"][:n_last + 1]) <= 1e-6
    assert rel_max(rho, g["rho_comp"][list(g["rho_steps"]).index(n_last)]) <= 1e-6


def _points_golden():
    """The 3D Landau workload's later steps, pinned on a given history
    (tests/golden/make_points_golden.py): the reference's rho at steps 10,
    50, 100 over all 134M points, and its eval_ftilda at 2^20 seeded points
    (the first 2^16 values exactly, all of them through the sums of 1024
    blocks of 1024 points)."""
    import importlib.util
    from conftest import GOLDEN
    from numericalflowiteration_gb300.config import Config
    spec = importlib.util.spec_from_file_location("make_points_golden", GOLDEN / "make_points_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    z = np.load(GOLDEN / "landau_3d_16x32_points.npz")
    return mod, Config.from_bytes(z["config"].tobytes()), z


def test_fp64_landau_3d_16x32_later_steps_and_points(nufi):
    """FP64 rho at steps 10, 50, 100 of the 16^3 x 32^3 workload (all 134M
    points) and f~ at 2^20 points of phase space, on the history the
    reference's code was evaluated on: 1e-12 (rel_max)."""
    mod, cfg, z = _points_golden()
    hist = np.ascontiguousarray(z["hist32"].astype(np.float64))
    pts = mod.points_3d(int(z["npts"]), int(z["seed"]))
    nb = int(z["block"])
    with nufi.Simulation(cfg) as sim:
        for n in range(cfg.Nt + 1):
            sim.upload_phi(n, hist)
        for i, n in enumerate(z["steps"]):
            sim.compute_rho(int(n))
            rho = sim.download_rho(np.zeros(cfg.n_spatial))
            assert rel_max(rho, z["rho_comp"][i]) <= 1e-12, int(n)
            f = sim.eval_points(int(n), pts, mode=sim.EVAL_FTILDA)
            ne = z["f_exact"].shape[1]
            assert rel_max(f[:ne], z["f_exact"][i]) <= 1e-12, int(n)
            assert rel_max(f.reshape(-1, nb).sum(axis=1), z["f_block_sums"][i]) <= 1e-12, int(n)


def test_split_landau_3d_16x32_later_steps_within_gate(nufi):
    """The FP32-split rho at steps 10, 50, 100 on the same history (its
    tables derived from the uploaded FP64 slabs) against the reference's."""
    mod, cfg, z = _points_golden()
    hist = np.ascontiguousarray(z["hist32"].astype(np.float64))
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        for n in range(cfg.Nt + 1):
            sim.upload_phi(n, hist)
        for i, n in enumerate(z["steps"]):
            sim.compute_rho(int(n))
            rho = sim.download_rho(np.zeros(cfg.n_spatial))
            assert rel_max(rho, z["rho_comp"][i]) <= 1e-6, int(n)
