"""Phase-space sampling (nufi_eval_points: eval_f, eval_ftilda and the 1D
eval_phase_flow) against the oracle on the reference's own histories, and
the coefficient history on disk: save / load round trip, resuming a run from
a loaded history, and files without the header (the 1D driver's dumps)."""
import numpy as np
import pytest

from conftest import golden, rel_max

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nufi():
    import numericalflowiteration_gb300 as m
    from numericalflowiteration_gb300 import build
    build.build()
    m.load()
    return m


def _pts(cfg, count, seed):
    rng = np.random.default_rng(seed)
    d = cfg.dim
    lo = np.array(list(cfg.x_min[:d]) + list(cfg.v_min[:d]))
    hi = np.array(list(cfg.x_max[:d]) + list(cfg.v_max[:d]))
    return lo + (hi - lo) * rng.random((count, 2 * d))


@pytest.mark.parametrize("name", ["metrics_landau_1d_64x256_T30", "metrics_small_landau_2d_8x8",
                                  "metrics_small_landau_3d_4x4", "metrics_two_stream_1d_64x256_T50"])
@pytest.mark.parametrize("mode", [0, 1])
def test_eval_points_match_oracle(nufi, oracle_mod, name, mode):
    """f and f~ at random points (FP64, tolerance 1e-12 of max)."""
    cfg, g = golden(name)
    hist = np.ascontiguousarray(g["slabs"].reshape(-1))
    pts = _pts(cfg, 2000, 3)
    n = int(g["n_last"])
    with nufi.Simulation(cfg) as sim:
        for k in range(n + 1):
            sim.upload_phi(k, hist)
        f, feet = sim.eval_points(n, pts, mode=mode, feet=True)
    ref, ref_feet = oracle_mod.eval_points(cfg, n, hist, pts, mode=mode, feet=True)
    assert rel_max(f, ref) <= 1e-12
    assert rel_max(feet, ref_feet) <= 1e-12


def test_phase_flow_matches_reference_semantics(nufi, oracle_mod):
    """eval_phase_flow: the eval_f trajectory only when n > 1, then x
    wrapped as x - L floor(x / L) (nufi/rho.hpp:98-131)."""
    cfg, g = golden("metrics_landau_1d_64x256_T30")
    hist = np.ascontiguousarray(g["slabs"].reshape(-1))
    pts = _pts(cfg, 1000, 5)
    L = cfg.x_max[0] - cfg.x_min[0]
    with nufi.Simulation(cfg) as sim:
        for k in range(int(g["n_last"]) + 1):
            sim.upload_phi(k, hist)
        for n in (0, 1, 2, 100):
            _, flow = sim.eval_points(n, pts, mode=2)
            ref = oracle_mod.eval_points(cfg, n, hist, pts, mode=1, feet=True)[1] if n > 1 else pts.copy()
            ref[:, 0] = ref[:, 0] - L * np.floor(ref[:, 0] / L)
            assert rel_max(flow, ref) <= 1e-12, n


def test_history_round_trip_and_resume(nufi, tmp_path):
    """save_history writes the reference's text layout; a fresh handle that
    loads it and runs the remaining steps reproduces the straight run bit
    for bit (17 significant digits carry every FP64 value exactly)."""
    from numericalflowiteration_gb300.config import landau_1d
    cfg = landau_1d(Nx=32, Nv=64, Nt=60)
    with nufi.Simulation(cfg) as a:
        e_all = a.run()
        a.save_history(tmp_path / "h.txt", 30)
        hist = a.history()
    text = (tmp_path / "h.txt").read_text().splitlines()
    # the reference's header: the configuration's Nt, dt as std::to_string
    assert text[0] == "Nt = 60" and text[1] == "dt = 0.062500" and text[2] == "Nx = 32"
    assert text[5] == "order = 4" and text[6] == ""
    # all Nt + 1 slabs, as the reference's reader takes; zeros after step 30
    assert len(text) == 7 + 61 * cfg.stride_t
    assert all(v == "0" for v in text[7 + 31 * cfg.stride_t:])
    with nufi.Simulation(cfg) as b:
        assert b.load_history(tmp_path / "h.txt") == 31
        e_rest = b.run(31, cfg.Nt)
        hb = b.history()
    assert np.array_equal(e_rest, e_all[31:])
    assert np.array_equal(hb, hist)
    # a dump without the header, as the 1D GPU driver writes
    (tmp_path / "plain.txt").write_text("\n".join(repr(float(v)) for v in hist[:10 * cfg.stride_t]) + "\n")
    with nufi.Simulation(cfg) as c:
        assert c.load_history(tmp_path / "plain.txt") == 10
        assert np.array_equal(c.history()[:10 * cfg.stride_t], hist[:10 * cfg.stride_t])
    # whitespace-separated values on one long line (the reference reads with >>)
    (tmp_path / "line.txt").write_text(" ".join(repr(float(v)) for v in hist[:12 * cfg.stride_t]))
    with nufi.Simulation(cfg) as c:
        assert c.load_history(tmp_path / "line.txt") == 12
        assert np.array_equal(c.history()[:12 * cfg.stride_t], hist[:12 * cfg.stride_t])
    # a header for another grid is refused
    with nufi.Simulation(landau_1d(Nx=16, Nv=32, Nt=60)) as d:
        with pytest.raises(ValueError):
            d.load_history(tmp_path / "h.txt")
