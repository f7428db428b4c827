"""GPU parity: the sm_103a kernels, called through the C ABI, against the
reference's golden vectors (tests/golden/) and the CPU oracle.

Measures: max |d| / max |ref| for rho, slabs and energy histories.
FP64 plain must agree with the reference to 1e-12: against the reference
run with compensated rho sums (the GPU sums in a fixed, compensated tree)
and, against the reference's in-order sums, within 1e-12 or 3x that case's
measured FP64 summation floor (conftest.energy_tol).  FP32-split must stay
within 1e-6 of the FP64 energy history (the metric's gate).
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


def _slabs_ok(cfg, hist, g, tol=1e-11):
    st = cfg.stride_t
    for i, n in enumerate(g["slab_steps"]):
        if n <= int(g["n_last"]):
            assert rel_max(hist[n * st:(n + 1) * st], g["slabs"][i]) <= tol, f"slab {n}"


@pytest.mark.parametrize("name", ["small_landau_1d_16x32", "small_landau_2d_8x8", "small_landau_3d_4x4",
                                  "order3_landau_1d_32x64", "order5_landau_1d_32x64",
                                  "ordernd3_landau_2d_8x8", "ordernd5_landau_2d_8x8",
                                  "ordernd3_landau_3d_4x4", "ordernd5_landau_3d_4x4",
                                  "orderhi6_landau_1d_32x64", "orderhi7_landau_1d_32x64",
                                  "orderhi8_landau_1d_32x64", "orderhi6_landau_2d_8x8"])
def test_fp64_stepwise_rho_energy_slabs(nufi, name):
    cfg, g = golden(name)
    with nufi.Simulation(cfg) as sim:
        energies = []
        for n in range(int(g["n_last"]) + 1):
            energies.append(sim.step(n))
            rho = sim.download_rho(np.zeros(cfg.n_spatial))
            if n in list(g["rho_steps"]):
                i = list(g["rho_steps"]).index(n)
                assert rel_max(rho, g["rho"][i]) <= 1e-12, f"rho step {n}"
        assert rel_max(energies, g["energy_comp"]) <= 1e-12
        assert rel_max(energies, g["energy"]) <= energy_tol(g)
        _slabs_ok(cfg, sim.history(), g)
        assert sim.launches >= 2 * (int(g["n_last"]) + 1)


@pytest.mark.parametrize("name", ["landau_1d_64x256_T30", "bump_on_tail_1d_64x256_T20",
                                  "two_stream_1d_256x1024_n40", "landau_2d_16x16_T20", "landau_3d_8x8_T2",
                                  "landau_2d_32x64_n20", "landau_3d_16x32_n3",
                                  "params_bump_lo_1d_64x256_n60", "params_bump_hi_1d_128x512_n40",
                                  "params_landau_k03_1d_64x256_n60"])
def test_fp64_graph_run_matches_reference(nufi, name):
    cfg, g = golden(name)
    n_last = int(g["n_last"])
    with nufi.Simulation(cfg) as sim:
        e = sim.run(0, n_last)
        assert rel_max(e, g["energy_comp"]) <= 1e-12
        assert rel_max(e, g["energy"]) <= energy_tol(g)
        _slabs_ok(cfg, sim.history(), g)
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
        assert rel_max(rho, g["rho"][list(g["rho_steps"]).index(n_last)]) <= 1e-12


def test_fp64_bump_on_tail_3d_matches_oracle(nufi, oracle_mod):
    """The reference's compiled-in 3D configuration (bump-on-tail, v in
    [-9, 0]^3, x in [0, 20 pi / 3)^3), reduced to 4^3 x 6^3 and 6 steps:
    the FP64 run against the oracle with compensated sums (the oracle's f0
    matches the reference's compiled f0 to the last bit)."""
    from numericalflowiteration_gb300.config import bump_on_tail_3d
    cfg = bump_on_tail_3d(Nx=4, Nv=6, Nt=6)
    with nufi.Simulation(cfg) as sim:
        e = sim.run()
        hist = sim.history()
    oracle_mod.set_summation(1)
    try:
        e_ref, _, h_ref = oracle_mod.run(cfg, 0, cfg.Nt)
    finally:
        oracle_mod.set_summation(0)
    assert rel_max(e, e_ref) <= 1e-12
    assert rel_max(hist, h_ref) <= 1e-11


def test_fp64_two_stream_through_saturation(nufi):
    cfg, g = golden("two_stream_1d_64x256_T50")
    with nufi.Simulation(cfg) as sim:
        e = sim.run()
    assert rel_max(e[:200], g["energy_comp"][:200]) <= 1e-12
    assert rel_max(e[:200], g["energy"][:200]) <= max(2e-12, energy_tol(g))
    assert rel_max(e, g["energy"]) <= 1e-9


@pytest.mark.parametrize("name", ["solve_1d_64", "solve_1d_256", "solve_2d_32", "solve_3d_16",
                                  "solve_1d_64_order3", "solve_1d_64_order5", "solve_2d_256", "solve_3d_32"])
def test_device_field_solve_matches_reference(nufi, name):
    cfg, g = golden(name)
    with nufi.Simulation(cfg) as sim:
        slab, e = sim.field_solve(g["rho"])
    assert rel_max(slab, g["slab"]) <= 1e-12
    assert abs(e - float(g["energy"])) <= 1e-12 * abs(float(g["energy"]))


def test_dropin_upload_compute_download(nufi, oracle_mod):
    """The reference drivers' loop: upload_phi the reference's slabs, then
    compute_rho over a split q range and download_rho (which accumulates)."""
    cfg, g = golden("small_landau_1d_16x32")
    st = cfg.stride_t
    coeffs = np.zeros((cfg.Nt + 1) * st)
    for i, n in enumerate(g["slab_steps"]):
        coeffs[n * st:(n + 1) * st] = g["slabs"][i]
    with nufi.Simulation(cfg) as sim:
        for n in range(cfg.Nt + 1):
            sim.upload_phi(n, coeffs)
        for n in [0, 1, 7, cfg.Nt]:
            acc = np.zeros(cfg.n_spatial)
            cuts = [0, 37, 200, cfg.n_points]
            for a, b in zip(cuts[:-1], cuts[1:]):
                sim.compute_rho(n, a, b)
                sim.download_rho(acc)
            oracle_mod.set_summation(1)
            want = oracle_mod.rho(cfg, n, coeffs)
            oracle_mod.set_summation(0)
            assert rel_max(acc, want) <= 1e-13
            assert rel_max(acc, g["rho"][list(g["rho_steps"]).index(n)]) <= 1e-12
        # float buffers of the <float, order> instantiation
        acc32 = np.zeros(cfg.n_spatial, dtype=np.float32)
        sim.compute_rho(3)
        sim.download_rho(acc32)
        assert rel_max(acc32, g["rho"][3]) <= 1e-6


def test_dropin_errors_and_empty_range(nufi):
    cfg, _ = golden("small_landau_1d_16x32")
    with nufi.Simulation(cfg) as sim:
        with pytest.raises(IndexError):
            sim.compute_rho(cfg.Nt + 1)
        with pytest.raises(IndexError):
            sim.compute_rho(0, 0, cfg.n_points + 1)
        sim.compute_rho(0)
        a = sim.download_rho(np.zeros(cfg.n_spatial))
        sim.compute_rho(0, 5, 5)  # empty: the reference returns without touching rho
        b = sim.download_rho(np.zeros(cfg.n_spatial))
        assert np.array_equal(a, b)
        with pytest.raises(IndexError):
            sim.upload_phi(cfg.Nt + 1, np.zeros((cfg.Nt + 2) * cfg.stride_t))


def test_fp64_run_is_deterministic(nufi):
    cfg, _ = golden("landau_1d_64x256_T30")
    with nufi.Simulation(cfg) as a, nufi.Simulation(cfg) as b:
        ea, eb = a.run(), b.run()
        ea2 = a.run()
    assert np.array_equal(ea, eb) and np.array_equal(ea, ea2)


@pytest.mark.parametrize("name,tol", [("landau_1d_64x256_T30", 1e-6), ("bump_on_tail_1d_64x256_T20", 1e-6),
                                      ("small_landau_1d_16x32", 1e-6), ("landau_2d_32x64_n20", 1e-6),
                                      ("landau_2d_16x16_T20", 1e-6), ("small_landau_2d_8x8", 1e-6),
                                      ("landau_3d_16x32_n3", 1e-6), ("landau_3d_8x8_T2", 1e-6),
                                      ("small_landau_3d_4x4", 1e-6)])
def test_split_energy_within_gate(nufi, name, tol):
    cfg, g = golden(name)
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        e = sim.run(0, int(g["n_last"]))
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
    assert rel_max(e, g["energy"]) <= tol
    assert rel_max(rho, g["rho"][-1]) <= 1e-6


def test_split_two_stream_linear_phase(nufi):
    cfg, g = golden("two_stream_1d_64x256_T50")
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        e = sim.run()
    assert rel_max(e[:400], g["energy"][:400]) <= 1e-6


def test_split_dropin_matches_fp64(nufi):
    """The split form behind the drop-in calls: same slabs uploaded, rho
    within FP32-split accuracy of the FP64 rho."""
    cfg, g = golden("landau_1d_64x256_T30")
    st = cfg.stride_t
    with nufi.Simulation(cfg) as ref:
        ref.run(0, 100)
        coeffs = ref.history()
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        for n in range(101):
            sim.upload_phi(n, coeffs)
        sim.compute_rho(100)
        got = sim.download_rho(np.zeros(cfg.n_spatial))
    assert rel_max(got, g["rho"][list(g["rho_steps"]).index(100)]) <= 1e-6


@pytest.mark.parametrize("cfgname", ["two_stream_1d_64x256_T50", "landau_1d_64x256_T30"])
def test_split_staged_matches_unstaged(nufi, cfgname):
    """The shared-memory staged split trace (default: two-level kick sum)
    against the global-load form (Kahan-compensated kick per substep): two
    FP32-split arithmetics, each within the split gate of the FP64 history
    and of each other."""
    cfg, g = golden(cfgname)
    cfg = cfg.replace(precision="fp32split", Nt=min(cfg.Nt, 300))
    with nufi.Simulation(cfg) as a:
        ea = a.run()
    with nufi.Simulation(cfg, opts={"split_global_loads": 1}) as b:
        eb = b.run()
    assert rel_max(ea, eb) <= 1e-6
    assert rel_max(ea, g["energy"][:cfg.Nt + 1]) <= 1e-6
    assert rel_max(eb, g["energy"][:cfg.Nt + 1]) <= 1e-6


@pytest.mark.parametrize("cfgname", ["two_stream_1d_64x256_T50", "landau_1d_64x256_T30", "bump_on_tail_1d_64x256_T20"])
def test_persistent_run_matches_per_step_launches(nufi, cfgname):
    """nufi_run as one cooperative launch (all steps, grid barriers between
    the phases) against the graph of per-step launches: same arithmetic,
    only the order of a few FP64 sums differs."""
    cfg, g = golden(cfgname)
    cfg = cfg.replace(precision="fp32split", Nt=min(cfg.Nt, 300))
    with nufi.Simulation(cfg) as a:
        ea = a.run()
        ha = a.history()
        ra = a.download_rho(np.zeros(cfg.n_spatial))
    with nufi.Simulation(cfg, opts={"no_persistent": 1}) as b:
        eb = b.run()
        hb = b.history()
        rb = b.download_rho(np.zeros(cfg.n_spatial))
    assert rel_max(ea, eb) <= 1e-9
    assert rel_max(ha, hb) <= 1e-9
    assert rel_max(ra, rb) <= 1e-12
    assert rel_max(ea, g["energy"][:cfg.Nt + 1]) <= 1e-6


def test_split_landau_k03_phase_at_the_unwrapped_foot(nufi):
    """k = 0.3 on [0, 4 pi) (k L = 1.2 pi, feet wrap up to 3 times): f0's
    phase at the unwrapped foot (wrap counts in the staged traces), in the
    whole-run kernel, the per-step launches and the drop-in compute_rho on
    the FP64 history, against the reference's energy history and rho: the
    split gate.  The wrapped foot's phase would miss it by orders
    of magnitude (a 1.2 pi phase error per wrap of an alpha = 0.05 mode)."""
    cfg, g = golden("params_landau_k03_1d_64x256_n60")
    n = int(g["n_last"])
    c = cfg.replace(precision="fp32split")
    for opts in (None, {"no_persistent": 1}):
        with nufi.Simulation(c, opts=opts) as sim:
            e = sim.run(0, n)
            rho = sim.download_rho(np.zeros(cfg.n_spatial))
        assert rel_max(e, g["energy_comp"][:n + 1]) <= 1e-6, opts
        assert rel_max(rho, g["rho_comp"][list(g["rho_steps"]).index(n)]) <= 1e-6, opts
    # the drop-in compute_rho on the FP64 history (itself the reference's to
    # 1e-12, test_fp64_graph_run_matches_reference)
    with nufi.Simulation(cfg) as ref:
        ref.run(0, n)
        coeffs = ref.history()
    with nufi.Simulation(c) as sim:
        for k in range(n + 1):
            sim.upload_phi(k, coeffs)
        for k in (1, 30, 60):
            sim.compute_rho(k)
            got = sim.download_rho(np.zeros(cfg.n_spatial))
            assert rel_max(got, g["rho_comp"][list(g["rho_steps"]).index(k)]) <= 1e-6, k


@pytest.mark.parametrize("dim", [2, 3])
def test_split_nd_phase_at_the_unwrapped_foot(nufi, oracle_mod, dim):
    """2D/3D Landau with k = 0.3 on [0, 4 pi) per axis (feet wrap the domain):
    the split trace counts wraps per axis and turns each axis's phase by
    k L per wrap; the energy history against the oracle's (the reference's
    algorithm, f0 at the unwrapped foot): the split gate."""
    from numericalflowiteration_gb300.config import landau_2d, landau_3d
    cfg = (landau_2d(Nx=16, Nv=32, Nt=30, alpha=0.05, k=0.3) if dim == 2 else
           landau_3d(Nx=8, Nv=8, Nt=12, alpha=0.05, k=0.3))
    ref, _, _ = oracle_mod.run(cfg)
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        e = sim.run()
    assert rel_max(e, ref) <= 1e-6


def test_dropin_pending_upload_is_applied_everywhere(nufi):
    """upload_phi on a 1D split handle leaves the newest slab pending:
    compute_rho(n + 1) derives its table inside the trace, every other call
    applies it first.  The reference drivers' loop (compute_rho, download,
    upload per step) gives the same rho and history bits as the same loop
    with a synchronize after each upload (the table derived by its own
    launch), and metrics and eval_points between an upload and the next
    trace see the uploaded slab."""
    from numericalflowiteration_gb300.config import two_stream_1d
    cfg = two_stream_1d(Nx=64, Nv=256, Nt=40, precision="fp32split")
    with nufi.Simulation(cfg.replace(precision="fp64")) as ref:
        ref.run()
        coeffs = ref.history()

    def loop(sync_after_upload):
        rhos = []
        with nufi.Simulation(cfg) as sim:
            for n in range(cfg.Nt + 1):
                sim.compute_rho(n)
                rhos.append(sim.download_rho(np.zeros(cfg.n_spatial)))
                sim.upload_phi(n, coeffs)
                if sync_after_upload:
                    sim.synchronize()
            return np.array(rhos), sim.history()

    ra, ha = loop(False)
    rb, hb = loop(True)
    assert np.array_equal(ra, rb) and np.array_equal(ha, hb)
    assert np.array_equal(ha, coeffs)
    # a pending slab read by the metrics (FP64 eval_f on the history) and by
    # eval_points before any trace has derived it
    with nufi.Simulation(cfg) as sim, nufi.Simulation(cfg.replace(precision="fp64")) as ref:
        for n in range(6):
            sim.upload_phi(n, coeffs)
            ref.upload_phi(n, coeffs)
        sim.compute_metrics(5)
        ref.compute_metrics(5)
        assert np.array_equal(sim.download_metrics(), ref.download_metrics())
        pts = np.array([[1.0, 0.5], [7.0, -1.2], [3.3, 2.0]])
        assert np.array_equal(sim.eval_points(5, pts), ref.eval_points(5, pts))


def test_dropin_speculative_field_solve(nufi):
    """The reference drivers' loop with the device field solve (compute_rho,
    download, field_solve, upload per step): after the first step the
    handle queues the solve of its own rho behind each trace and returns it
    when field_solve's input is that rho.  Every rho, slab and energy is
    bit-identical to the same loop solved on a second handle (which never
    speculates); a different input at one step (the speculative result is
    discarded), a second compute_rho before the solve (the speculation goes
    unused) and the switch back on all keep the results exact.  While it
    speculates, each compute_rho is two launches (the trace, the solve);
    the solving handle's compute_rho stays one."""
    from numericalflowiteration_gb300.config import two_stream_1d
    cfg = two_stream_1d(Nx=64, Nv=256, Nt=40, precision="fp32split")

    def loop(own_solver):
        rhos, energies, extra, per_call = [], [], [], []
        with nufi.Simulation(cfg) as sim, nufi.Simulation(cfg) as other:
            solver = sim if own_solver else other
            coeffs = np.zeros((cfg.Nt + 1) * sim.stride_t)
            for n in range(cfg.Nt + 1):
                if n == 25:  # a trace whose rho nobody solves
                    sim.compute_rho(n)
                    sim.download_rho(np.zeros(cfg.n_spatial))
                l0 = sim.launches
                sim.compute_rho(n)
                per_call.append(sim.launches - l0)
                rho = sim.download_rho(np.zeros(cfg.n_spatial))
                if n == 12:  # another input first, then the step's own
                    extra.append(solver.field_solve(rho * 1.01))
                slab, e = solver.field_solve(rho)
                coeffs[n * sim.stride_t:(n + 1) * sim.stride_t] = slab
                sim.upload_phi(n, coeffs)
                rhos.append(rho)
                energies.append(e)
            return np.array(rhos), np.array(energies), coeffs, extra, per_call

    ra, ea, ca, xa, la = loop(True)
    rb, eb, cb, xb, lb = loop(False)
    assert la[30:40] == [2] * 10 and lb[30:40] == [1] * 10
    assert np.array_equal(ra, rb)
    assert np.array_equal(ea, eb)
    assert np.array_equal(ca, cb)
    assert np.array_equal(xa[0][0], xb[0][0]) and xa[0][1] == xb[0][1]
    # the loop is the simulation: its energies against the whole-run kernel's
    with nufi.Simulation(cfg) as sim:
        er = sim.run()
    assert rel_max(ea, er) <= 1e-6


def test_dropin_speculation_partial_ranges_and_interleaved_calls(nufi):
    """Partial q ranges (rho summed from two downloads) never equal the last
    published rho, so the handle does not speculate; once it does, a launch
    between compute_rho and field_solve (here compute_metrics) discards the
    pending speculative solve.  Every field_solve equals a second handle's
    ordinary solve of the same input, bit for bit."""
    from numericalflowiteration_gb300.config import two_stream_1d
    cfg = two_stream_1d(Nx=64, Nv=256, Nt=12, precision="fp32split")
    half = cfg.n_points // 2
    with nufi.Simulation(cfg) as sim, nufi.Simulation(cfg) as ref:
        coeffs = np.zeros((cfg.Nt + 1) * sim.stride_t)
        for n in range(cfg.Nt + 1):
            l0 = sim.launches
            if n < 5:
                rho = np.zeros(cfg.n_spatial)
                sim.compute_rho(n, 0, half)
                sim.download_rho(rho)
                sim.compute_rho(n, half, cfg.n_points)
                sim.download_rho(rho)
                assert sim.launches - l0 == 2, n  # no speculative solve behind either trace
            else:
                sim.compute_rho(n)
                # the first full-range step enables the speculation in its field_solve
                assert sim.launches - l0 == (1 if n == 5 else 2), n
                rho = sim.download_rho(np.zeros(cfg.n_spatial))
                if n == 9:
                    sim.compute_metrics(n)
                    sim.download_metrics()
            slab, e = sim.field_solve(rho)
            want_slab, want_e = ref.field_solve(rho)
            assert np.array_equal(slab, want_slab) and e == want_e, n
            coeffs[n * sim.stride_t:(n + 1) * sim.stride_t] = slab
            sim.upload_phi(n, coeffs)


def test_persistent_run_subrange_and_repeat(nufi):
    """Steps in two calls (0..k, k+1..Nt) and a repeated run give the same
    history as one call."""
    cfg, _ = golden("landau_1d_64x256_T30")
    cfg = cfg.replace(precision="fp32split", Nt=120)
    with nufi.Simulation(cfg) as a:
        e1 = a.run()
        e1b = a.run()
    with nufi.Simulation(cfg) as b:
        p1 = b.run(0, 50)
        p2 = b.run(51, cfg.Nt)
    assert np.array_equal(e1, e1b)
    assert np.array_equal(np.concatenate([p1, p2]), e1)


@pytest.mark.parametrize("cfgname", ["landau_2d_16x16_T20", "landau_3d_8x8_T2", "small_landau_2d_8x8"])
def test_split_nd_staged_matches_global_loads(nufi, cfgname):
    """2D/3D split trace with the slab tables streamed through shared memory
    against the same kernel reading them from global memory: same chunking
    of the kick sum, so the same bits."""
    cfg, g = golden(cfgname)
    cfg = cfg.replace(precision="fp32split")
    with nufi.Simulation(cfg) as a:
        ea = a.run()
        ra = a.download_rho(np.zeros(cfg.n_spatial))
    with nufi.Simulation(cfg, opts={"split_global_loads": 1}) as b:
        eb = b.run()
        rb = b.download_rho(np.zeros(cfg.n_spatial))
    assert np.array_equal(ea, eb)
    assert np.array_equal(ra, rb)
    assert rel_max(ea, g["energy"][:cfg.Nt + 1]) <= 1e-6


def test_split_nd_subrange_and_determinism(nufi):
    """2D split compute_rho over two q ranges sums to the full range, and
    repeated runs agree bit for bit."""
    cfg, g = golden("landau_2d_16x16_T20")
    cfg = cfg.replace(precision="fp32split", Nt=40)
    with nufi.Simulation(cfg) as a:
        e1 = a.run()
        e2 = a.run()
        assert np.array_equal(e1, e2)
        full = np.zeros(cfg.n_spatial)
        a.compute_rho(30)
        a.download_rho(full)
        parts = np.zeros(cfg.n_spatial)
        half = cfg.n_points // 3
        a.compute_rho(30, 0, half)
        a.download_rho(parts)
        a.compute_rho(30, half, cfg.n_points)
        a.download_rho(parts)
    assert rel_max(parts, full) <= 1e-13


@pytest.mark.parametrize("name", ["metrics_small_landau_1d_16x32", "metrics_landau_1d_64x256_T30",
                                  "metrics_two_stream_1d_64x256_T50", "metrics_bump_on_tail_1d_64x256_n80",
                                  "metrics_order5_landau_1d_32x64", "metrics_small_landau_2d_8x8",
                                  "metrics_landau_2d_16x16_n40", "metrics_small_landau_3d_4x4",
                                  "metrics_landau_3d_8x8_T2"])
@pytest.mark.parametrize("precision", ["fp64", "fp32split"])
def test_metrics_match_reference(nufi, name, precision):
    """compute_metrics / download_metrics on the reference's history against
    the reference's eval_f metrics, per component to 1e-12 relative (always
    FP64, also behind a split handle); download accumulates."""
    cfg, g = golden(name)
    hist = np.ascontiguousarray(g["slabs"].reshape(-1))
    if precision == "fp32split" and cfg.order != 4:
        # the FP32-split form is built for order 4; the C ABI refuses other
        # orders (the C++ drop-in maps <float, order> to the FP64 form)
        with pytest.raises(NotImplementedError):
            nufi.Simulation(cfg.replace(precision=precision))
        precision = "fp64"
    sim = nufi.Simulation(cfg.replace(precision=precision))
    with sim:
        for n in range(int(g["n_last"]) + 1):
            sim.upload_phi(n, hist)
        for n, ref in zip(g["steps"], g["metrics"]):
            sim.compute_metrics(int(n))
            got = sim.download_metrics()
            assert np.max(np.abs(got - ref) / np.abs(ref)) <= 1e-12, (int(n), got, ref)
        # accumulation and the empty range (no launch, device sums kept)
        acc = sim.download_metrics(np.array(g["metrics"][-1]))
        sim.compute_metrics(0, 5, 5)
        again = sim.download_metrics()
        assert np.allclose(acc, 2 * g["metrics"][-1], rtol=1e-12, atol=0)
        assert np.allclose(again, g["metrics"][-1], rtol=1e-12, atol=0)
        # a q-range partition sums to the full range
        n = int(g["steps"][-1])
        parts = np.zeros(4)
        cut = cfg.n_points // 3
        sim.compute_metrics(n, 0, cut)
        sim.download_metrics(parts)
        sim.compute_metrics(n, cut, cfg.n_points)
        sim.download_metrics(parts)
        assert np.allclose(parts, g["metrics"][-1], rtol=1e-12, atol=1e-15)
        with pytest.raises(IndexError):
            sim.compute_metrics(cfg.Nt + 1)


@pytest.mark.parametrize("name", ["metrics_landau_1d_64x256_T30", "metrics_small_landau_2d_8x8"])
def test_metrics_on_the_conf_metrics_grid(nufi, oracle_mod, name):
    """The reference's two-config kernel (nufi/cuda_kernel.cu:53-79,
    96-108): metrics points on another grid (finer, over a sub-domain),
    f = eval_f on the handle's own history.  Against the oracle's eval_f at
    the same points (itself bit for bit the reference's point function),
    summed exactly (math.fsum): 1e-12 per component.  A q range split in
    two sums to the whole; None returns to the rho grid."""
    import math
    cfg, g = golden(name)
    hist = np.ascontiguousarray(g["slabs"].reshape(-1))
    n = int(g["steps"][-1])
    d = cfg.dim
    Nx = [int(v) * 3 // 2 for v in cfg.Nx[:d]]
    Nv = [int(v) * 2 for v in cfg.Nv[:d]]
    xlo = [a + 0.1 * (b - a) for a, b in zip(cfg.x_min[:d], cfg.x_max[:d])]
    xhi = [a + 0.9 * (b - a) for a, b in zip(cfg.x_min[:d], cfg.x_max[:d])]
    vlo = [0.8 * a for a in cfg.v_min[:d]]
    vhi = [0.8 * b for b in cfg.v_max[:d]]
    mcfg = cfg.replace(Nx=Nx, Nv=Nv, x_min=xlo, x_max=xhi, v_min=vlo, v_max=vhi)
    dx = [(b - a) / k for a, b, k in zip(xlo, xhi, Nx)]
    dv = [(b - a) / k for a, b, k in zip(vlo, vhi, Nv)]
    # point q = s * Nm + m, s and m x-fastest over the axes (as the rho grid)
    xs = [xlo[a] + np.arange(Nx[a]) * dx[a] for a in range(d)]
    vs = [vlo[a] + np.arange(Nv[a]) * dv[a] + dv[a] / 2 for a in range(d)]
    X = np.stack(np.meshgrid(*xs[::-1], indexing="ij")[::-1], -1).reshape(-1, d)
    V = np.stack(np.meshgrid(*vs[::-1], indexing="ij")[::-1], -1).reshape(-1, d)
    pts = np.concatenate([np.repeat(X, len(V), 0), np.tile(V, (len(X), 1))], 1)
    f = oracle_mod.eval_points(cfg, n, hist, np.ascontiguousarray(pts), mode=1)
    w = float(np.prod(dv)) * (float(np.prod(dx)) if d < 3 else 1.0)
    u2 = np.sum(pts[:, d:] ** 2, 1)
    pos = f > 0
    ref = np.array([math.fsum(w * f), math.fsum(w * f * f), math.fsum(w * (u2 * f / 2)),
                    math.fsum(-w * f[pos] * np.log(f[pos]))])
    with nufi.Simulation(cfg) as sim:
        for k in range(int(g["n_last"]) + 1):
            sim.upload_phi(k, hist)
        sim.set_metrics_grid(mcfg)
        sim.compute_metrics(n)
        got = sim.download_metrics()
        assert np.max(np.abs(got - ref) / np.abs(ref)) <= 1e-12, (got, ref)
        cut = len(pts) // 3
        sim.compute_metrics(n, 0, cut)
        parts = sim.download_metrics()
        sim.compute_metrics(n, cut, len(pts))
        sim.download_metrics(parts)
        assert np.max(np.abs(parts - ref) / np.abs(ref)) <= 1e-12
        with pytest.raises(IndexError):
            sim.compute_metrics(n, 0, len(pts) + 1)
        sim.set_metrics_grid(None)
        sim.compute_metrics(n)
        back = sim.download_metrics()
        assert np.max(np.abs(back - g["metrics"][-1]) / np.abs(g["metrics"][-1])) <= 1e-12


def test_fp64_velocity_grid_beyond_one_launch_row(nufi, oracle_mod):
    """A velocity grid with more blocks than the launch grid's y axis holds
    (2D, 1024^2 velocity nodes: 65536 blocks of 16 against 65535): the FP64
    traces stride over the extra blocks.  rho (the cell-unit order-4 trace)
    and the metrics (the general FP64 trace) against the oracle on the same
    history."""
    from numericalflowiteration_gb300.config import landau_2d
    cfg = landau_2d(Nx=4, Nv=1024, Nt=3)
    with nufi.Simulation(cfg) as sim:
        assert sim.describe()["fp64_shape"]["vblocks"] > 65535
        sim.run(0, cfg.Nt)
        hist = sim.history()
        sim.compute_rho(cfg.Nt)
        rho = sim.download_rho(np.zeros(cfg.n_spatial))
        sim.compute_metrics(cfg.Nt)
        m = sim.download_metrics()
    oracle_mod.set_summation(1)
    try:
        want = oracle_mod.rho(cfg, cfg.Nt, hist)
        want_m = oracle_mod.metrics(cfg, cfg.Nt, hist)
    finally:
        oracle_mod.set_summation(0)
    assert rel_max(rho, want) <= 1e-12
    for k in range(4):
        assert abs(m[k] - want_m[k]) <= 1e-12 * abs(want_m[k]), k


@pytest.mark.parametrize("which", ["2d", "3d"])
def test_spectral_solve_run_matches_oracle(nufi, oracle_mod, which):
    """Grids above 16384 nodes take the spectral field solve (per-axis DFTs
    around the same diagonals as the circulant kernels): a 256^2 (2D) and a
    32^3 (3D) run, FP64 against the oracle with compensated sums (1e-12),
    and the FP32-split form within its gate."""
    from numericalflowiteration_gb300.config import landau_2d, landau_3d
    cfg = landau_2d(Nx=256, Nv=4, Nt=3) if which == "2d" else landau_3d(Nx=32, Nv=2, Nt=3)
    with nufi.Simulation(cfg) as sim:
        assert sim.describe()["solve"]["kernel"] == "spectral_solve<2>"
        e = sim.run()
        hist = sim.history()
    oracle_mod.set_summation(1)
    try:
        e_ref, _, h_ref = oracle_mod.run(cfg, 0, cfg.Nt)
    finally:
        oracle_mod.set_summation(0)
    assert rel_max(e, e_ref) <= 1e-12
    assert rel_max(hist, h_ref) <= 1e-11
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        es = sim.run()
    assert rel_max(es, e_ref) <= 1e-6
