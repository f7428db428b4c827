"""(CPU) Launch plans over many sizes (nufi_plan: the same planning code
nufi_create runs, without a device), checked against the invariants the
kernels rely on: every velocity chain covered, shared memory within the
227 KB a CTA may take, 16-byte slab pitches for the bulk copies, launch
grids within CUDA's limits, and the 2D/3D table row stride that keeps a
warp's gathers on distinct banks."""
import itertools

import pytest

from numericalflowiteration_gb300 import _lib, plan
from numericalflowiteration_gb300.config import bump_on_tail_1d, landau_1d, landau_2d, landau_3d, two_stream_1d

SMEM_PER_CTA = 227 * 1024
SMS = (1, 8, 148, 152)


@pytest.fixture(scope="module", autouse=True)
def lib():
    from numericalflowiteration_gb300 import build
    build.build()
    return _lib.load()


def check_common(cfg, pl, sms):
    lay = pl["layout"]
    assert lay["Nq"] == lay["Ns"] * lay["Nm"] == cfg.n_points
    assert lay["stride_t"] == cfg.stride_t
    assert lay["hist_stride"] >= lay["stride_t"] and lay["hist_stride"] % 2 == 0  # 16-byte FP64 slabs
    assert lay["table_stride"] % 4 == 0  # 16-byte FP32 slabs
    fs = pl["fp64_shape"]
    assert fs["warps"] in (1, 2, 4) and fs["ppt"] in (1, 2, 4)
    assert fs["vblocks"] * fs["warps"] * fs["ppt"] >= lay["Nm"]
    # the FP64 traces stride over velocity blocks beyond the grid's y extent
    assert fs["vblocks"] >= 1
    assert lay["partial_rows"] >= min(fs["vblocks"], 65535)
    sv = pl["solve"]
    if lay["Ns"] <= 16384:
        assert sv["ok"] == 1 and pl["solve_why"] == "" and sv["kernel"].startswith("circulant_solve_kernel")
        assert sv["blocks"] * sv["nodes_per_block"] >= lay["Ns"]
        assert sv["nodes_per_block"] in (1, 2, 4, 8)
        assert pl["solve_smem"] <= 160 * 1024
    elif max(cfg.Nx[:cfg.dim]) <= 4096:  # per-axis DFTs, a line in shared memory
        assert sv["ok"] == 1 and sv["kernel"] == "spectral_solve<2>" and sv["blocks"] * 256 >= lay["Ns"]
    else:
        assert sv["ok"] == 0 and "4096" in pl["solve_why"]


def check_staged_1d(cfg, pl, sms):
    st, lay = pl["staged"], pl["layout"]
    if cfg.Nx[0] > 256:
        assert st["ok"] == 0
        return
    assert st["ok"] == 1
    assert 1 <= st["ppt"] <= 8 and st["slabs_per_chunk"] >= 1
    assert st["ctas"] * st["ppt"] * pl["staged_tpn"] >= lay["Nm"]  # every velocity chain has a thread
    assert st["threads"] % 32 == 0 and st["threads"] <= 1024
    assert st["threads"] >= pl["staged_tpn"] * cfg.Nx[0]
    ring_bytes = st["ring"] * st["slabs_per_chunk"] * lay["table_stride"] * 4
    assert ring_bytes <= st["smem"] <= SMEM_PER_CTA
    assert lay["partial_rows"] >= st["ctas"]
    ps = pl["persistent"]
    if ps["ok"]:
        assert pl["run"] == "run_split_1d_kernel"
        assert ps["ctas"] == st["ctas"] <= 2 * sms
        assert 32 <= ps["threads"] <= 512 and ps["ppt"] == st["ppt"]
        assert -(-cfg.Nx[0] // ps["ctas"]) <= ps["threads"] // 32  # reduce/solve nodes per CTA
        assert ring_bytes <= ps["smem"] <= 220 * 1024


def check_staged_nd(cfg, pl, sms):
    st, lay = pl["staged"], pl["layout"]
    N0, N1 = cfg.Nx[0], cfg.Nx[1]
    P0 = N0 + cfg.order - 1
    assert lay["table_sx"] >= P0
    if lay["row_step"] > 0:
        # the g = 32 / N0 rows a warp holds are row_step apart and start on
        # banks r * N0 (mod 32): disjoint
        g = 32 // N0
        assert 32 % N0 == 0 and N1 % g == 0 and g * lay["row_step"] == N1
        for r in range(g):
            assert (r * lay["row_step"] * lay["table_sx"]) % 32 == (r * N0) % 32
    elif N0 < 32:
        assert lay["table_sx"] % 32 == N0 % 32
    P_rest = 1
    for a in range(1, cfg.dim):
        P_rest *= cfg.Nx[a] + cfg.order - 1
    assert lay["table_stride"] >= lay["table_sx"] * P_rest
    if cfg.order != 4 or cfg.precision != "fp32split":
        assert st["ok"] == 0
        return
    assert st["ok"] == 1 and st["ctas"] == min(lay["Nm"], sms)
    assert st["threads"] % 32 == 0 and st["threads"] <= 512
    if st["ring"] > 0:
        ring_bytes = st["ring"] * st["slabs_per_chunk"] * lay["table_stride"] * 4
        assert st["slabs_per_chunk"] >= 1 and ring_bytes <= st["smem"] <= SMEM_PER_CTA
    assert pl["persistent"]["ok"] == 0


def check_adjoint(cfg, pl):
    ad, lay = pl["adjoint"], pl["layout"]
    if cfg.dim != 1 or cfg.order not in (4, 6):
        assert ad["ok"] == 0
        return
    assert ad["ok"] == (1 if cfg.Nx[0] <= 16384 else 0)
    assert ad["threads"] % 32 == 0 and 32 <= ad["threads"] <= 256
    assert ad["grid_x"] * ad["threads"] >= cfg.Nx[0]
    assert 1 <= ad["grid_y"] <= 65535
    P = cfg.Nx[0] + cfg.order - 1
    assert ad["chunk"] == 1 or ad["chunk"] * 8 * P <= 40 * 1024


CASES_1D = [f(Nx=nx, Nv=nv, Nt=16, precision=prec)
            for f, nx, nv, prec in itertools.product(
                (landau_1d, two_stream_1d, bump_on_tail_1d), (4, 16, 33, 64, 128, 256, 300, 1024),
                (8, 100, 256, 1024, 4096), ("fp64", "fp32split"))]
CASES_1D += [landau_1d(Nx=nx, Nv=nv, Nt=8, order=o)
             for nx, nv, o in itertools.product((16, 64, 256), (32, 1024), (3, 5, 6, 7, 8))]


@pytest.mark.parametrize("sms", SMS)
def test_plans_1d(sms):
    for cfg in CASES_1D:
        pl = plan(cfg, sms)
        check_common(cfg, pl, sms)
        check_adjoint(cfg, pl)
        if cfg.precision == "fp32split":
            check_staged_1d(cfg, pl, sms)
            assert pl["trace"] in ("trace_split_1d_staged_kernel", "trace_split_1d_kernel")
        else:
            # order 4: the cell-unit trace over FP64 derivative tables
            want = "trace_fp64_1d_table_kernel" if cfg.order == 4 else "trace_fp64_kernel"
            assert pl["trace"] == want and pl["staged"]["ok"] == 0


CASES_ND = [landau_2d(Nx=nx, Nv=nv, Nt=8, precision=prec)
            for nx, nv, prec in itertools.product((4, 8, 12, 16, 20, 32, 64, 128), (8, 32, 64, 256),
                                                  ("fp64", "fp32split"))]
CASES_ND += [landau_3d(Nx=nx, Nv=nv, Nt=4, precision=prec)
             for nx, nv, prec in itertools.product((4, 8, 12, 16, 24, 32), (4, 16, 32, 64), ("fp64", "fp32split"))]
CASES_ND += [landau_2d(Nx=16, Nv=16, Nt=4, order=o) for o in (3, 5, 6)]
CASES_ND += [landau_3d(Nx=8, Nv=8, Nt=4, order=o) for o in (3, 5)]


@pytest.mark.parametrize("sms", SMS)
def test_plans_nd(sms):
    for cfg in CASES_ND:
        pl = plan(cfg, sms)
        check_common(cfg, pl, sms)
        check_adjoint(cfg, pl)
        check_staged_nd(cfg, pl, sms)
        if cfg.precision == "fp32split":
            want = "trace_split_nd_kernel"
        else:  # 2D order 4: the cell-unit trace over FP64 derivative tables
            want = {2: "trace_fp64_2d_table_kernel", 3: "trace_fp64_3d_cells_kernel"}[cfg.dim] \
                if cfg.order == 4 else "trace_fp64_kernel"
        assert pl["trace"] == want


def test_plan_of_the_measured_workloads():
    """The shapes the GB300 runs of the measured workloads reported
    (nufi_describe on 152 SMs)."""
    pl = plan(two_stream_1d(precision="fp32split"), 152)
    assert pl["staged"] == {"ok": 1, "ctas": 152, "threads": 256, "ppt": 7, "slabs_per_chunk": 13, "ring": 3,
                            "smem": 122880}
    assert pl["persistent"]["ok"] == 1 and pl["persistent"]["smem"] == 132096
    pl = plan(landau_3d(precision="fp32split"), 152)
    assert (pl["layout"]["table_sx"], pl["layout"]["row_step"]) == (22, 8)
    assert pl["staged"]["slabs_per_chunk"] == 2 and pl["staged"]["smem"] == 190656
    pl = plan(landau_2d(precision="fp32split"), 152)
    assert pl["staged"]["slabs_per_chunk"] == 15 and pl["staged"]["smem"] == 221040


@pytest.mark.gpu
def test_plan_matches_the_handles_choice():
    """On a device, nufi_create's shapes (nufi_describe) are nufi_plan's for
    the device's multiprocessor count."""
    import torch
    import numericalflowiteration_gb300 as nufi
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for cfg in (two_stream_1d(Nt=4, precision="fp32split"), landau_1d(Nt=4), bump_on_tail_1d(Nt=4, Nv=4096,
                precision="fp32split"), landau_2d(Nt=4, precision="fp32split"), landau_3d(Nt=2, precision="fp32split"),
                landau_3d(Nt=2), landau_2d(Nx=16, Nv=16, Nt=4, order=5)):
        pl = plan(cfg, sms)
        with nufi.Simulation(cfg) as sim:
            got = sim.describe()
        assert got == {k: pl[k] for k in got}, cfg


def test_plan_errors():
    with pytest.raises(ValueError):
        plan(landau_1d(), 0)
    with pytest.raises(ValueError):
        plan(landau_1d(order=12))
    with pytest.raises(IndexError):
        plan(landau_1d(Nt=2 ** 31))


def test_launch_options_select_the_kernels():
    """nufi_options (no environment variables): each option picks the
    kernel or shape it documents, and an invalid value is refused before
    any CUDA call."""
    cfg = two_stream_1d(precision="fp32split")
    assert plan(cfg, 152)["run"] == "run_split_1d_kernel"
    assert plan(cfg, 152, {"no_persistent": 1})["run"] == "graph of per-step launches"
    pl = plan(cfg, 152, {"split_global_loads": 1})
    assert pl["trace"] == "trace_split_1d_kernel" and pl["staged"]["ok"] == 0
    assert plan(cfg, 152, {"split_plain_kick": 1})["trace"] == "trace_split_1d_kernel"
    assert plan(cfg, 152, {"split_ctas_per_sm": 2})["staged"]["ctas"] == 304
    assert plan(cfg, 152, {"split_threads_per_node": 2})["staged_tpn"] == 2
    pl = plan(landau_2d(precision="fp32split"), 152, {"split_global_loads": 1})
    assert pl["staged"]["ring"] == 0 and pl["staged"]["smem"] == 0
    for bad in ({"no_persistent": 2}, {"split_ctas_per_sm": 3}, {"batch_adjoint_ppt": 3},
                {"split_threads_per_node": -1}):
        with pytest.raises(ValueError):
            plan(cfg, 152, bad)
    with pytest.raises(ValueError):
        plan(cfg, 152, {"not_an_option": 1})
