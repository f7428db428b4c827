"""The allocation-free rho entry point, nufi_compute_rho_noalloc, against
the regular drop-in path (nufi_compute_rho + nufi_download_rho).

It serves callers that must not allocate device memory: a plugin whose
host framework owns all device memory through its own pool, or a real-time
loop that reserves its device memory up front (cudaMalloc can synchronise
the device and take unbounded time).  Such a caller hands in its own
device buffers (the test makes them with torch); the entry point keeps its
scratch in a fixed 8 MiB array inside the library.  The file name sorts
last so that a stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu


def test_noalloc_rho_matches_compute_rho_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300 import build
    from numericalflowiteration_gb300.config import landau_1d, two_stream_1d

    build.build()
    lib = nufi.load()
    torch.cuda.init()
    for cfg in (landau_1d(Nx=64, Nv=256, Nt=40), two_stream_1d(Nx=128, Nv=512, Nt=30)):
        steps = (17, cfg.Nt)
        with nufi.Simulation(cfg) as sim:
            sim.run()
            hist = sim.history()
            want = {}
            for n in steps:
                sim.compute_rho(n)
                want[n] = sim.download_rho(np.zeros(cfg.n_spatial))
        dev_hist = torch.from_numpy(hist).cuda()
        rho = torch.full((cfg.n_spatial,), float("nan"), dtype=torch.float64, device="cuda")
        c = cfg.to_c()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for i, n in enumerate(steps):  # two calls in a row share the library's scratch
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            st = lib.nufi_compute_rho_noalloc(ctypes.byref(c), n, ctypes.c_void_p(dev_hist.data_ptr()),
                                              cfg.stride_t, 0, cfg.n_points, ctypes.c_void_p(rho.data_ptr()),
                                              stream)
            assert st == 0, lib.nufi_last_error(None).decode()
            torch.cuda.synchronize()
            if i > 0:  # after the first call (which may load the library's module): no device allocation
                assert torch.cuda.mem_get_info()[0] == free0
            assert rel_max(rho.cpu().numpy(), want[n]) <= 1e-13


def test_noalloc_rejects_problems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300.config import landau_3d

    lib = nufi.load()
    torch.cuda.init()
    cfg = landau_3d()  # 16^3 x 32^3: partial sums need ~64 MiB
    c = cfg.to_c()
    # buffers of their real sizes, so that a regressed size check would give
    # a wrong status, not accesses past the caller's buffers
    hist = torch.zeros((cfg.Nt + 1) * cfg.stride_t, dtype=torch.float64, device="cuda")
    rho = torch.zeros(cfg.n_spatial, dtype=torch.float64, device="cuda")
    st = lib.nufi_compute_rho_noalloc(ctypes.byref(c), 1, ctypes.c_void_p(hist.data_ptr()), cfg.stride_t, 0,
                                      cfg.n_points, ctypes.c_void_p(rho.data_ptr()), None)
    torch.cuda.synchronize()
    assert st == 2 and b"bytes of scratch" in lib.nufi_last_error(None)


def test_fp64_3d_double_float_contraction_against_fp64_kernel():
    """The FP64 3D order-4 trace takes the 4^3 window contraction and the
    cubic bases in double-float arithmetic (trace_fp64_3d_cells_kernel);
    the allocation-free entry point traces with the generic kernel, whose
    contraction is FP64 throughout (trace_fp64_kernel).  On the same
    history their rho agree far inside the reference-parity bar (1e-12):
    measured 5.9e-16 and 7.5e-16 of max |rho| at steps 3 and 12."""
    torch = pytest.importorskip("torch")
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300 import build
    from numericalflowiteration_gb300.config import landau_3d

    build.build()
    lib = nufi.load()
    torch.cuda.init()
    cfg = landau_3d(Nx=8, Nv=8, Nt=12, alpha=0.05)
    with nufi.Simulation(cfg) as sim:
        assert sim.describe()["trace"] == "trace_fp64_3d_cells_kernel"
        sim.run()
        hist = sim.history()
        want = {}
        for n in (3, cfg.Nt):
            sim.compute_rho(n)
            want[n] = sim.download_rho(np.zeros(cfg.n_spatial))
    dev_hist = torch.from_numpy(hist).cuda()
    rho = torch.zeros(cfg.n_spatial, dtype=torch.float64, device="cuda")
    c = cfg.to_c()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n, w in want.items():
        st = lib.nufi_compute_rho_noalloc(ctypes.byref(c), n, ctypes.c_void_p(dev_hist.data_ptr()), cfg.stride_t,
                                          0, cfg.n_points, ctypes.c_void_p(rho.data_ptr()), stream)
        assert st == 0, lib.nufi_last_error(None).decode()
        torch.cuda.synchronize()
        d = rel_max(w, rho.cpu().numpy())
        print(f"step {n}: double-float vs FP64 contraction, max |d rho| / max |rho| = {d:.2e}")
        assert d <= 1e-14
