"""The reference's own GPU kernel (nufi/cuda_kernel.cu built for sm_103a by
oracle/ref/Makefile, launched by oracle/ref/ref_gpu.py) against the new FP64
path on the same coefficient history: cuda_eval_rho<double,4> must give the
new FP64 rho to rounding (its atomicAdd order is arbitrary), and
cuda_eval_rho<float,4> (the reference 1D driver's type) to FP32 accuracy.
Skipped where the reference's GPU build is absent (it is made only where the
reference sources are)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_gpu():
    from oracle.ref import ref_gpu
    if not ref_gpu.available():
        pytest.skip("no reference GPU build in oracle/_ref")
    import numericalflowiteration_gb300 as m
    from numericalflowiteration_gb300 import build
    build.build()
    m.load()
    return ref_gpu


@pytest.mark.parametrize("make", ["landau", "two_stream", "bump_on_tail"])
def test_reference_gpu_rho_matches_new_fp64(ref_gpu, make):
    import torch
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300 import config
    cfg = {"landau": lambda: config.landau_1d(Nx=64, Nv=256, Nt=40),
           "two_stream": lambda: config.two_stream_1d(Nx=64, Nv=256, Nt=40),
           "bump_on_tail": lambda: config.bump_on_tail_1d(Nx=64, Nv=256, Nt=40)}[make]()
    Nx, Nu, Nt = cfg.Nx[0], cfg.Nv[0], cfg.Nt
    steps = [0, 1, 2, 20, 40]
    with nufi.Simulation(cfg) as sim:
        sim.run()
        hist = sim.history()
        new = {}
        for n in steps:
            sim.compute_rho(n)
            new[n] = sim.download_rho(np.zeros(Nx))
    ref = ref_gpu.RefGpu()
    ref.set_f0(config._F0_NAMES[cfg.f0], cfg.f0_params)
    for real, tol in (("double", 1e-12), ("float", 2e-4)):
        coeffs = ref_gpu.device_history(cfg, hist, real)
        rho = torch.zeros(Nx, dtype=coeffs.dtype, device="cuda")
        conf = ref.pack_conf(real, Nx, Nu, Nt, cfg.dt, cfg.x_min[0], cfg.x_max[0], cfg.v_min[0], cfg.v_max[0])
        for n in steps:
            ref.eval_rho(real, cfg.order, n, coeffs, conf, rho, 0, Nx * Nu, Nx, Nu, Nt)
            r = rho.double().cpu().numpy()
            scale = np.max(np.abs(new[n]))
            assert np.max(np.abs(r - new[n])) <= tol * scale, (real, n)
