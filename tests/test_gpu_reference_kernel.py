"""The reference's own GPU kernels (nufi/cuda_kernel.cu built for sm_103a by
oracle/ref/Makefile, launched by oracle/ref/ref_gpu.py) against the new FP64
path on the same coefficient history: dim{1,2,3}::cuda_eval_rho<double,4>
must give the new FP64 rho to rounding (its atomicAdd order is arbitrary),
and cuda_eval_rho<float,4> (the reference 1D driver's type) to FP32
accuracy.  Skipped where the reference's GPU build is absent (it is made
only where the reference sources are)."""
import numpy as np
import pytest

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


def _cases():
    from numericalflowiteration_gb300 import config
    return {"landau_1d": lambda: config.landau_1d(Nx=64, Nv=256, Nt=40),
            "two_stream_1d": lambda: config.two_stream_1d(Nx=64, Nv=256, Nt=40),
            "bump_on_tail_1d": lambda: config.bump_on_tail_1d(Nx=64, Nv=256, Nt=40),
            "landau_2d": lambda: config.landau_2d(Nx=8, Nv=16, Nt=20),
            "landau_3d": lambda: config.landau_3d(Nx=4, Nv=8, Nt=12)}


@pytest.mark.gpu
@pytest.mark.parametrize("make", ["landau_1d", "two_stream_1d", "bump_on_tail_1d", "landau_2d", "landau_3d"])
def test_reference_gpu_rho_matches_new_fp64(ref_gpu, make):
    import torch
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300 import config
    cfg = _cases()[make]()
    Ns, Nt = cfg.n_spatial, cfg.Nt
    steps = sorted({0, 1, 2, Nt // 2, Nt})
    with nufi.Simulation(cfg) as sim:
        sim.run()
        hist = sim.history()
        new = {}
        for n in steps:
            sim.compute_rho(n)
            new[n] = sim.download_rho(np.zeros(Ns))
    ref = ref_gpu.RefGpu()
    ref.set_f0(config._F0_NAMES[cfg.f0], cfg.f0_params)
    for real, tol in (("double", 1e-12), ("float", 2e-4)):
        coeffs = ref_gpu.device_history(cfg, hist, real)
        rho = torch.zeros(Ns, dtype=coeffs.dtype, device="cuda")
        conf = ref.pack_conf(real, cfg)
        for n in steps:
            ref.eval_rho(real, cfg, n, coeffs, conf, rho)
            r = rho.double().cpu().numpy()
            scale = np.max(np.abs(new[n]))
            assert np.max(np.abs(r - new[n])) <= tol * scale, (real, n, np.max(np.abs(r - new[n])) / scale)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_reference_config_packing(dim):
    """(CPU) The by-value config_t<real> packs every field of the reference's
    struct (layout probed from its header) with the constructor's derived
    values, rounded to real."""
    import json
    from oracle.ref import ref_gpu
    from numericalflowiteration_gb300 import config
    path = ref_gpu.REF_DIR / "ref_gpu_layout.json"
    if not path.exists():
        pytest.skip("no reference layout in oracle/_ref")
    cfg = {1: config.two_stream_1d, 2: config.landau_2d, 3: config.landau_3d}[dim]()

    class Packer(ref_gpu.RefGpu):
        def __init__(self):
            self.layout = json.loads(path.read_text())

    pk = Packer()
    for real, R in (("float", np.float32), ("double", np.float64)):
        lay = pk.layout[f"dim{dim}::config_t<{real}>"]
        b = pk.pack_conf(real, cfg)
        assert len(b) == lay["size"]
        off = lay["fields"]
        get = lambda name: np.frombuffer(b[off[name]:off[name] + R().itemsize], dtype=R)[0]
        assert int.from_bytes(b[off["Nx"]:off["Nx"] + 8], "little") == cfg.Nx[0]
        assert int.from_bytes(b[off["Nt"]:off["Nt"] + 8], "little") == cfg.Nt
        L = R(R(cfg.x_max[0]) - R(cfg.x_min[0]))
        assert get("Lx") == L and get("dx") == R(L / R(cfg.Nx[0])) and get("dx_inv") == R(R(1) / R(L / R(cfg.Nx[0])))
        assert get("du") == R(R(R(cfg.v_max[0]) - R(cfg.v_min[0])) / R(cfg.Nv[0]))


def test_reference_cubin_holds_the_launched_entries():
    """(CPU) The reference GPU build lists the six kernels ref_gpu.py
    launches (dim 1-3 cuda_eval_rho, float and double, order 4)."""
    from oracle.ref import ref_gpu
    if not ref_gpu.available():
        pytest.skip("no reference GPU build in oracle/_ref")
    entries = (ref_gpu.REF_DIR / "nufi_ref_gpu.entries").read_text().split()
    for dim in (1, 2, 3):
        for tag in ("If", "Id"):
            prefix = f"_ZN4nufi4dim{dim}13cuda_eval_rho{tag}Lm4E"
            assert sum(e.startswith(prefix) for e in entries) == 1, prefix
