"""The C++ interfaces: include/nufi_gb300/nufi_gb300.hpp (run, forward /
backward, batch) compiled against the library, and the drop-in
nufi/cuda_kernel.hpp compiled inside the reference's own scheduler header
where the reference sources are present."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle.ref import reference_dir

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "numericalflowiteration_gb300"
REF = reference_dir() or Path("reference-sources-absent")


def _build_demo(tmp_path):
    from numericalflowiteration_gb300 import build
    build.build()
    exe = tmp_path / "api_demo"
    subprocess.run(["g++", "-std=c++17", "-O1", str(ROOT / "tests" / "cpp" / "api_demo.cpp"), "-I", str(ROOT / "include"),
                    "-L", str(PKG), "-lnufi_gb300", f"-Wl,-rpath,{PKG}", "-o", str(exe)], check=True)
    return exe


def test_cpp_api_compiles_and_maps_errors(tmp_path):
    exe = _build_demo(tmp_path)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert "invalid: invalid_argument" in out
    import torch
    if not torch.cuda.is_available():
        assert "runtime_error:" in out


@pytest.mark.gpu
def test_cpp_api_forward_backward_match_python(tmp_path):
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300.config import landau_1d
    exe = _build_demo(tmp_path)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    vals = {ln.split(" ", 1)[0]: ln.split() for ln in out.splitlines()}
    J = float(vals["J"][1])
    g = np.array([float(v) for v in vals["grad"][1:]])
    with nufi.Simulation(landau_1d(Nx=32, Nv=64, Nt=40)) as s:
        Jp = s.forward()
        gp = s.backward()
    assert abs(J - Jp) <= 1e-14 * abs(Jp)
    assert np.max(np.abs(g - gp)) <= 1e-12 * np.max(np.abs(gp))
    assert "batch J" in out


@pytest.mark.skipif(not (REF / "bin" / "test_nufi_gpu_1d.cpp").exists(), reason="reference sources not present")
@pytest.mark.parametrize("driver", ["test_nufi_gpu_1d.cpp", "test_nufi_gpu_2d.cpp", "test_nufi_gpu_3d.cpp"])
def test_reference_drivers_build_unchanged_against_the_dropin(driver, tmp_path):
    """The reference's own GPU drivers (bin/test_nufi_gpu_{1d,2d,3d}.cpp),
    unchanged, compile and link against the drop-in nufi/cuda_kernel.hpp and
    libnufi_gb300.so (with the reference's poisson.cpp and the oracle's FFTW
    and BLAS shims, as the reference build would): their scheduler includes
    this repository's header, not the reference's.  Stand-ins cover the
    libraries absent here (single-rank MPI for 2D/3D, armadillo for the 1D
    plots).  Without a GPU the program stops where the reference's does: its
    scheduler's device count throws nufi::cuda::exception."""
    from numericalflowiteration_gb300 import build
    build.build()
    exe = tmp_path / "driver"
    r = subprocess.run(["g++", "-std=c++17", "-O0", "-fopenmp", "-w", "-H",
                        "-I", str(ROOT / "include" / "nufi_gb300"), "-I", str(ROOT / "include"),
                        "-I", str(ROOT / "tests" / "cpp" / "stubs"), "-I", str(ROOT / "oracle" / "ref" / "shim"),
                        "-I", str(REF), "-I", "/usr/local/cuda/include", str(REF / "bin" / driver),
                        str(REF / "nufi" / "poisson.cpp"), str(ROOT / "oracle" / "ref" / "shim_fftw.cpp"),
                        str(ROOT / "oracle" / "ref" / "shim_blas.cpp"), "-L", str(PKG), "-lnufi_gb300",
                        "-L", "/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{PKG}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    kernel_headers = [ln.strip(". ") for ln in r.stderr.splitlines() if ln.endswith("cuda_kernel.hpp")]
    assert kernel_headers and all(str(ROOT / "include" / "nufi_gb300") in str(Path(h).resolve())
                                  for h in kernel_headers), kernel_headers
    import torch
    if torch.cuda.is_available():
        return  # the full simulation is not run here
    run = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert run.returncode != 0 and "nufi::cuda::exception" in run.stderr, run.stderr[-2000:]


@pytest.mark.skipif(not (REF / "nufi" / "config.hpp").exists(), reason="reference sources not present")
def test_dropin_metrics_grid_reaches_device_creation(tmp_path):
    """The two-config constructor takes conf_metrics's grid (a finer
    velocity grid here, and the drivers' own equal grid): both get through
    the header to device creation, the grid set by nufi_set_metrics_grid
    (its GPU results are pinned in test_gpu_parity.py)."""
    from numericalflowiteration_gb300 import build
    build.build()
    src = tmp_path / "grid.cpp"
    src.write_text(r'''
#include <cstdio>
#include <stdexcept>
#include <nufi/cuda_kernel.hpp>
int main()
{
    nufi::dim1::config_t<double> c, cm;
    cm.Nu = 2 * c.Nu;
    cm.du = (cm.u_max - cm.u_min) / cm.Nu;
    try { nufi::dim1::cuda_kernel<double, 4> k(c, cm, 0); std::puts("finer: created"); }
    catch (const std::invalid_argument &) { std::puts("finer: invalid_argument"); }
    catch (const std::exception &) { std::puts("finer: device error"); }
    nufi::dim1::config_t<double> same;
    same.Nx = c.Nx; same.Nu = c.Nu;
    same.dx = (same.x_max - same.x_min) / same.Nx;
    same.du = (same.u_max - same.u_min) / same.Nu;
    try { nufi::dim1::cuda_kernel<double, 4> k(c, same, 0); std::puts("same: created"); }
    catch (const std::invalid_argument &) { std::puts("same: invalid_argument"); }
    catch (const std::exception &) { std::puts("same: device error"); }
    return 0;
}
''')
    exe = tmp_path / "grid"
    subprocess.run(["g++", "-std=c++17", "-O0", "-w", "-I", str(ROOT / "include" / "nufi_gb300"), "-I",
                    str(ROOT / "include"), "-I", str(REF), "-I", "/usr/local/cuda/include", str(src), "-L", str(PKG),
                    "-lnufi_gb300", "-L", "/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{PKG}", "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120).stdout.split("\n")
    import torch
    want = "created" if torch.cuda.is_available() else "device error"
    assert out[0] == "finer: " + want and out[1] == "same: " + want, out


@pytest.mark.skipif(not (REF / "nufi" / "cuda_scheduler.hpp").exists(), reason="reference sources not present")
def test_dropin_header_compiles_inside_reference_scheduler(tmp_path):
    src = tmp_path / "tu.cpp"
    # the reference's drivers include <vector> before the scheduler header
    src.write_text(
        "#include <vector>\n#include <nufi/cuda_scheduler.hpp>\n"
        "template class nufi::dim1::cuda_scheduler<double, 4>;\n"
        "template class nufi::dim1::cuda_scheduler<float, 4>;\n"
        "template class nufi::dim2::cuda_scheduler<double, 4>;\n"
        "template class nufi::dim3::cuda_scheduler<double, 4>;\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include" / "nufi_gb300"), "-I", str(REF),
                        "-I", "/usr/local/cuda/include", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def _build_dropin_gpu(tmp_path):
    """tests/cpp/dropin_gpu.cpp against the drop-in header, with the
    interface-only stand-ins of the reference's config.hpp and
    cuda_runtime.hpp (tests/cpp/dropin_stubs): builds wherever the CUDA
    toolkit is, also without the reference sources."""
    from numericalflowiteration_gb300 import build
    build.build()
    exe = tmp_path / "dropin_gpu"
    subprocess.run(["g++", "-std=c++17", "-O1", "-w", "-I", str(ROOT / "tests" / "cpp" / "dropin_stubs"),
                    "-I", str(ROOT / "include" / "nufi_gb300"), "-I", str(ROOT / "include"),
                    "-I", "/usr/local/cuda/include", str(ROOT / "tests" / "cpp" / "dropin_gpu.cpp"),
                    "-L", str(PKG), "-lnufi_gb300", "-L", "/usr/local/cuda/lib64", "-lcudart",
                    f"-Wl,-rpath,{PKG}", "-o", str(exe)], check=True)
    return exe


DROPIN_CASES = [(1, "small_landau_1d_16x32", 16, 32), (2, "small_landau_2d_8x8", 8, 8),
                (3, "small_landau_3d_4x4", 4, 4)]


def test_dropin_class_builds_without_reference_headers(tmp_path):
    """The drop-in class compiles and links from this repository alone; on
    a machine without a GPU its constructor throws nufi::cuda::exception,
    as the reference's does."""
    import torch
    exe = _build_dropin_gpu(tmp_path)
    if torch.cuda.is_available():
        return
    from conftest import golden
    cfg, g = golden("small_landau_1d_16x32")
    h = tmp_path / "h.bin"
    np.asarray(g["slabs"], dtype=np.float64).tofile(h)
    r = subprocess.run([str(exe), "1", "d", "16", "32", str(cfg.Nt), str(h), str(tmp_path / "rho.bin")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 4 and "nufi::cuda::exception" in r.stderr, (r.returncode, r.stderr)


@pytest.mark.gpu
@pytest.mark.parametrize("real", ["d", "f"])
@pytest.mark.parametrize("dim,name,N,Nv", DROPIN_CASES)
def test_dropin_class_on_gpu_matches_reference(tmp_path, dim, name, N, Nv, real):
    """nufi::dimN::cuda_kernel<double|float, 4> (the drop-in class, not the
    Python mirror) on the GPU: upload_phi of the reference's history, then
    compute_rho over a split q range and download_rho (accumulating) for
    every step, against the reference's rho.  double: 1e-12 (FP64 plain);
    float: the FP32-split form on the float-rounded history, 1e-6."""
    from conftest import golden, rel_max
    exe = _build_dropin_gpu(tmp_path)
    cfg, g = golden(name)
    assert list(g["slab_steps"]) == list(range(cfg.Nt + 1))
    h = tmp_path / "h.bin"
    np.asarray(g["slabs"], dtype=np.float64).tofile(h)
    out = tmp_path / "rho.bin"
    r = subprocess.run([str(exe), str(dim), real, str(N), str(Nv), str(cfg.Nt), str(h), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    rho = np.fromfile(out).reshape(cfg.Nt + 1, cfg.n_spatial)
    tol = 1e-12 if real == "d" else 1e-6
    for i, n in enumerate(g["rho_steps"]):
        assert rel_max(rho[n], g["rho"][i]) <= tol, (n, rel_max(rho[n], g["rho"][i]))
