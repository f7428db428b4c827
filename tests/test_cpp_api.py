"""The C++ interfaces: include/nufi_gb300/nufi_gb300.hpp (run, forward /
backward, batch) compiled against the library, and the drop-in
nufi/cuda_kernel.hpp compiled inside the reference's own scheduler header
where the reference sources are present."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "numericalflowiteration_gb300"
REF = Path(os.environ.get("NUFI_REFERENCE_DIR", "/root/reference"))


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
def test_dropin_refuses_a_different_metrics_grid(tmp_path):
    """The drop-in's metrics use the rho grid, as the reference's drivers
    pass it (bin/test_nufi_gpu_1d.cpp:216-221); a conf_metrics with other
    node counts is refused with std::invalid_argument before any CUDA call,
    and the drivers' own equal grid gets through to device creation."""
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
    catch (const std::exception &e) { std::printf("finer: other %s\n", e.what()); }
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
    assert out[0] == "finer: invalid_argument"
    import torch
    assert out[1] == ("same: created" if torch.cuda.is_available() else "same: device error"), out


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
