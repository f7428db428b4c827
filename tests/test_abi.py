"""The C ABI library without running compute: it loads, exports every
function include/nufi_gb300.h declares, agrees on the layout of
nufi_config, and rejects bad configurations before touching the GPU."""
import ctypes
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

import numericalflowiteration_gb300 as nufi
from numericalflowiteration_gb300 import _lib, plan
from numericalflowiteration_gb300.config import NufiConfigC, landau_1d, two_stream_1d

HEADER = ROOT / "include" / "nufi_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nufi_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from numericalflowiteration_gb300 import build
    build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), "binding and header disagree"


def test_config_layout_matches_c(tmp_path):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "nufi_gb300.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu\\n\", sizeof(nufi_config), offsetof(nufi_config, Nx),"
        " offsetof(nufi_config, dt), offsetof(nufi_config, v_max), offsetof(nufi_config, f0_params));return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = list(map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()))
    want = [ctypes.sizeof(NufiConfigC), NufiConfigC.Nx.offset, NufiConfigC.dt.offset, NufiConfigC.v_max.offset,
            NufiConfigC.f0_params.offset]
    assert got == want


def _create_status(lib, cfg_c):
    h = ctypes.c_void_p()
    st = lib.nufi_create(ctypes.byref(cfg_c), 0, ctypes.byref(h))
    msg = lib.nufi_last_error(None).decode()
    if st == 0:
        lib.nufi_destroy(h)
    return st, msg


@pytest.mark.parametrize("mutate,code", [
    (lambda c: c.x_max.__setitem__(0, float("inf")), _lib.ERR_INVALID),
    (lambda c: c.v_min.__setitem__(0, float("-inf")), _lib.ERR_INVALID),
    (lambda c: c.f0_params.__setitem__(0, float("nan")), _lib.ERR_INVALID),
    (lambda c: (setattr(c, "f0_kind", 2), c.f0_params.__setitem__(3, 0.0)), _lib.ERR_INVALID),
    (lambda c: setattr(c, "dim", 4), _lib.ERR_INVALID),
    (lambda c: setattr(c, "order", 9), _lib.ERR_INVALID),
    (lambda c: setattr(c, "dt", -1.0), _lib.ERR_INVALID),
    (lambda c: setattr(c, "precision", 7), _lib.ERR_INVALID),
    (lambda c: c.Nx.__setitem__(0, 0), _lib.ERR_INVALID),
])
def test_invalid_configs_rejected_before_cuda(lib, mutate, code):
    c = landau_1d().to_c()
    mutate(c)
    st, msg = _create_status(lib, c)
    assert st == code and msg.startswith("nufi_create:")


def test_oversized_runs_rejected_before_cuda(lib):
    """Step counts, node counts and history sizes whose 64-bit products
    could wrap are range errors at create (as the reference's range_error
    for too many blocks, nufi/cuda_kernel.cu:115-116), before any CUDA
    call; the largest accepted step count still reaches CUDA."""
    from numericalflowiteration_gb300.config import landau_3d
    cases = [landau_1d(Nt=2 ** 30 + 1), landau_1d(Nt=2 ** 62),
             landau_3d(Nx=2048, Nv=8, Nt=2), landau_3d(Nx=8, Nv=2048, Nt=2),
             landau_3d(Nx=1024, Nv=8, Nt=2 ** 20), landau_1d(Nx=2 ** 20, Nt=2 ** 30)]
    for cfg in cases:
        st, msg = _create_status(lib, cfg.to_c())
        assert st == _lib.ERR_RANGE and msg.startswith("nufi_create:") and "too large" in msg, (cfg, msg)
        with pytest.raises(IndexError):
            nufi.Simulation(cfg)
    st, msg = _create_status(lib, landau_1d(Nt=2 ** 30).to_c())
    assert not msg.startswith("nufi_create:"), msg


def test_fp64_takes_large_velocity_grids(lib):
    """The FP64 traces stride over velocity blocks beyond the launch grid's
    y axis (65535 blocks), so FP64 handles of more than 1048560 velocity
    nodes (here 128^3 = 2.1M) are admitted and reach CUDA, as the
    reference's flat 1-D launch grid admits them."""
    from numericalflowiteration_gb300.config import landau_3d
    for cfg in (landau_3d(Nx=4, Nv=128, Nt=2), landau_3d(Nx=4, Nv=128, Nt=2, precision="fp32split"),
                landau_3d(Nx=4, Nv=101, Nt=2)):
        st, msg = _create_status(lib, cfg.to_c())
        assert not msg.startswith("nufi_create:"), msg


def test_bump_on_tail_in_3d_is_fp64_only(lib):
    """Bump-on-tail (the reference's compiled-in 3D f0) is admitted in 3D for
    the FP64 trace; the FP32-split 3D trace is Landau only, and 2D takes
    Landau only."""
    from numericalflowiteration_gb300.config import bump_on_tail_3d, landau_2d
    st, msg = _create_status(lib, bump_on_tail_3d().to_c())
    assert not msg.startswith("nufi_create:"), msg
    st, msg = _create_status(lib, bump_on_tail_3d(precision="fp32split").to_c())
    assert st == _lib.ERR_UNSUPPORTED and "FP32-split" in msg
    c = landau_2d(Nx=8, Nv=8, Nt=2).to_c()
    c.f0_kind = 2
    c.f0_params[2], c.f0_params[3] = 4.5, 0.5
    st, msg = _create_status(lib, c)
    assert st == _lib.ERR_UNSUPPORTED


def test_split_f0_phase_at_the_unwrapped_foot(lib):
    """The reference (nufi/rho.hpp:59-60) and the FP64 trace evaluate
    cos(k x) at the unwrapped foot.  The FP32-split traces take the wrapped
    cell's phase; when k (x_max - x_min) is not a multiple of 2 pi they also
    count each chain's wraps per axis and turn the phase by k L per wrap,
    for every Nx a power of two (in 1D up to 256, the staged trace).  Other
    split handles with such a k are refused at create (and by nufi_plan), as
    are the options that select the global-load 1D trace; FP64 takes any
    k."""
    from numericalflowiteration_gb300.config import bump_on_tail_1d, landau_2d, landau_3d
    for cfg in (landau_1d(k=0.3, Nx=100, precision="fp32split"), landau_1d(k=0.3, Nx=512, precision="fp32split"),
                landau_2d(k=0.25, Nx=12, precision="fp32split"), landau_3d(k=0.75, Nx=12, precision="fp32split")):
        st, msg = _create_status(lib, cfg.to_c())
        assert st == _lib.ERR_UNSUPPORTED and "2 pi" in msg, (cfg, msg)
    # admitted: 1D staged forms, and the reference's <float, 4> 1D
    # configuration through the drop-in header (x_max = 4 pi computed in
    # float, 2.8e-8 above 4 pi: periodic within the tolerance)
    float_4pi = float(np.float32(4 * np.pi))
    for cfg in (landau_1d(k=0.3), landau_1d(k=0.3, Nx=64, precision="fp32split"),
                landau_2d(k=0.25, precision="fp32split"), landau_3d(k=0.75, precision="fp32split"),
                two_stream_1d(k=0.45, precision="fp32split"), landau_1d(k=1.0, precision="fp32split"),
                landau_2d(k=1.5, precision="fp32split"), bump_on_tail_1d(k=0.37, precision="fp32split"),
                bump_on_tail_1d(k=0.3, precision="fp32split"), landau_3d(precision="fp32split"),
                two_stream_1d(Nx=256, Nv=512, Nt=1600, precision="fp32split").replace(x_max=[float_4pi])):
        st, msg = _create_status(lib, cfg.to_c())
        assert not msg.startswith("nufi_create:"), (cfg, msg)
    for opts in ({"split_global_loads": 1}, {"split_plain_kick": 1}):
        with pytest.raises(NotImplementedError, match="staged"):
            plan(landau_1d(k=0.3, Nx=64, precision="fp32split"), 152, opts)
    assert plan(landau_1d(k=0.3, Nx=64, precision="fp32split"), 152)["trace"] == "trace_split_1d_staged_kernel"
    with pytest.raises(NotImplementedError):
        nufi.Simulation(landau_1d(k=0.3, Nx=100, precision="fp32split"))


_NOALLOC_REFUSALS = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
from numericalflowiteration_gb300 import _lib, plan
from numericalflowiteration_gb300.config import landau_1d
lib = _lib.load()
cfg = landau_1d(Nx=16, Nv=32, Nt=8)
c = cfg.to_c()
dummy = ctypes.c_void_p(0x1000)
call = lambda stride, n: lib.nufi_compute_rho_noalloc(ctypes.byref(c), n, dummy, stride, 0, cfg.n_points,
                                                      dummy, None)
assert call(cfg.stride_t - 1, 1) == _lib.ERR_INVALID
assert call(2 ** 62, 1) == _lib.ERR_RANGE
assert "2^50" in lib.nufi_last_error(None).decode()
assert call(cfg.stride_t, 9) == _lib.ERR_RANGE
assert lib.nufi_compute_rho_noalloc(ctypes.byref(c), 1, None, cfg.stride_t, 0, 1, dummy, None) == _lib.ERR_INVALID
print("refusals ok")
"""


def test_noalloc_rejects_bad_strides_before_cuda(lib):
    """nufi_compute_rho_noalloc checks the caller's history stride (at least
    one slab; history within 2^50 bytes) and the step before any CUDA call.
    The calls pass a made-up device address; they run in a child process
    that sees no GPU (CUDA_VISIBLE_DEVICES empty), so a regressed check
    could never launch on that address."""
    import os
    import sys
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", _NOALLOC_REFUSALS, str(ROOT)], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0 and "refusals ok" in r.stdout, r.stderr[-2000:]


def test_create_without_a_device_reports_the_cuda_error(lib):
    """A valid configuration where no device is usable fails with the CUDA
    error's name and text (the reference's cuda::exception,
    nufi/cuda_runtime.hpp:46-51), and the library stays usable."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    st, msg = _create_status(lib, landau_1d().to_c())
    assert st == _lib.ERR_CUDA and "cudaError" in msg
    with pytest.raises(nufi.NufiError):
        nufi.Simulation(landau_1d())
    st, _ = _create_status(lib, landau_1d(order=12).to_c())
    assert st == _lib.ERR_INVALID


def test_unbuilt_combinations_report_unsupported(lib):
    c = landau_1d(order=5, precision="fp32split").to_c()
    st, msg = _create_status(lib, c)
    assert st == _lib.ERR_UNSUPPORTED and "FP32-split" in msg
    c = landau_1d().to_c()
    c.dim = 2
    c.f0_kind = 1
    c.Nx[1] = 8
    c.Nv[1] = 8
    c.x_max[1] = 1.0
    c.v_max[1] = 1.0
    st, msg = _create_status(lib, c)
    assert st == _lib.ERR_UNSUPPORTED


def test_python_errors_map_to_reference_exception_types(lib):
    with pytest.raises(ValueError):
        nufi.Simulation(landau_1d(order=12))
    with pytest.raises(NotImplementedError):
        nufi.Simulation(two_stream_1d(order=3, precision="fp32split"))


def test_handle_less_errors_are_per_thread(lib):
    """nufi_last_error(NULL) keeps each host thread's own message: a
    second thread's failure does not overwrite the first thread's."""
    import threading
    first_done, second_done = threading.Event(), threading.Event()
    seen = {}

    def first():
        c = landau_1d().to_c()
        c.dim = 4
        seen["st1"] = _create_status_raw(lib, c)
        first_done.set()
        second_done.wait(30)
        seen["msg1"] = lib.nufi_last_error(None).decode()

    def second():
        first_done.wait(30)
        c = landau_1d().to_c()
        c.order = 12
        seen["st2"] = _create_status_raw(lib, c)
        seen["msg2"] = lib.nufi_last_error(None).decode()
        second_done.set()

    threads = [threading.Thread(target=first), threading.Thread(target=second)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(60)
    assert seen["st1"] == seen["st2"] == _lib.ERR_INVALID
    assert "dim" in seen["msg1"] and "order" in seen["msg2"], seen


def test_python_mirror_checks_host_buffers():
    """The C ABI takes bare pointers; the Python mirror refuses host arrays
    that are too small or not contiguous before calling the library (a
    stand-in library fails the test if reached)."""
    class NoLibrary:
        def __getattr__(self, name):
            raise AssertionError(f"{name} reached the library")

    cfg = landau_1d(Nx=16, Nv=32, Nt=8)
    sim = object.__new__(nufi.Simulation)
    sim.cfg, sim._lib, sim._h = cfg, NoLibrary(), None
    sim.stride_t, sim.n_spatial, sim.n_points = cfg.stride_t, cfg.n_spatial, cfg.n_points
    with pytest.raises(ValueError):
        sim.download_rho(np.zeros(cfg.n_spatial - 1))
    with pytest.raises(TypeError):
        sim.download_rho(np.zeros(2 * cfg.n_spatial)[::2])
    with pytest.raises(ValueError):
        sim.upload_phi(3, np.zeros(3 * cfg.stride_t))
    with pytest.raises(ValueError):
        sim.history(0, 5, out=np.zeros(5 * cfg.stride_t))
    with pytest.raises(TypeError):
        sim.history(0, 5, out=np.zeros(6 * cfg.stride_t, dtype=np.float32))
    with pytest.raises(ValueError):
        sim.field_solve(np.zeros(cfg.n_spatial - 2))
    with pytest.raises(ValueError):
        sim.eval_points(1, np.zeros((10, 3)))
    sim._h = None  # nothing to destroy


def _create_status_raw(lib, cfg_c):
    h = ctypes.c_void_p()
    return lib.nufi_create(ctypes.byref(cfg_c), 0, ctypes.byref(h))


def test_null_handle_calls_fail_cleanly(lib):
    assert lib.nufi_compute_rho(None, 0, 0, 1) == _lib.ERR_INVALID
    assert lib.nufi_destroy(None) == 0
    assert lib.nufi_last_error(None) is not None


def test_point_step_count():
    cfg = two_stream_1d()
    assert cfg.n_points == 262144
    assert cfg.point_steps() == 262144 * 800 * 801 // 2
    assert cfg.point_steps(10, 20) == 262144 * sum(range(10, 21))


def _batch_status(lib, cfgs):
    arr = (NufiConfigC * len(cfgs))(*[c.to_c() for c in cfgs]) if cfgs else None
    h = ctypes.c_void_p()
    st = lib.nufi_batch_create(arr, len(cfgs), 0, ctypes.byref(h))
    msg = lib.nufi_batch_last_error(None).decode()
    if st == 0:
        lib.nufi_batch_destroy(h)
    return st, msg


def test_batch_rejects_bad_sets_before_cuda(lib):
    """nufi_batch_create checks the whole set before any instance touches
    the GPU: 1D, order 4, one precision, Nx dividing 256; a member's own
    config errors come back with its index."""
    from numericalflowiteration_gb300.config import bump_on_tail_1d, landau_2d
    b = bump_on_tail_1d
    assert _batch_status(lib, [])[0] == _lib.ERR_INVALID
    st, msg = _batch_status(lib, [b(), landau_2d(Nx=8, Nv=8, Nt=4)])
    assert st == _lib.ERR_UNSUPPORTED and "order 4" in msg
    st, _ = _batch_status(lib, [b(), b(precision="fp32split")])
    assert st == _lib.ERR_UNSUPPORTED
    st, _ = _batch_status(lib, [b(), b(order=5)])
    assert st == _lib.ERR_UNSUPPORTED
    for nx in (96, 512):
        st, msg = _batch_status(lib, [b(Nx=nx)])
        assert st == _lib.ERR_UNSUPPORTED and "divide 256" in msg
    st, msg = _batch_status(lib, [b(dt=-1.0), b()])
    assert st == _lib.ERR_INVALID and msg.startswith("instance 0:")


def test_batch_null_calls_fail_cleanly(lib):
    buf = (ctypes.c_double * 8)()
    assert lib.nufi_batch_forward(None, buf) == _lib.ERR_INVALID
    assert lib.nufi_batch_backward(None, buf) == _lib.ERR_INVALID
    assert lib.nufi_batch_energy(None, 0, buf) == _lib.ERR_INVALID
    s = ctypes.create_string_buffer(16)
    assert lib.nufi_batch_describe(None, s, 16) == _lib.ERR_INVALID
    assert lib.nufi_batch_destroy(None) == 0


def test_batch_python_errors(lib):
    from numericalflowiteration_gb300.config import bump_on_tail_1d, landau_2d
    with pytest.raises(ValueError):
        nufi.Batch([])
    with pytest.raises(NotImplementedError):
        nufi.Batch([landau_2d(Nx=8, Nv=8, Nt=4)])


def test_options_layout_matches_c(tmp_path):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    src = tmp_path / "opt.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "nufi_gb300.h"\n'
        "int main(void){printf(\"%zu %zu %zu\\n\", sizeof(nufi_options), offsetof(nufi_options, batch_adjoint_ppt),"
        " offsetof(nufi_options, reserved));return 0;}\n")
    exe = tmp_path / "opt"
    subprocess.run([gcc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = list(map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()))
    O = _lib.NufiOptionsC
    assert got == [ctypes.sizeof(O), O.batch_adjoint_ppt.offset, O.reserved.offset]
