"""Build libnufi_gb300.so (the C ABI of include/nufi_gb300.h) for sm_103a.

Each .cu file under csrc/ is compiled by nvcc in parallel, then linked into
a shared library next to this file:

    python -m numericalflowiteration_gb300.build [--force] [--verbose]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libnufi_gb300.so"
PROBES = HERE / "probes"
PROBE_LIB = HERE / "libnufi_probes.so"
E2E_SRC = HERE / "e2e_loop.cpp"
E2E_EXE = HERE / "e2e_loop"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnufi_gb300.so")
    return cand


def sources():
    return sorted(CSRC.glob("*.cu"))


def headers():
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


_ELF_MACHINE = {"x86_64": 62, "amd64": 62, "aarch64": 183, "arm64": 183}


def elf_matches_host(path: Path) -> bool:
    """True if `path` is an ELF object for this machine (a copy built on
    another architecture must be rebuilt, whatever its timestamp)."""
    import platform
    want = _ELF_MACHINE.get(platform.machine().lower())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    machine = int.from_bytes(head[18:20], "little")
    return want is None or machine == want


def _stale(target: Path, deps) -> bool:
    if not target.exists() or not elf_matches_host(target):
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> Path:
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    hdrs = headers()
    flags = NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    objs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *hdrs, Path(__file__)]):
            jobs.append([cc, *ARCH, *flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{Path(cmd[0]).name} failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, LIB)
    # the reference drivers' loop through the C ABI (timed by bench.py)
    if E2E_SRC.exists() and (force or _stale(E2E_EXE, [E2E_SRC, LIB, *hdrs])):
        cxx = shutil.which("g++") or "g++"
        tmp = E2E_EXE.with_suffix(".tmp")
        run([cxx, "-std=c++17", "-O2", f"-I{INCLUDE}", str(E2E_SRC), f"-L{HERE}", "-lnufi_gb300",
             f"-Wl,-rpath,{HERE}", "-o", str(tmp)])
        os.replace(tmp, E2E_EXE)
    probe_src = sorted(PROBES.glob("*.cu"))
    if probe_src and (force or _stale(PROBE_LIB, probe_src)):
        tmp = PROBE_LIB.with_suffix(".so.tmp")
        run([cc, *ARCH, *flags, "-shared", "-o", str(tmp), *map(str, probe_src), "-lcudart"])
        os.replace(tmp, PROBE_LIB)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true", help="print register/spill use per kernel")
    a = ap.parse_args(argv)
    extra = ["-Xptxas", "-v"] if a.ptxas_v else []
    print(build(force=a.force or a.ptxas_v, verbose=a.verbose or a.ptxas_v, extra_flags=extra))


if __name__ == "__main__":
    sys.exit(main())
