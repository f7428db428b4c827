"""Generate the golden vectors in tests/golden/ from the REFERENCE's own
code, built from its sources by oracle/ref/Makefile into oracle/_ref/.

Run where the reference sources are present (REF = their directory):
    python tests/golden/make_golden.py --ref REF [--only NAME] [--full]
(or set NUFI_REFERENCE_DIR instead of --ref).  --full adds the cases at
the benchmark configurations' own sizes, which take many minutes each.

Each case runs `ref_driver run` (the reference's eval_ftilda / eval /
splines / poisson::solve / interpolate with LSMR, on the configured f0) and
keeps a compact subset: the whole energy history, rho at a few steps and a
few coefficient slabs.  Field-solve cases feed a seeded random rho through
`ref_driver solve`.  The known-answer checks of bin/test_poisson.cpp and
bin/test_fields.cpp are stored as the numbers the reference prints.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from numericalflowiteration_gb300.config import (bump_on_tail_1d, landau_1d, landau_2d,  # noqa: E402
                                                 landau_3d, two_stream_1d)

DRIVER = REPO / "oracle" / "_ref" / "ref_driver"

# name -> (config, n_last, rho steps kept, slab steps kept)
RUN_CASES = {
    "landau_1d_64x256_T30": (landau_1d(), 480, [0, 1, 2, 10, 100, 240, 480], [0, 1, 479, 480]),
    "two_stream_1d_256x1024_n40": (two_stream_1d(), 40, [0, 1, 2, 20, 40], [0, 1, 39, 40]),
    "two_stream_1d_64x256_T50": (two_stream_1d(Nx=64, Nv=256), 800, [0, 1, 400, 800], [0, 799, 800]),
    "bump_on_tail_1d_64x256_T20": (bump_on_tail_1d(), 320, [0, 1, 160, 320], [0, 319, 320]),
    "small_landau_1d_16x32": (landau_1d(Nx=16, Nv=32, Nt=20), 20, list(range(21)), list(range(21))),
    "order3_landau_1d_32x64": (landau_1d(Nx=32, Nv=64, Nt=12, order=3), 12, [0, 1, 6, 12], [0, 6, 12]),
    "order5_landau_1d_32x64": (landau_1d(Nx=32, Nv=64, Nt=12, order=5), 12, [0, 1, 6, 12], [0, 6, 12]),
    "landau_2d_32x64_n20": (landau_2d(), 20, [0, 1, 2, 10, 20], [0, 1, 19, 20]),
    "landau_2d_16x16_T20": (landau_2d(Nx=16, Nv=16), 160, [0, 1, 80, 160], [0, 159, 160]),
    "small_landau_2d_8x8": (landau_2d(Nx=8, Nv=8, Nt=10), 10, list(range(11)), list(range(11))),
    "landau_3d_16x32_n3": (landau_3d(), 3, [0, 1, 2, 3], [0, 1, 2, 3]),
    "landau_3d_8x8_T2": (landau_3d(Nx=8, Nv=8, Nt=20), 20, [0, 1, 10, 20], [0, 19, 20]),
    "small_landau_3d_4x4": (landau_3d(Nx=4, Nv=4, Nt=5), 5, list(range(6)), list(range(6))),
    # spline orders other than 4 in 2D and 3D
    "ordernd3_landau_2d_8x8": (landau_2d(Nx=8, Nv=8, Nt=10, order=3), 10, [0, 1, 5, 10], [0, 5, 10]),
    "ordernd5_landau_2d_8x8": (landau_2d(Nx=8, Nv=8, Nt=10, order=5), 10, [0, 1, 5, 10], [0, 5, 10]),
    "ordernd3_landau_3d_4x4": (landau_3d(Nx=4, Nv=4, Nt=5, order=3), 5, [0, 1, 3, 5], [0, 3, 5]),
    "ordernd5_landau_3d_4x4": (landau_3d(Nx=4, Nv=4, Nt=5, order=5), 5, [0, 1, 3, 5], [0, 3, 5]),
    # the highest orders the FP64 path takes: 6..8 in 1D, 6 in 2D
    "orderhi6_landau_1d_32x64": (landau_1d(Nx=32, Nv=64, Nt=12, order=6), 12, [0, 1, 6, 12], [0, 6, 12]),
    "orderhi7_landau_1d_32x64": (landau_1d(Nx=32, Nv=64, Nt=12, order=7), 12, [0, 1, 6, 12], [0, 6, 12]),
    "orderhi8_landau_1d_32x64": (landau_1d(Nx=32, Nv=64, Nt=12, order=8), 12, [0, 1, 6, 12], [0, 6, 12]),
    "orderhi6_landau_2d_8x8": (landau_2d(Nx=8, Nv=8, Nt=10, order=6), 10, [0, 1, 5, 10], [0, 5, 10]),
    # f0 parameters at the corners of the batched workload's ranges
    # (alpha in [0.01, 0.05], k in [0.3, 0.5], u_b in [4, 5], sigma_b in
    # [0.4, 0.6]; the bump-on-tail domain is [0, 2 pi / k)).  The Landau case
    # keeps [0, 4 pi) with k = 0.3, where cos(kx) is not periodic, so f0 at
    # the unwrapped foot (nufi/rho.hpp:59-60) matters
    "params_bump_lo_1d_64x256_n60": (bump_on_tail_1d(Nt=60, alpha=0.05, k=0.3, u_b=4.0, sigma_b=0.4), 60,
                                     [0, 1, 30, 60], [0, 30, 60]),
    "params_bump_hi_1d_128x512_n40": (bump_on_tail_1d(Nx=128, Nv=512, Nt=40, alpha=0.01, k=0.5, u_b=5.0,
                                                      sigma_b=0.6), 40, [0, 1, 20, 40], [0, 20, 40]),
    "params_landau_k03_1d_64x256_n60": (landau_1d(Nt=60, alpha=0.05, k=0.3), 60, [0, 1, 30, 60], [0, 30, 60]),
}

# The benchmark configurations at their own sizes (generated with --full):
# the two-stream 256 x 1024 run over all 800 steps, the 2D Landau
# 32^2 x 64^2 run over all 160 steps, and the first 10 steps of the 3D
# Landau 16^3 x 32^3 run (its whole run is hours of CPU time; its later
# steps are pinned by FULL_POINT_CASES below)
FULL_RUN_CASES = {
    "two_stream_1d_256x1024_T50": (two_stream_1d(), 800, [0, 1, 200, 400, 600, 800], [0, 400, 799, 800]),
    "landau_2d_32x64_T20": (landau_2d(), 160, [0, 1, 40, 80, 160], [0, 80, 159, 160]),
    "landau_3d_16x32_n10": (landau_3d(), 10, [0, 1, 5, 10], [0, 10]),
}

# name -> (config, metrics steps): the reference's eval_f metrics of its own
# in-order run, at the listed steps (ref_driver metrics)
METRICS_CASES = {
    "metrics_small_landau_1d_16x32": (landau_1d(Nx=16, Nv=32, Nt=20), [0, 1, 10, 20]),
    "metrics_landau_1d_64x256_T30": (landau_1d(), [0, 100, 480]),
    "metrics_two_stream_1d_64x256_T50": (two_stream_1d(Nx=64, Nv=256), [0, 400, 800]),
    "metrics_bump_on_tail_1d_64x256_n80": (bump_on_tail_1d(Nt=80), [0, 80]),
    "metrics_order5_landau_1d_32x64": (landau_1d(Nx=32, Nv=64, Nt=12, order=5), [0, 12]),
    "metrics_small_landau_2d_8x8": (landau_2d(Nx=8, Nv=8, Nt=10), [0, 1, 10]),
    "metrics_landau_2d_16x16_n40": (landau_2d(Nx=16, Nv=16, Nt=40), [0, 20, 40]),
    "metrics_small_landau_3d_4x4": (landau_3d(Nx=4, Nv=4, Nt=5), [0, 1, 5]),
    "metrics_landau_3d_8x8_T2": (landau_3d(Nx=8, Nv=8, Nt=20), [0, 10, 20]),
}

SOLVE_CASES = {
    "solve_1d_64": landau_1d(),
    "solve_1d_256": two_stream_1d(),
    "solve_2d_32": landau_2d(),
    "solve_3d_16": landau_3d(),
    "solve_1d_64_order3": landau_1d(order=3),
    "solve_1d_64_order5": landau_1d(order=5),
    # above 16384 nodes the device solve takes its spectral form
    "solve_2d_256": landau_2d(Nx=256, Nv=4),
    "solve_3d_32": landau_3d(Nx=32, Nv=4),
}


def _driver_run(cfg, n_last, p: Path, summation: int):
    env = dict(os.environ, NUFI_REF_SUMMATION=str(summation))
    subprocess.run([str(DRIVER), "run", str(p.with_suffix(".cfg")), "0", str(n_last), str(p)], check=True, env=env)
    energy = np.fromfile(str(p) + ".energy")
    rho = np.fromfile(str(p) + ".rho").reshape(n_last + 1, cfg.n_spatial)
    coeffs = np.fromfile(str(p) + ".coeffs").reshape(cfg.Nt + 1, cfg.stride_t)
    return energy, rho, coeffs


def run_case(name, cfg, n_last, rho_keep, slab_keep, tmp: Path):
    """The reference's loop twice: rho summed in q order (its CPU loop) and
    compensated (the exact sum of the same f~ values); the gap between the
    two energy histories is the FP64 summation floor of the case."""
    p = tmp / name
    (p.with_suffix(".cfg")).write_bytes(cfg.to_bytes())
    energy, rho, coeffs = _driver_run(cfg, n_last, p, 0)
    energy_c, rho_c, coeffs_c = _driver_run(cfg, n_last, p, 1)
    floor = float(np.max(np.abs(energy - energy_c)) / np.max(np.abs(energy_c)))
    np.savez_compressed(HERE / f"{name}.npz", config=np.frombuffer(cfg.to_bytes(), dtype=np.uint8),
                        n_last=n_last, energy=energy, rho_steps=np.array(rho_keep), rho=rho[rho_keep],
                        slab_steps=np.array(slab_keep), slabs=coeffs[slab_keep], energy_comp=energy_c,
                        rho_comp=rho_c[rho_keep], slabs_comp=coeffs_c[slab_keep], summation_floor=floor)
    return {"n_last": n_last, "energy_max": float(np.max(energy)), "energy_last": float(energy[-1]),
            "summation_floor": floor}


def metrics_case(name, cfg, steps, tmp: Path):
    """The reference's run to the last listed step, then its eval_f metrics
    at each listed step on that history."""
    p = tmp / name
    (p.with_suffix(".cfg")).write_bytes(cfg.to_bytes())
    n_last = max(steps)
    _, _, coeffs = _driver_run(cfg, n_last, p, 0)
    coeffs.tofile(str(p) + ".hist")
    out = []
    for n in steps:
        subprocess.run([str(DRIVER), "metrics", str(p.with_suffix(".cfg")), str(p) + ".hist", str(n), str(p)],
                       check=True)
        out.append(np.fromfile(str(p) + ".metrics"))
    keep = list(range(n_last + 1))  # eval_f at step n reads slabs 0 .. n
    np.savez_compressed(HERE / f"{name}.npz", config=np.frombuffer(cfg.to_bytes(), dtype=np.uint8),
                        steps=np.array(steps), metrics=np.array(out), n_last=n_last,
                        slab_steps=np.array(keep), slabs=coeffs[keep])
    return {"steps": steps, "metrics_last": [float(v) for v in out[-1]]}


def solve_case(name, cfg, tmp: Path, seed: int):
    rng = np.random.default_rng(seed)
    rho = -1.0 + 1e-2 * rng.standard_normal(cfg.n_spatial)
    p = tmp / name
    p.with_suffix(".cfg").write_bytes(cfg.to_bytes())
    rho.tofile(str(p) + ".rhoin")
    subprocess.run([str(DRIVER), "solve", str(p.with_suffix(".cfg")), str(p) + ".rhoin", str(p)], check=True)
    slab = np.fromfile(str(p) + ".slab")
    energy = np.fromfile(str(p) + ".energy")[0]
    np.savez_compressed(HERE / f"{name}.npz", config=np.frombuffer(cfg.to_bytes(), dtype=np.uint8),
                        rho=rho, slab=slab, energy=energy)
    return {"energy": float(energy)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("NUFI_REFERENCE_DIR"),
                    help="directory of the reference sources (default: $NUFI_REFERENCE_DIR)")
    ap.add_argument("--only", default=None)
    ap.add_argument("--full", action="store_true", help="also the cases at the benchmark sizes (slow)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("the reference sources are needed: --ref REF or NUFI_REFERENCE_DIR")
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle" / "ref"), f"REF={args.ref}"], check=True)
    manifest = {"generator": "tests/golden/make_golden.py", "driver": "oracle/ref/ref_driver.cpp",
                "cases": {}}
    mpath = HERE / "manifest.json"
    if mpath.exists():
        manifest = json.loads(mpath.read_text())
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        cases = dict(RUN_CASES, **(FULL_RUN_CASES if args.full else {}))
        for name, (cfg, n_last, rk, sk) in cases.items():
            if args.only and args.only not in name:
                continue
            manifest["cases"][name] = run_case(name, cfg, n_last, rk, sk, tmp)
            print(name, manifest["cases"][name], flush=True)
        for name, (cfg, steps) in METRICS_CASES.items():
            if args.only and args.only not in name:
                continue
            manifest["cases"][name] = metrics_case(name, cfg, steps, tmp)
            print(name, manifest["cases"][name], flush=True)
        for i, (name, cfg) in enumerate(SOLVE_CASES.items()):
            if args.only and args.only not in name:
                continue
            manifest["cases"][name] = solve_case(name, cfg, tmp, 20261203 + i)
            print(name, manifest["cases"][name], flush=True)
    kat_p = json.loads(subprocess.run([str(DRIVER), "poisson_kat"], check=True, capture_output=True,
                                      text=True).stdout)
    kat_f = json.loads(subprocess.run([str(DRIVER), "fields_kat"], check=True, capture_output=True,
                                      text=True).stdout)
    manifest["kat"] = {"test_poisson_rel_l1": kat_p, "test_fields_2d": kat_f}
    mpath.write_text(json.dumps(manifest, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
