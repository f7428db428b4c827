"""The 3D Landau workload (16^3 x 32^3, 134M points per step, dt = 0.1,
T = 10) pinned at its later steps, where running the reference's whole loop
on the CPU would take hours: the reference's own code evaluated on a given
coefficient history.

Two stages:

  python tests/golden/make_points_golden.py history OUT_DIR     (on a GPU)
      runs the workload's whole FP64 run (101 steps) and its FP32-split run
      on the GPU and writes OUT_DIR/landau_3d_16x32_T10_run.npz: the FP64
      coefficient history, both energy histories and the run times.

  python tests/golden/make_points_golden.py golden RUN_NPZ --ref REF
      (where the reference sources are, with oracle/ref built) rounds that
      history to single precision (so that the fixture is half the size;
      the rounded values are the history every check uses, exactly), and
      runs the reference's code on it (oracle/_ref/ref_driver): rho at
      steps 10, 50, 100 with compensated sums over all 134M points, and
      eval_ftilda at 2^20 seeded points of phase space at the same steps.
      Writes tests/golden/landau_3d_16x32_points.npz: the rounded history,
      rho, the first 2^16 f~ values exactly, the sums of f~ over the 1024
      blocks of 1024 consecutive points, and the energy histories of the
      GPU runs (FP64 and FP32-split, for the record).

The points come from points_3d() below (splitmix64, so the same on every
machine): x uniform in [0, 4 pi)^3, v uniform in [-6, 6]^3.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from numericalflowiteration_gb300.config import landau_3d  # noqa: E402

STEPS = (10, 50, 100)
NPTS = 1 << 20
NEXACT = 1 << 16
BLOCK = 1024
SEED = 20261204


def points_3d(n: int = NPTS, seed: int = SEED) -> np.ndarray:
    """n points (x, y, z, u, v, w) from a splitmix64 stream: x in [0, 4 pi),
    v in [-6, 6) per axis; platform independent (uint64 arithmetic)."""
    with np.errstate(over="ignore"):
        i = np.arange(6 * n, dtype=np.uint64) + np.uint64(seed)
        z = i * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)  # [0, 1)
    u = u.reshape(n, 6)
    pts = np.empty_like(u)
    pts[:, :3] = u[:, :3] * (4.0 * np.pi)
    pts[:, 3:] = -6.0 + 12.0 * u[:, 3:]
    return pts


def stage_history(out_dir: Path):
    import numericalflowiteration_gb300 as nufi
    from numericalflowiteration_gb300 import build
    build.build()
    nufi.load()
    cfg = landau_3d()
    t0 = time.perf_counter()
    with nufi.Simulation(cfg) as sim:
        e64 = sim.run()
        hist = sim.history()
    t64 = time.perf_counter() - t0
    t0 = time.perf_counter()
    with nufi.Simulation(cfg.replace(precision="fp32split")) as sim:
        es = sim.run()
    ts = time.perf_counter() - t0
    out_dir.mkdir(parents=True, exist_ok=True)
    np.savez(out_dir / "landau_3d_16x32_T10_run.npz", hist=hist, energy_fp64=e64, energy_split=es,
             seconds_fp64=t64, seconds_split=ts)
    print(f"fp64 {t64:.1f} s, split {ts:.1f} s, energy err {np.max(np.abs(es - e64)) / np.max(np.abs(e64)):.3e}")


def stage_golden(run_npz: Path, ref: str):
    driver = REPO / "oracle" / "_ref" / "ref_driver"
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle" / "ref"), f"REF={ref}"], check=True)
    run = np.load(run_npz)
    cfg = landau_3d()
    hist32 = run["hist"].astype(np.float32)
    hist = hist32.astype(np.float64)
    pts = points_3d()
    rho, f_exact, f_blocks = [], [], []
    with tempfile.TemporaryDirectory() as td:
        t = Path(td)
        (t / "c.cfg").write_bytes(cfg.to_bytes())
        hist.tofile(t / "hist")
        pts.tofile(t / "pts")
        env = dict(os.environ, NUFI_REF_SUMMATION="1")
        for n in STEPS:
            subprocess.run([str(driver), "rho", str(t / "c.cfg"), str(t / "hist"), str(n), str(t / "r"), "1"],
                           check=True, env=env, stdout=subprocess.DEVNULL)
            rho.append(np.fromfile(str(t / "r") + ".rho"))
            subprocess.run([str(driver), "points", str(t / "c.cfg"), str(t / "hist"), str(n), "0", str(t / "pts"),
                            str(t / "p")], check=True)
            f = np.fromfile(str(t / "p") + ".f")
            f_exact.append(f[:NEXACT])
            f_blocks.append(f.reshape(-1, BLOCK).sum(axis=1))
            print(f"step {n}: rho max {np.max(np.abs(rho[-1])):.6e}, f~ sum {f.sum():.12e}", flush=True)
    np.savez_compressed(HERE / "landau_3d_16x32_points.npz", config=np.frombuffer(cfg.to_bytes(), dtype=np.uint8),
                        hist32=hist32, steps=np.array(STEPS), rho_comp=np.array(rho), npts=NPTS, seed=SEED,
                        block=BLOCK, f_exact=np.array(f_exact), f_block_sums=np.array(f_blocks),
                        energy_fp64_gpu=run["energy_fp64"], energy_split_gpu=run["energy_split"])


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    h = sub.add_parser("history")
    h.add_argument("out_dir")
    g = sub.add_parser("golden")
    g.add_argument("run_npz")
    g.add_argument("--ref", default=os.environ.get("NUFI_REFERENCE_DIR"))
    a = ap.parse_args()
    if a.cmd == "history":
        stage_history(Path(a.out_dir))
    else:
        if not a.ref:
            ap.error("the reference sources are needed: --ref REF or NUFI_REFERENCE_DIR")
        stage_golden(Path(a.run_npz), a.ref)


if __name__ == "__main__":
    main()
