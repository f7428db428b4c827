"""bench.py's multi-GPU path runs independent replicas (the path is not
sharded across GPUs): the slowest rank's time and the whole-job rate,
checked here with two gloo ranks on the CPU.  Also the reference arm's
JSON line, which runs on the host cores only."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    ms, value = bench.aggregate_replicas(total_ms=100.0 * (rank + 1), steps=5, point_steps=1000, ws=ws, device="cpu")
    out[rank] = (ms, value)
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    ws = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    for r in range(ws):
        ms, value = res[r]
        assert ms == pytest.approx(200.0 / 5)
        assert value == pytest.approx(ws * 1000 / (40e-3))


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    ms, value = bench.aggregate_replicas(total_ms=50.0, steps=5, point_steps=1000, ws=1)
    assert ms == 10.0 and value == pytest.approx(1000 / 10e-3)


FAKE_SMI = """#!{python}
import sys, time
# stands in for nvidia-smi --query-gpu=... -lms N: one CSV line per interval
rows = [("1980", "none"), ("2070", "none"), ("2070", "Active"), ("2070", "none")] * 1000
ms = int(sys.argv[sys.argv.index("-lms") + 1])
time.sleep({delay})
for sm, hw in rows:
    print(f"0, {{sm}}, 2070, 900.0, 0x0, {{hw}}, Not Active, Not Active, Not Active", flush=True)
    time.sleep(ms / 1000)
"""


def test_clock_sampler_keeps_the_timed_window(tmp_path, monkeypatch):
    """Samples are stamped on arrival and only those inside the timed
    window count; start() waits for the first sample; an Active
    hw_slowdown is reported by name."""
    sys.path.insert(0, str(ROOT))
    import time
    import bench
    smi = tmp_path / "nvidia-smi"
    smi.write_text(FAKE_SMI.format(python=sys.executable, delay=0.3))
    smi.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    s = bench.ClockSampler(0, interval_ms=20)
    t_call = time.monotonic()
    s.start()
    assert s.lines and time.monotonic() - t_call >= 0.25  # waited for the first sample
    t0 = time.monotonic()
    time.sleep(0.5)
    t1 = time.monotonic()
    time.sleep(0.2)
    c = s.stop(t0, t1)
    assert c["in_timed_window"] and 5 <= c["samples"] <= 40
    assert len(s.lines) > c["samples"]  # the samples after t1 were left out
    assert c["sm_max_mhz"] == 2070 and c["sm_mhz"] in (1980, 2070)
    assert c["reasons"] == ["hw_slowdown"]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("PATH", str(tmp_path))
    s = bench.ClockSampler(0)
    s.start()
    assert s.stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def _bench(args, env_extra=None):
    import json
    import subprocess
    env = dict(os.environ, **(env_extra or {}))
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_line():
    """bench.py --impl reference (the oracle port on the host cores, a
    bounded sample per step) prints one line with the contract's keys and a
    zero-copy e2e; under a multi-rank launch only rank 0 prints."""
    (line,) = _bench(["--impl", "reference", "--steps", "1", "--warmup", "3", "--cpu-windows", "0:3,10:2,-1:1"])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["steps"] == 1 and line["warmup"] == 3
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"] == "two_stream_1d_256x1024_T50"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the same workload as the GPU arm: the whole run's rate, extrapolated
    # from the timed windows by the fitted per-step cost c0 + c1 n
    cb = line["cpu_baseline"]
    assert line["config"]["same_config"] is True and cb["same_config"] is True
    assert cb["fit_c0_s"] >= 0 and cb["fit_c1_s"] > 0 and "0..2,10..11,800..800" in cb["sample"]
    nt = line["config"]["Nt"]
    assert abs(cb["full_run_s_extrapolated"] - ((nt + 1) * cb["fit_c0_s"] + cb["fit_c1_s"] * nt * (nt + 1) / 2)) \
        <= 1e-9 * cb["full_run_s_extrapolated"]
    assert abs(line["value"] * cb["full_run_s_extrapolated"] - line["config"]["point_steps_per_step"]) \
        <= 1e-9 * line["config"]["point_steps_per_step"]
    assert _bench(["--impl", "reference", "--steps", "1", "--warmup", "3", "--cpu-windows", "0:3,10:2,-1:1"],
                  {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []
