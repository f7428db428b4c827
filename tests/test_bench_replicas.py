"""bench.py's multi-GPU path runs independent replicas (the path is not
sharded across GPUs): the slowest rank's time and the whole-job rate,
checked here with two gloo ranks on the CPU."""
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
