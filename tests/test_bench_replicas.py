"""bench.py's replica aggregation on 2 ranks (gloo, CPU): the step time is the
maximum over ranks and the value counts the bytes of every rank."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, ws, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench

    step_ms, value = bench.replica_value(1.0 + rank, 1_000_000, ws, torch.device("cpu"))
    out[rank] = (step_ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_value_two_ranks():
    ws = 2
    port = 29500 + os.getpid() % 2000
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    for r in range(ws):
        step_ms, value = res[r]
        assert step_ms == 2.0  # slowest rank
        assert value == pytest.approx(ws * 1_000_000 / 2e-3 / 1e9)
