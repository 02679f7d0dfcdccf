"""The multi-GPU bookkeeping (physicsbasedanimationtoolkit_gb300.replicas) with two ranks over the
gloo backend on the CPU: the barrier, the slowest rank's time and the ranks' total work, as
bench.py uses them under torchrun."""

import json
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from physicsbasedanimationtoolkit_gb300.replicas import Replicas

    g = Replicas("gloo", device=torch.device("cpu"))
    g.barrier()
    slowest = g.max(1.0 + rank)  # rank r "took" 1 + r seconds
    work = g.sum(100.0 * (rank + 1))
    if g.is_root:
        with open(out, "w") as f:
            json.dump({"world": g.world, "max": slowest, "sum": work}, f)
    g.close()


def test_two_ranks_take_the_slowest_time_and_add_their_work(tmp_path):
    import torch.multiprocessing as mp

    out = tmp_path / "root.json"
    mp.spawn(_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    r = json.loads(out.read_text())
    assert r == {"world": 2, "max": 2.0, "sum": 300.0}


def test_single_rank_needs_no_process_group(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from physicsbasedanimationtoolkit_gb300.replicas import Replicas

    g = Replicas("gloo")
    assert g.world == 1 and g.is_root
    g.barrier()
    assert g.max(3.5) == 3.5 and g.sum(7.0) == 7.0
    g.close()
