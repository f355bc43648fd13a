"""Multi-rank host logic of bench.py on CPU: two gloo ranks, as torchrun would
start them.  Replicas only: the ranks exchange nothing but the barrier and the
max-over-ranks step time."""
import json
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_setup()
    bench.dist_barrier(w)
    # Each rank reports a different step time; every rank must see the maximum.
    got = bench.dist_max(10.0 + 5.0 * rank, w)
    # The reference arm runs on rank 0 only; other ranks leave without work.
    other = None
    if rank != 0:
        other = bench.run_reference_arm(None, w, r)
    bench.dist_barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"world": w, "rank": r, "local": local, "max": got, "other": other}, f)


def test_two_gloo_ranks_max_and_barrier(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for rank in range(world):
        res = json.load(open(tmp_path / f"rank{rank}.json"))
        assert res["world"] == world and res["rank"] == rank and res["local"] == rank
        assert res["max"] == 10.0 + 5.0 * (world - 1)
        assert res["other"] is None
    assert torch is not None


def test_single_rank_needs_no_process_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    assert bench.dist_setup() == (1, 0, 0)
    assert bench.dist_max(3.5, 1) == 3.5
    bench.dist_barrier(1)
