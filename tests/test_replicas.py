"""Replicas on several processes (the ``bench.py --gpus N`` path), on CPU with gloo.

PIV pairs are independent: N GPUs run N replicas with no collective on the data
path; the only exchange is the job's time, the maximum over ranks of each rank's
step time.  Two gloo ranks on 127.0.0.1 check that reduction and the whole-job
throughput built from it.
"""

import json
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: step 10 + r ms, series 7 - r ms, single call 3 ms
        got = bench.max_over_ranks([10.0 + rank, 7.0 - rank, 3.0], dist)
        value = bench.replica_throughput(65025, world, got[0])
        Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"max": got, "value": value}))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_single_process():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks([1.5, 2]) == [1.5, 2.0]
    assert bench.replica_throughput(1000, 1, 2.0) == pytest.approx(5e5)


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    for rank in range(world):
        r = json.loads((tmp_path / f"rank{rank}.json").read_text())
        assert r["max"] == [11.0, 7.0, 3.0]
        # two replicas of 65025 vectors in 11 ms (the slower rank)
        assert r["value"] == pytest.approx(2 * 65025 / 11e-3)
