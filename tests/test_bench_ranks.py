"""The benchmark's multi-rank logic on the CPU (gloo, world size 2): one replica per
rank, the job's time is its slowest rank's, rank 0's autotuner decisions reach every
rank, and every rank searches its own queries against the same objects."""
import os
import socket
import tempfile

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import json
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slowest = bench.reduce_max(10.0 + rank, world, device="cpu")
        choice = bench.broadcast_choice({"P": 8 + rank, "probes": [(1.0 * rank, {"T": 128})]}, world)

        class Args:
            n, nq, dim = 64, 16, 8
        base, queries = bench.workload(Args, rank)
        np.save(os.path.join(out_dir, "base%d.npy" % rank), base)
        np.save(os.path.join(out_dir, "queries%d.npy" % rank), queries)
        with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
            json.dump({"slowest": slowest, "choice": choice, "index": bench.index_path(
                type("A", (), {"workdir": "/w", "n": 64, "dim": 8}), rank)}, f)
    finally:
        dist.destroy_process_group()


def test_two_ranks_share_decisions_and_take_the_slowest_time():
    import json
    import torch.multiprocessing as mp
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(2, _free_port(), d), nprocs=2, start_method="spawn")
        r = [json.load(open(os.path.join(d, "rank%d.json" % i))) for i in range(2)]
        assert r[0]["slowest"] == r[1]["slowest"] == 11.0
        assert r[0]["choice"] == r[1]["choice"] == {"P": 8, "probes": [[0.0, {"T": 128}]]}
        assert r[0]["index"] != r[1]["index"]                       # one replica per rank
        b0, b1 = np.load(os.path.join(d, "base0.npy")), np.load(os.path.join(d, "base1.npy"))
        q0, q1 = np.load(os.path.join(d, "queries0.npy")), np.load(os.path.join(d, "queries1.npy"))
        assert np.array_equal(b0, b1) and not np.array_equal(q0, q1)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    assert bench.broadcast_choice({"x": 1}, 1) == {"x": 1}
