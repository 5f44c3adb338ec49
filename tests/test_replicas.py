"""The multi-GPU form of the bench is N independent replicas; their only exchange is the
end-of-run aggregation (max of the timed region over ranks, sum of the units).  Here it
runs as two gloo ranks on the CPU; the reference arm's non-zero ranks return at once."""
import json
import os
import socket
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, outdir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        dist.barrier()
        t, u = bench.replica_aggregate(dist, 100.0 + 25.0 * rank, 16 + 3 * rank, "cpu")
        with open(os.path.join(outdir, f"r{rank}.json"), "w") as f:
            json.dump([t, u], f)
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_over_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    mp.spawn(_rank, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        t, u = json.load(open(tmp_path / f"r{r}.json"))
        assert t == 125.0 and u == 35   # slowest rank's time, all ranks' units


def test_single_process_and_reference_arm_ranks():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_aggregate(None, 12.5, 7, "cpu") == (12.5, 7)
    assert bench.reference_arm(None, rank=1, world=2) is None   # no work, no output
