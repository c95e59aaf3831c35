"""The N > 1 bench path on CPU: two gloo ranks, replicas with no data-path
collective; the timed region is the slowest rank's and the value counts the
samples of every rank."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # each replica generates the same stream independently
    k, v = bench.make_workload(seed=5, num_keys=512, total=1 << 14, batch=1 << 12)
    local_ms = 10.0 + 5.0 * rank
    mx = bench.max_over_ranks(dist, local_ms)
    out[rank] = (mx, bench.replica_value(world, 3, 1 << 12, mx), int(k.sum()), float(v.sum()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_time_and_value():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        r0, r1 = out[0], out[1]
    assert r0[0] == r1[0] == 15.0  # max over ranks
    assert r0[1] == pytest.approx(2 * 3 * 4096 / 0.015)
    assert r0[2:] == r1[2:]  # identical replica streams
