"""The multi-rank (replica) reduction of bench.py on world_size 2 with the gloo backend (CPU):
max over ranks of the device time, sum over ranks of the pairs."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dev_ms = [10.0, 12.5][rank]
    pairs = [1000, 3000][rank]
    res = bench.combine_ranks(dist, "cpu", maxes=[dev_ms, 1.0 + rank], sums=[pairs, 2 * pairs])
    q.put((rank, res))
    dist.barrier()
    dist.destroy_process_group()


def test_combine_ranks_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        maxes, sums = out[r]
        assert maxes == [12.5, 2.0]
        assert sums == [4000.0, 8000.0]


def test_combine_ranks_single_process():
    maxes, sums = bench.combine_ranks(None, "cpu", maxes=[3.0], sums=[7])
    assert maxes == [3.0] and sums == [7.0]
