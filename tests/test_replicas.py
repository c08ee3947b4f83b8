"""Replica (multi-rank) logic of bench.py on CPU with gloo, world size 2:
disjoint event ranges per rank and the max over ranks of the step time.
Events are independent, so ranks exchange nothing but this one value."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        first = bench.rank_first_event(rank)
        ms = bench.max_over_ranks(10. + 5. * rank, torch.device("cpu"), world)
        dist.barrier()
        out[rank] = (first, ms)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out),
                       nprocs=world, start_method="spawn")
    firsts = sorted(v[0] for v in out.values())
    assert firsts == [0, 10 ** 12]
    assert all(v[1] == 15. for v in out.values())


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None, 1) == 3.5
