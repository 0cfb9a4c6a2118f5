"""The multi-rank path of the benchmark on CPU (gloo, world size 2): the path
shards into independent replicas, so the only collective is the barrier and
the max-over-ranks of the timed region."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank_main(rank, ws, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    got_ws, got_rank, got_local = bench.dist_env()
    dist.barrier()
    ms = bench.max_over_ranks(torch, 10.0 + 5.0 * rank, got_ws, device="cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got_ws, got_rank, got_local, ms))


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 0, 0, 15.0), (1, 2, 1, 1, 15.0)]


def test_single_rank_needs_no_process_group():
    torch = pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(torch, 3.25, 1) == 3.25
