"""Replica helpers over gloo on CPU, world size 2: the whole-job reductions bench.py uses, and
failure detection on the host (a rank that leaves before a collective makes the other rank's
collective fail within its process-group timeout instead of hanging)."""
import datetime
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, mode, out):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    from opensbli_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    try:
        if mode == "reduce":
            r, w, lr = replicas.dist_env()
            out[rank] = (r, w, lr, replicas.max_over_ranks(rank + 1.5), replicas.sum_over_ranks(rank + 1.0))
        elif mode == "leave":
            replicas.max_over_ranks(1.0)  # both ranks meet once
            if rank == 1:
                out[rank] = "left"
                os._exit(0)  # leaves between steps, nothing in flight
            try:
                replicas.max_over_ranks(2.0)
                out[rank] = "no error"
            except Exception as ex:  # the peer is gone: the collective must fail, not hang
                out[rank] = "error: %s" % type(ex).__name__
    finally:
        if mode == "reduce":
            dist.destroy_process_group()


def _run(mode):
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, mode, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert not p.is_alive()
    return dict(out)


def test_max_and_sum_over_two_ranks():
    out = _run("reduce")
    assert out[0] == (0, 2, 0, 2.5, 3.0)
    assert out[1] == (1, 2, 1, 2.5, 3.0)


def test_rank_leaving_fails_the_next_collective():
    out = _run("leave")
    assert out[1] == "left"
    assert out[0].startswith("error"), out[0]
