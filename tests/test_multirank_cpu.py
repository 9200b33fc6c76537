"""Multi-rank harness of bench.py on CPU (gloo, world_size 2).

Beams are independent, so ranks shard them with no data-path collective;
the only collectives are the timing barrier and the max-over-ranks of the
step time.  This runs those pieces as two gloo processes on 127.0.0.1.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    w, r = bench.dist_init("gloo")
    assert (w, r) == (world, rank)
    bench.barrier()
    seeds = [bench.beam_seed(rank, i) for i in range(8)]
    t = bench.max_over_ranks(1.5 + rank)          # rank 1 is the slow one
    out.put((rank, seeds, t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_sharding_and_timing():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    (r0, s0, t0), (r1, s1, t1) = res
    assert t0 == t1 == 2.5                         # max over ranks
    assert not set(s0) & set(s1)                   # disjoint beams per rank


def test_single_process_defaults(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench
    assert bench.dist_env() == (1, 0, 0)
    assert bench.max_over_ranks(3.25) == 3.25


def test_reference_arm_other_ranks_exit(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    assert bench.main(["--impl", "reference", "--steps", "1", "--warmup", "3"]) == 0
    assert capsys.readouterr().out == ""
