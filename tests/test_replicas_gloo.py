"""The N-GPU form of bench.py runs independent replicas: a barrier around the timed region
and the maximum of the ranks' times.  Its host logic is checked here with two `gloo` ranks on
the CPU (no GPU, no NCCL): rendezvous on 127.0.0.1, barrier, max-over-ranks, and the
whole-job rate computed from it."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "SALTY_BENCH_GLOO": "1"})
    import bench
    w, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    mine = 10.0 + 5.0 * r                       # this replica's timed region, ms
    slowest = bench.max_over_ranks(pg, mine, "cpu")
    rays_per_rank = 1000
    value = w * rays_per_rank / (slowest / 1e3) / 1e6  # whole-job Mrays/s, as bench.py reports it
    q.put((r, w, slowest, value))
    pg.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2, 2]
    assert all(o[2] == 15.0 for o in out)        # both ranks report the slower replica
    assert out[0][3] == pytest.approx(2 * 1000 / 0.015 / 1e6)
