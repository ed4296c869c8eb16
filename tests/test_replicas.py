"""bench.py's multi-GPU mode is replicas only: each rank steps its own domain,
and the ranks share only a barrier and the max of their step times.  These
run that host-side logic as two gloo ranks on the CPU (no GPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    r, w, local, pg = bench.dist_setup(world)
    bench.barrier(pg)
    ms = 10.0 * (rank + 1)          # rank 1 is the slow replica
    m = bench.reduce_max(pg, ms)
    particles = 1000                 # per replica (weak scaling)
    value = w * particles * 5 / (m * 1e-3)
    bench.barrier(pg)
    q.put((r, w, local, m, value))
    pg.destroy_process_group()


def test_two_gloo_replicas_agree_on_the_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == 20.0 for o in out)          # max over ranks
    assert out[0][4] == out[1][4] == 2 * 1000 * 5 / 0.02


def test_single_process_needs_no_group():
    r, w, local, pg = bench.dist_setup(1)
    assert pg is None and w == 1
    assert bench.reduce_max(pg, 3.5) == 3.5
