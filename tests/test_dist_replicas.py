"""Replica bookkeeping of bench.py under torchrun, on the CPU: two gloo ranks
join, pass the barriers and agree on the maximum of their step times (the
value every rank reports is the slowest replica's)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local, pg = bench._dist()
    bench._barrier(pg)
    v = bench._max_over_ranks(pg, 1.0 + r)
    bench._barrier(pg)
    q.put((r, w, local, v))
    pg.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_replicas_agree_on_max():
    ws = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in range(ws))
    for p in procs:
        p.join(30)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == ws and o[3] == 2.0 for o in out)


def test_single_process_has_no_group():
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    w, r, local, pg = bench._dist()
    assert (w, r, local, pg) == (1, 0, 0, None)
    assert bench._max_over_ranks(pg, 3.5) == 3.5
