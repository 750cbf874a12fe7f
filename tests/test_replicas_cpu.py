"""Multi-process replica bookkeeping on CPU (gloo, world size 2)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    import torch.distributed as dist
    from crava_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, lr = replicas.world()
    replicas.barrier(ws)
    my_ms = 1.5 + rank  # rank 1 is the slower replica
    m = replicas.max_over_ranks(my_ms, ws)
    rate = replicas.whole_job_rate(1000000, m, ws)
    q.put((r, ws, m, rate))
    dist.destroy_process_group()


def test_two_replicas_report_max_time_and_total_bins():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for r, ws, m, rate in out:
        assert ws == 2
        assert m == pytest.approx(2.5)
        assert rate == pytest.approx(2 * 1e6 / 2.5e-3 / 1e6)


def test_single_process_defaults():
    from crava_gb300 import replicas
    assert replicas.max_over_ranks(3.0, 1) == 3.0
    assert replicas.whole_job_rate(8454144, 1.0, 1) == pytest.approx(8454.144)
