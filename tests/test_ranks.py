"""The multi-rank path of bench.py (fuzzyblue_gb300.ranks) on two gloo ranks on
CPU: every rank reports the slowest rank's time, and the whole-job rate counts
the atmospheres of all ranks over that time. Replicas only: no rank exchanges
tables."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as td
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from fuzzyblue_gb300 import ranks
        w, r, local = ranks.layout()
        ranks.barrier(w)
        slowest = ranks.max_over_ranks(w, 1.5 + r)  # rank 1 is the slower one
        out.put((r, w, local, slowest, ranks.whole_job_rate(w, 256, slowest)))
        ranks.barrier(w)
    finally:
        td.destroy_process_group()


def test_two_replica_ranks_report_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [g[0] for g in got] == [0, 1]
    for r, w, local, slowest, rate in got:
        assert w == 2 and local == r
        assert slowest == pytest.approx(2.5)
        assert rate == pytest.approx(2 * 256 / 2.5)
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_needs_no_process_group(monkeypatch):
    from fuzzyblue_gb300 import ranks
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert ranks.layout() == (1, 0, 0)
    ranks.barrier(1)
    assert ranks.max_over_ranks(1, 3.0) == 3.0
    assert ranks.whole_job_rate(1, 64, 0.5) == 128.0
