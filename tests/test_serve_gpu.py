"""The request loop (fb_server_*): continuous batching under an HBM budget with
a device-resident LRU cache. Every result must be the same alone and in the mix."""
import time

import numpy as np
import pytest

from fuzzyblue_gb300 import workloads
from fuzzyblue_gb300.params import PRECISION_MIXED, Parameters, smoke_parameters
from tests.golden.make_golden import tiny_parameters

pytestmark = pytest.mark.gpu


def alone(builder, p):
    from fuzzyblue_gb300.api import Atmosphere
    pend = Atmosphere.build(builder, p)
    pend.wait()
    out = pend.atmosphere().to_host()
    pend.release()
    return out


def _mix():
    rng = np.random.default_rng(5)
    ps = [smoke_parameters(), tiny_parameters(), smoke_parameters(precision=PRECISION_MIXED, order=3)]
    for _ in range(5):
        p = workloads.draw_atmosphere(rng, order=int(rng.integers(2, 6)), precision=int(rng.integers(0, 2)))
        ps.append(p.replace(**workloads.CLASSES["half"]))
    return ps


def test_results_same_alone_and_in_the_mix(builder):
    from fuzzyblue_gb300.api import Server
    ps = _mix()
    with Server(builder, max_batch=3, max_inflight=3) as srv:
        tickets = [srv.submit(p) for p in ps]
        outs = []
        for t in tickets:
            atm = srv.wait(t, 60000)
            assert atm is not None
            outs.append(atm.to_host())
            srv.release(t)
        st = srv.stats()
    assert st["completed"] == len(ps) and st["batches"] >= 1
    assert st["p99_ms"] >= st["p50_ms"] > 0
    for p, o in zip(ps, outs):
        ref = alone(builder, p)
        for k in ("transmittance", "irradiance", "scattering"):
            assert np.array_equal(o[k], ref[k]), k


def test_identical_requests_share_one_build(builder):
    from fuzzyblue_gb300.api import Server
    p = smoke_parameters()
    with Server(builder) as srv:
        t1 = srv.submit(p)
        t2 = srv.submit(p)
        a1 = srv.wait(t1, 60000)
        a2 = srv.wait(t2, 60000)
        assert a1.transmittance() == a2.transmittance()
        st = srv.stats()
        assert st["cache_hits"] >= 1
        srv.release(t1)
        srv.release(t2)
        t3 = srv.submit(p)  # resident: answered at once
        assert srv.poll(t3) is not None
        srv.release(t3)


def test_request_over_budget_is_rejected(builder):
    from fuzzyblue_gb300 import _native as N
    from fuzzyblue_gb300.api import Server
    with Server(builder, hbm_budget_bytes=64 << 10) as srv:
        with pytest.raises(N.FuzzyblueError) as ei:
            srv.submit(smoke_parameters())
        assert ei.value.status == N.FB_ERR_BUDGET
        assert srv.stats()["rejected"] == 1


def test_admission_keeps_within_budget_and_evicts(builder):
    from fuzzyblue_gb300.api import Server, device_bytes
    ps = _mix()
    need = max(sum(device_bytes(p)) for p in ps)
    out_max = max(device_bytes(p)[0] for p in ps)
    budget = 2 * need + out_max
    with Server(builder, hbm_budget_bytes=budget, max_batch=2, max_inflight=4) as srv:
        tickets = [srv.submit(p) for p in ps]
        peak = 0
        done = 0
        deadline = time.time() + 120
        pending = list(tickets)
        while pending and time.time() < deadline:
            st = srv.stats()
            peak = max(peak, st["resident_bytes"] + st["inflight_bytes"])
            still = []
            for t in pending:
                if srv.poll(t) is not None:
                    srv.release(t)  # unpinned: may be evicted for later requests
                    done += 1
                else:
                    still.append(t)
            pending = still
            time.sleep(0.001)
        st = srv.stats()
    assert done == len(ps)
    assert peak <= budget
    assert st["evictions"] >= 1


def test_cancel_queued_request(builder):
    from fuzzyblue_gb300.api import Server
    from fuzzyblue_gb300 import _native as N
    with Server(builder, max_batch=1, max_inflight=1) as srv:
        big = Parameters()  # keeps the only stream busy for a few ms
        t0 = srv.submit(big)
        t1 = srv.submit(smoke_parameters(order=2))
        cancelled = srv.cancel(t1)
        srv.wait(t0, 60000)
        srv.release(t0)
        if cancelled:
            with pytest.raises(N.FuzzyblueError) as ei:
                srv.poll(t1)
            assert ei.value.status == N.FB_ERR_CANCELLED
            assert srv.stats()["cancelled"] == 1
        else:  # it had already started: it completes normally
            assert srv.wait(t1, 60000) is not None


def test_completion_queue_lists_every_finished_ticket_once(builder):
    """fb_server_completed: every submitted ticket, cache hits included, comes
    out of the completion queue exactly once; polling it then gives its tables."""
    from fuzzyblue_gb300.api import Server
    ps = _mix()
    ps.append(ps[0])  # identical to the first: shared with its build or resident
    with Server(builder, max_batch=3, max_inflight=3) as srv:
        tickets = [srv.submit(p) for p in ps]
        seen = []
        t0 = time.perf_counter()
        while len(seen) < len(tickets) and time.perf_counter() - t0 < 120:
            seen.extend(srv.completed(timeout_ms=100))
        assert sorted(seen) == sorted(tickets)
        assert srv.completed(timeout_ms=0) == []
        for t in tickets:
            assert srv.poll(t) is not None
            srv.release(t)
