"""Stream handoff: fb_pending_acquire makes a consumer stream wait for a build
(the analogue of PendingAtmosphere::acquire_ownership, src/precompute.rs:2147),
so work enqueued there after it sees the finished tables without a host wait."""
import numpy as np
import pytest

from fuzzyblue_gb300.params import PRECISION_MIXED, smoke_parameters
from tests.golden.make_golden import tiny_parameters

pytestmark = pytest.mark.gpu


def _build(builder, params, stream):
    from fuzzyblue_gb300.api import build_batch
    return build_batch(builder, params, stream=stream)


def test_consumer_stream_sees_finished_tables(builder):
    import torch
    from fuzzyblue_gb300.api import Atmosphere
    producer, consumer = torch.cuda.Stream(), torch.cuda.Stream()
    params = [tiny_parameters().replace(order=4), smoke_parameters(precision=PRECISION_MIXED, order=5)]
    pend = _build(builder, params, producer)
    pend.acquire(consumer)  # no host wait: the consumer waits on the device
    copies = []
    with torch.cuda.stream(consumer):
        for i in range(len(params)):
            views = pend.atmosphere(i).device_views()
            copies.append({k: torch.as_tensor(v, device="cuda").clone() for k, v in views.items()})
    consumer.synchronize()
    for i, p in enumerate(params):
        ref = pend.atmosphere(i).to_host()
        for k in ref:
            assert np.array_equal(copies[i][k].cpu().numpy(), ref[k]), k
        alone = Atmosphere.build(builder, p)
        alone.wait()
        single = alone.atmosphere().to_host()
        alone.release()
        for k in ref:
            assert np.array_equal(single[k], ref[k]), k
    pend.release()


def test_build_on_a_caller_stream_then_query(builder):
    import torch
    from fuzzyblue_gb300.api import Atmosphere
    s = torch.cuda.Stream()
    pend = Atmosphere.build(builder, smoke_parameters(), stream=s)
    s.synchronize()
    assert pend.query()
    pend.release()


def test_async_copies_overlap_the_next_build(builder):
    """fb_atmosphere_copy_to_host_async enqueues the copies without a host
    wait: a build's copies on one stream and the next build on another give
    host tables equal to the blocking copy of the same atmospheres."""
    import torch
    s0, s1 = torch.cuda.Stream(), torch.cuda.Stream()
    params = [tiny_parameters().replace(order=3), smoke_parameters(precision=PRECISION_MIXED, order=4)]
    first = _build(builder, params, s0)
    hosts = []
    for i, p in enumerate(params):
        tw, th = p.transmittance_extent()
        iw, ih = p.irradiance_extent()
        sw, sh, sd = p.scattering_extent()
        h = {k: torch.empty(n * 4, dtype=torch.float32, pin_memory=True).numpy()
             for k, n in (("transmittance", tw * th), ("irradiance", iw * ih), ("scattering", sw * sh * sd))}
        first.atmosphere(i).copy_to_host_async(h["transmittance"], h["irradiance"], h["scattering"], stream=s0)
        hosts.append(h)
    second = _build(builder, list(reversed(params)), s1)  # runs while the copies are in flight
    s0.synchronize()
    for i in range(len(params)):
        ref = first.atmosphere(i).to_host()
        for k in ("transmittance", "irradiance", "scattering"):
            assert np.array_equal(hosts[i][k], ref[k].reshape(-1)), k
    second.wait()
    first.release()
    second.release()
