"""fb_atmosphere_build_noalloc: the build for callers that may not allocate
device memory (an engine owning every allocation, a render loop that cannot
afford an allocation's synchronisation). It must give the same tables as the
allocating entry point, call after call, although every call reuses one fixed
scratch array. This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from fuzzyblue_gb300.params import PRECISION_MIXED, dump_parameters, smoke_parameters
from tests.errors import summary

pytestmark = pytest.mark.gpu
PLAIN_MAX = 2e-3  # the tolerance of the parity tests; the two paths should agree exactly


def _reference_tables(builder, p):
    from fuzzyblue_gb300.api import Atmosphere
    pend = Atmosphere.build(builder, p)
    pend.wait()
    out = pend.atmosphere().to_host()
    pend.release()
    return out


def _noalloc_tables(lib, p):
    import torch
    tw, th = p.transmittance_extent()
    iw, ih = p.irradiance_extent()
    sw, sh, sd = p.scattering_extent()
    # the caller owns the outputs (allocated here by the test, not by the entry point)
    tr = torch.zeros((th, tw, 4), dtype=torch.float32, device="cuda")
    ir = torch.zeros((ih, iw, 4), dtype=torch.float32, device="cuda")
    sc = torch.zeros((sd, sh, sw, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    c = p.to_c()
    rc = lib.fb_atmosphere_build_noalloc(ctypes.c_void_p(stream.cuda_stream), ctypes.byref(c),
                                         ctypes.c_void_p(tr.data_ptr()), ctypes.c_void_p(ir.data_ptr()),
                                         ctypes.c_void_p(sc.data_ptr()))
    assert rc == 0, lib.fb_last_error()
    torch.cuda.synchronize()
    return {"transmittance": tr.cpu().numpy(), "irradiance": ir.cpu().numpy(), "scattering": sc.cpu().numpy()}


def test_noalloc_matches_allocating_build_twice(native_lib):
    import torch
    from fuzzyblue_gb300.api import Builder
    torch.cuda.set_device(0)
    b = Builder(0)
    # two calls in a row with different table sizes and precision: the second
    # reuses the scratch the first one left behind
    for p in (smoke_parameters(), dump_parameters(precision=PRECISION_MIXED)):
        ref = _reference_tables(b, p)
        got = _noalloc_tables(native_lib, p)
        for k in ("transmittance", "irradiance", "scattering"):
            assert summary(got[k], ref[k])["max"] <= PLAIN_MAX, k
            assert np.array_equal(got[k], ref[k]), k
    b.close()


def test_noalloc_refuses_builds_beyond_its_scratch(native_lib):
    import torch
    from fuzzyblue_gb300 import _native as N
    from fuzzyblue_gb300.params import Parameters
    torch.cuda.set_device(0)
    p = Parameters()  # default sizes need far more than the fixed scratch
    c = p.to_c()
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = native_lib.fb_atmosphere_build_noalloc(None, ctypes.byref(c), ctypes.c_void_p(buf.data_ptr()),
                                                ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()))
    assert rc == N.FB_ERR_BUDGET
    assert b"scratch" in native_lib.fb_last_error()


def test_noalloc_error_enqueues_nothing(native_lib):
    """A build whose second pass cannot run (single scattering with 1024 steps
    on rows of 16 texels needs more shared memory than a CTA can have) is
    refused before anything is enqueued: the caller's tables keep their
    contents, and the next call still builds correctly."""
    import torch
    from fuzzyblue_gb300 import _native as N
    from fuzzyblue_gb300.api import Builder
    torch.cuda.set_device(0)
    p = smoke_parameters().replace(single_scattering_steps=1024)
    tw, th = p.transmittance_extent()
    iw, ih = p.irradiance_extent()
    sw, sh, sd = p.scattering_extent()
    sentinel = 1234.5
    tr = torch.full((th, tw, 4), sentinel, dtype=torch.float32, device="cuda")
    ir = torch.full((ih, iw, 4), sentinel, dtype=torch.float32, device="cuda")
    sc = torch.full((sd, sh, sw, 4), sentinel, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    c = p.to_c()
    rc = native_lib.fb_atmosphere_build_noalloc(ctypes.c_void_p(stream.cuda_stream), ctypes.byref(c),
                                                ctypes.c_void_p(tr.data_ptr()), ctypes.c_void_p(ir.data_ptr()),
                                                ctypes.c_void_p(sc.data_ptr()))
    assert rc == N.FB_ERR_INVALID_PARAMS, native_lib.fb_last_error()
    assert b"shared memory" in native_lib.fb_last_error()
    torch.cuda.synchronize()
    for t in (tr, ir, sc):
        assert bool((t == sentinel).all())
    b = Builder(0)
    q = smoke_parameters()
    ref = _reference_tables(b, q)
    got = _noalloc_tables(native_lib, q)
    for k in ("transmittance", "irradiance", "scattering"):
        assert np.array_equal(got[k], ref[k]), k
    b.close()
