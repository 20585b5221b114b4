"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests, `__graft_entry__.smoke()` and bench.py's CPU-baseline leg import
this module. It loads oracle/_build/libfb_oracle.so (the C++ restatement) and,
when it was built, oracle/_ref/libfbref.so (the reference's own shader code
compiled as C++), building them on first use.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from fuzzyblue_gb300._native import c_draw_parameters  # noqa: E402
from fuzzyblue_gb300.params import Parameters, c_params  # noqa: E402
from oracle import build as _build  # noqa: E402

_lib = None
_ref = None
_ref_checked = False

_F = ctypes.POINTER(ctypes.c_float)
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int64)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(_build.build_oracle())
        P = ctypes.POINTER(c_params)
        L.fbo_precompute_f32.argtypes = [P, ctypes.c_int] + [_F] * 7
        L.fbo_precompute_f64.argtypes = [P, ctypes.c_int] + [_D] * 7
        L.fbo_transmittance_f32.argtypes = [P, ctypes.c_int, _I, ctypes.c_int64, _F]
        L.fbo_transmittance_f64.argtypes = [P, ctypes.c_int, _I, ctypes.c_int64, _D]
        L.fbo_direct_irradiance_f32.argtypes = [P, ctypes.c_int, _F, _I, ctypes.c_int64, _F]
        L.fbo_direct_irradiance_f64.argtypes = [P, ctypes.c_int, _D, _I, ctypes.c_int64, _D]
        L.fbo_single_scattering_f32.argtypes = [P, ctypes.c_int, _F, _I, ctypes.c_int64, _F, _F]
        L.fbo_single_scattering_f64.argtypes = [P, ctypes.c_int, _D, _I, ctypes.c_int64, _D, _D]
        L.fbo_indirect_irradiance_f64.argtypes = [P, ctypes.c_int, ctypes.c_int] + [_D] * 3 + [_I, ctypes.c_int64, _D]
        L.fbo_scattering_density_f32.argtypes = [P, ctypes.c_int, ctypes.c_int] + [_F] * 5 + [_I, ctypes.c_int64, _F]
        L.fbo_scattering_density_f64.argtypes = [P, ctypes.c_int, ctypes.c_int] + [_D] * 5 + [_I, ctypes.c_int64, _D]
        L.fbo_indirect_irradiance_f32.argtypes = [P, ctypes.c_int, ctypes.c_int] + [_F] * 3 + [_I, ctypes.c_int64, _F]
        L.fbo_multiple_scattering_f32.argtypes = [P, ctypes.c_int, _F, _F, _I, ctypes.c_int64, _F, _F]
        L.fbo_multiple_scattering_f64.argtypes = [P, ctypes.c_int, _D, _D, _I, ctypes.c_int64, _D, _D]
        L.fbo_params_default.argtypes = [P]
        L.fbo_count_ops.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, _D]
        DP = ctypes.POINTER(c_draw_parameters)
        L.fbo_render_sky_f32.argtypes = [P, _F, _F, DP, _F, ctypes.c_uint32, ctypes.c_uint32, _F, _F]
        L.fbo_render_sky_f64.argtypes = [P, _D, _D, DP, _D, ctypes.c_uint32, ctypes.c_uint32, _D, _D]
        L.fbo_sun_and_sky_irradiance_f32.argtypes = [P] + [_F] * 5 + [ctypes.c_int64, _F, _F]
        L.fbo_sun_and_sky_irradiance_f64.argtypes = [P] + [_D] * 5 + [ctypes.c_int64, _D, _D]
        _lib = L
    return _lib


def ref_lib():
    """The reference's shaders compiled as C++, or None if unavailable."""
    global _ref, _ref_checked
    if not _ref_checked:
        _ref_checked = True
        try:
            path = _build.build_reference()
        except RuntimeError:
            path = None
        if path:
            L = ctypes.CDLL(path)
            L.fbref_precompute.argtypes = [ctypes.POINTER(c_params)] + [_F] * 7
            L.fbref_render_sky.argtypes = [ctypes.POINTER(c_params), _F, _F, ctypes.POINTER(c_draw_parameters), _F,
                                           ctypes.c_uint32, ctypes.c_uint32, _F, _F]
            L.fbref_sun_and_sky_irradiance.argtypes = [ctypes.POINTER(c_params)] + [_F] * 5 + [ctypes.c_int64, _F, _F]
            _ref = L
    return _ref


def _ptr(a, kind):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(kind)


def _shapes(p: Parameters):
    tw, th = p.transmittance_extent()
    iw, ih = p.irradiance_extent()
    sw, sh, sd = p.scattering_extent()
    return (th, tw, 4), (ih, iw, 4), (sd, sh, sw, 4)


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed with status %d" % (what, rc))


def precompute(p: Parameters, dtype=np.float32, intermediates=False, nthreads=0, reference=False):
    """Full precompute. Returns a dict with 'transmittance', 'irradiance',
    'scattering' and, with intermediates=True, 'orders_ms' (order-1 tables),
    'orders_irr', 'single_rayleigh', 'single_mie'. reference=True runs the
    reference's shader code (float32 only)."""
    trs, irs, scs = _shapes(p)
    n = max(p.order - 1, 0)
    out = {
        "transmittance": np.zeros(trs, dtype),
        "irradiance": np.zeros(irs, dtype),
        "scattering": np.zeros(scs, dtype),
    }
    if intermediates:
        out["orders_ms"] = np.zeros((n,) + scs, dtype)
        out["orders_irr"] = np.zeros((n,) + irs, dtype)
        out["single_rayleigh"] = np.zeros(scs, dtype)
        out["single_mie"] = np.zeros(scs, dtype)
    kind = _F if dtype == np.float32 else _D
    args = [_ptr(out["transmittance"], kind), _ptr(out["irradiance"], kind), _ptr(out["scattering"], kind)]
    for k in ("orders_ms", "orders_irr", "single_rayleigh", "single_mie"):
        args.append(_ptr(out[k], kind) if intermediates and n >= 0 and out[k].size else None)
    c = p.to_c()
    if reference:
        R = ref_lib()
        if R is None:
            raise RuntimeError("reference shader build unavailable")
        assert dtype == np.float32
        _check(R.fbref_precompute(ctypes.byref(c), *args), "fbref_precompute")
    elif dtype == np.float32:
        _check(lib().fbo_precompute_f32(ctypes.byref(c), nthreads, *args), "fbo_precompute_f32")
    else:
        _check(lib().fbo_precompute_f64(ctypes.byref(c), nthreads, *args), "fbo_precompute_f64")
    return out


def _idx(idx):
    if idx is None:
        return None, 0
    a = np.ascontiguousarray(idx, dtype=np.int64)
    return a, a.size


def _kind(dtype):
    return (_F, "f32") if np.dtype(dtype) == np.float32 else (_D, "f64")


def transmittance(p, idx=None, nthreads=0, dtype=np.float32):
    a, n = _idx(idx)
    kind, sfx = _kind(dtype)
    cnt = n if a is not None else p.texel_counts()[0]
    out = np.zeros((cnt, 4), dtype)
    fn = getattr(lib(), "fbo_transmittance_" + sfx)
    _check(fn(ctypes.byref(p.to_c()), nthreads, _ptr(a, _I), n, _ptr(out, kind)), "transmittance")
    return out


def direct_irradiance(p, tr, idx=None, nthreads=0, dtype=np.float32):
    a, n = _idx(idx)
    kind, sfx = _kind(dtype)
    cnt = n if a is not None else p.texel_counts()[1]
    out = np.zeros((cnt, 4), dtype)
    tr = np.ascontiguousarray(tr, dtype)
    fn = getattr(lib(), "fbo_direct_irradiance_" + sfx)
    _check(fn(ctypes.byref(p.to_c()), nthreads, _ptr(tr, kind), _ptr(a, _I), n, _ptr(out, kind)), "direct_irradiance")
    return out


def single_scattering(p, tr, idx=None, nthreads=0, dtype=np.float32):
    a, n = _idx(idx)
    kind, sfx = _kind(dtype)
    cnt = n if a is not None else p.texel_counts()[2]
    r = np.zeros((cnt, 4), dtype)
    m = np.zeros((cnt, 4), dtype)
    tr = np.ascontiguousarray(tr, dtype)
    fn = getattr(lib(), "fbo_single_scattering_" + sfx)
    _check(fn(ctypes.byref(p.to_c()), nthreads, _ptr(tr, kind), _ptr(a, _I), n, _ptr(r, kind), _ptr(m, kind)),
           "single_scattering")
    return r, m


def scattering_density(p, order, tr, single_r, single_m, multiple, delta_irr, idx=None, nthreads=0,
                       dtype=np.float32):
    a, n = _idx(idx)
    cnt = n if a is not None else p.texel_counts()[2]
    kind = _F if dtype == np.float32 else _D
    out = np.zeros((cnt, 4), dtype)
    conv = [None if x is None else np.ascontiguousarray(x, dtype) for x in (tr, single_r, single_m, multiple, delta_irr)]
    fn = lib().fbo_scattering_density_f32 if dtype == np.float32 else lib().fbo_scattering_density_f64
    _check(fn(ctypes.byref(p.to_c()), nthreads, order, *[_ptr(x, kind) for x in conv], _ptr(a, _I), n,
              _ptr(out, kind)), "scattering_density")
    return out


def indirect_irradiance(p, order, single_r, single_m, multiple, idx=None, nthreads=0, dtype=np.float32):
    a, n = _idx(idx)
    kind, sfx = _kind(dtype)
    cnt = n if a is not None else p.texel_counts()[1]
    out = np.zeros((cnt, 4), dtype)
    conv = [None if x is None else np.ascontiguousarray(x, dtype) for x in (single_r, single_m, multiple)]
    fn = getattr(lib(), "fbo_indirect_irradiance_" + sfx)
    _check(fn(ctypes.byref(p.to_c()), nthreads, order, *[_ptr(x, kind) for x in conv], _ptr(a, _I), n,
              _ptr(out, kind)), "indirect_irradiance")
    return out


def multiple_scattering(p, tr, density, idx=None, nthreads=0, dtype=np.float32):
    a, n = _idx(idx)
    cnt = n if a is not None else p.texel_counts()[2]
    kind = _F if dtype == np.float32 else _D
    out = np.zeros((cnt, 4), dtype)
    phase = np.zeros((cnt,), dtype)
    tr = np.ascontiguousarray(tr, dtype)
    density = np.ascontiguousarray(density, dtype)
    fn = lib().fbo_multiple_scattering_f32 if dtype == np.float32 else lib().fbo_multiple_scattering_f64
    _check(fn(ctypes.byref(p.to_c()), nthreads, _ptr(tr, kind), _ptr(density, kind), _ptr(a, _I), n,
              _ptr(out, kind), _ptr(phase, kind)), "multiple_scattering")
    return out, phase


def default_params_c() -> c_params:
    c = c_params()
    lib().fbo_params_default(ctypes.byref(c))
    return c


PASSES = ("transmittance", "direct_irradiance", "single_scattering", "scattering_density",
          "indirect_irradiance", "multiple_scattering")


def count_ops(p: Parameters, pass_name: str, order: int = 3, samples: int = 256, seed: int = 0) -> dict:
    """Shader arithmetic per texel of one pass of the reference's algorithm
    (oracle op count; sampler filtering excluded): adds, muls, divs, sqrts,
    transcendentals, and `flops`, their sum."""
    out = np.zeros(5, np.float64)
    c = p.to_c()
    _check(lib().fbo_count_ops(ctypes.byref(c), PASSES.index(pass_name), order, samples, seed, _ptr(out, _D)),
           "fbo_count_ops")
    d = dict(zip(("add", "mul", "div", "sqrt", "transc"), out.tolist()))
    d["flops"] = float(out.sum())
    return d


def render_sky(p: Parameters, transmittance, scattering, draw, width, height, depth=None, dtype=np.float32,
               reference=False):
    """The sky pass (render_sky.frag over render_sky.h) on host tables:
    (radiance, transmittance) arrays (height, width, 4). reference=True runs
    the reference's own shading code compiled as C++ (FP32)."""
    kind = _F if dtype == np.float32 else _D
    tr = np.ascontiguousarray(transmittance, dtype)
    sc = np.ascontiguousarray(scattering, dtype)
    dep = None if depth is None else np.ascontiguousarray(depth, dtype)
    color = np.zeros((height, width, 4), dtype)
    trans = np.zeros((height, width, 4), dtype)
    c = draw.to_c()
    if reference:
        L = ref_lib()
        if L is None:
            raise RuntimeError("the reference's shaders are not available")
        fn = L.fbref_render_sky
    else:
        fn = lib().fbo_render_sky_f32 if dtype == np.float32 else lib().fbo_render_sky_f64
    _check(fn(ctypes.byref(p.to_c()), _ptr(tr, kind), _ptr(sc, kind), ctypes.byref(c), _ptr(dep, kind), width,
              height, _ptr(color, kind), _ptr(trans, kind)), "render_sky")
    return color, trans


def sun_and_sky_irradiance(p: Parameters, transmittance, irradiance, points, normals, sun_direction,
                           dtype=np.float32, reference=False):
    """GetSunAndSkyIrradiance (render_lighting.h) at points (n, 3): (sun, sky) arrays (n, 3)."""
    kind = _F if dtype == np.float32 else _D
    tr = np.ascontiguousarray(transmittance, dtype)
    ir = np.ascontiguousarray(irradiance, dtype)
    pts = np.ascontiguousarray(points, dtype)
    nrm = np.ascontiguousarray(normals, dtype)
    sun = np.ascontiguousarray(sun_direction, dtype)
    n = pts.shape[0]
    out_sun = np.zeros((n, 3), dtype)
    out_sky = np.zeros((n, 3), dtype)
    if reference:
        L = ref_lib()
        if L is None:
            raise RuntimeError("the reference's shaders are not available")
        fn = L.fbref_sun_and_sky_irradiance
    else:
        fn = lib().fbo_sun_and_sky_irradiance_f32 if dtype == np.float32 else lib().fbo_sun_and_sky_irradiance_f64
    _check(fn(ctypes.byref(p.to_c()), _ptr(tr, kind), _ptr(ir, kind), _ptr(pts, kind), _ptr(nrm, kind),
              _ptr(sun, kind), n, _ptr(out_sun, kind), _ptr(out_sky, kind)), "sun_and_sky_irradiance")
    return out_sun, out_sky

