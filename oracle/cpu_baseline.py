"""Bounded-sample CPU timing of one atmosphere precompute (TEST INFRASTRUCTURE:
only bench.py's CPU-baseline leg and its reference arm call this).

Timing a whole default-size atmosphere on the host takes minutes, so every pass
is timed on a fixed random subset of its output texels and scaled by the
texel count and by the number of times the pass runs (orders). Inputs of the
later passes are synthetic constant tables: the cost per texel of the
reference's quadratures does not depend on the table values.

impl = "reference": the reference's own shader code compiled as C++
           (oracle/_ref, see oracle/ref_glsl), through fbref_run_pass;
       "port":      the oracle's C++ restatement (oracle/fb_oracle.cpp).
"""
from __future__ import annotations

import ctypes
import os
import time

import numpy as np

from fuzzyblue_gb300.params import Parameters, c_params
from oracle import py_oracle

_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int64)


def reference_available() -> bool:
    return _ref() is not None


def _ref():
    L = py_oracle.ref_lib()
    if L is not None and not getattr(L, "_run_pass_typed", False):
        L.fbref_run_pass.argtypes = [ctypes.c_int, ctypes.POINTER(c_params), ctypes.c_int] + [_F] * 8 + [
            _I, ctypes.c_int64]
        L._run_pass_typed = True
    return L


def _subset(rng, n, frac, minimum=8):
    k = int(min(n, max(minimum, round(n * frac))))
    return np.sort(rng.choice(n, size=k, replace=False)).astype(np.int64)


def threads_available() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def estimate(p: Parameters, impl: str = "port", fraction: float = 1.0 / 32, seed: int = 0) -> dict:
    """Seconds one atmosphere takes on the host, estimated from a sample."""
    rng = np.random.default_rng(seed)
    ntr, nir, nsc = p.texel_counts()
    tw, th = p.transmittance_extent()
    iw, ih = p.irradiance_extent()
    sw, sh, sd = p.scattering_extent()
    c = p.to_c()
    # inputs: the full transmittance table (untimed), constant tables for the rest
    tr = py_oracle.transmittance(p).reshape(th, tw, 4)
    dirr = np.full((ih, iw, 4), 1e-2, np.float32)
    big = lambda: np.full((sd, sh, sw, 4), 1e-3, np.float32)
    dr, dm, dms, dens, sc = big(), big(), big(), big(), big()
    ir = np.zeros((ih, iw, 4), np.float32)
    ptr = lambda a: a.ctypes.data_as(_F)
    sets = {
        "transmittance": (_subset(rng, ntr, fraction), ntr, 1),
        "direct": (np.arange(nir, dtype=np.int64), nir, 1),
        "single": (_subset(rng, nsc, fraction), nsc, 1),
        "density2": (_subset(rng, nsc, fraction / 4), nsc, 1 if p.order >= 2 else 0),
        "density3": (_subset(rng, nsc, fraction / 4), nsc, max(p.order - 2, 0)),
        "indirect1": (_subset(rng, nir, fraction * 4), nir, 1 if p.order >= 2 else 0),
        "indirect2": (_subset(rng, nir, fraction * 4), nir, max(p.order - 2, 0)),
        "multiple": (_subset(rng, nsc, fraction), nsc, max(p.order - 1, 0)),
    }
    timings = {}
    if impl == "reference":
        R = _ref()
        if R is None:
            raise RuntimeError("reference shader build unavailable")
        calls = {
            "transmittance": (0, 0), "direct": (1, 0), "single": (2, 0), "density2": (3, 2),
            "density3": (3, 3), "indirect1": (4, 1), "indirect2": (4, 2), "multiple": (5, 0),
        }
        trc = tr.copy()
        for name, (idx, total, reps) in sets.items():
            if reps == 0:
                continue
            pass_id, order = calls[name]
            target = trc if pass_id == 0 else tr
            t0 = time.perf_counter()
            rc = R.fbref_run_pass(pass_id, ctypes.byref(c), order, ptr(target), ptr(dirr), ptr(dr), ptr(dm), ptr(dms),
                                  ptr(dens), ptr(ir), ptr(sc), idx.ctypes.data_as(_I), idx.size)
            dt = time.perf_counter() - t0
            if rc != 0:
                raise RuntimeError("fbref_run_pass(%d) failed: %d" % (pass_id, rc))
            timings[name] = (dt, idx.size, total, reps)
    else:
        O = py_oracle
        fns = {
            "transmittance": lambda idx: O.transmittance(p, idx),
            "direct": lambda idx: O.direct_irradiance(p, tr, idx),
            "single": lambda idx: O.single_scattering(p, tr, idx),
            "density2": lambda idx: O.scattering_density(p, 2, tr, dr, dm, None, dirr, idx),
            "density3": lambda idx: O.scattering_density(p, 3, tr, None, None, dms, dirr, idx),
            "indirect1": lambda idx: O.indirect_irradiance(p, 1, dr, dm, None, idx),
            "indirect2": lambda idx: O.indirect_irradiance(p, 2, None, None, dms, idx),
            "multiple": lambda idx: O.multiple_scattering(p, tr, dens, idx),
        }
        for name, (idx, total, reps) in sets.items():
            if reps == 0:
                continue
            t0 = time.perf_counter()
            fns[name](idx)
            timings[name] = (time.perf_counter() - t0, idx.size, total, reps)
    est = sum(dt / n * total * reps for (dt, n, total, reps) in timings.values())
    measured = sum(dt for (dt, _, _, _) in timings.values())
    return {
        "seconds_per_atmosphere": est,
        "sample_seconds": measured,
        "threads": threads_available(),
        "passes": {k: {"sample_texels": int(n), "texels": int(t), "runs": int(r), "seconds": round(dt, 4)}
                   for k, (dt, n, t, r) in timings.items()},
        "sample": "every pass of one atmosphere on a fixed random %.4g of its texels (density %.4g, indirect %.4g), "
                  "scaled by texel count and order count; %.1f s on the host" % (
                      min(fraction, 1.0), min(fraction / 4, 1.0), min(fraction * 4, 1.0), measured),
    }
