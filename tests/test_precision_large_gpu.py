"""MIXED precision at 4x table resolution (transmittance 512x128 with 2000
steps, irradiance 128x32, scattering r64 mu256 mu_s64 nu16) on the Earth
atmosphere: every pass against the FP64 oracle, fed the GPU's own inputs.

A whole FP64 precompute at this size is out of reach of the CPU oracle (about
10^11 direction evaluations per order), so each pass is checked on its own:
transmittance, direct and indirect irradiance on every texel, single
scattering, scattering density (orders 2 and 3) and multiple scattering
(orders 2 and 3) on 4096 texels drawn with a fixed seed. The end-to-end error
of an order is bounded by the sum of its passes' errors; every pass must meet
the 1e-3 target. The per-pass figures are printed (pytest -s)."""
import numpy as np
import pytest

from fuzzyblue_gb300 import workloads
from fuzzyblue_gb300.params import PRECISION_MIXED, Parameters
from tests.errors import summary

pytestmark = pytest.mark.gpu

MIXED_MAX = 1e-3
SAMPLES = 4096


def _build(builder, p):
    from fuzzyblue_gb300.api import Atmosphere
    pend = Atmosphere.build(builder, p)
    pend.wait()
    out = pend.atmosphere().to_host()
    out.update({k: v.to_numpy() for k, v in pend.intermediates().items()})
    pend.release()
    return out


def test_mixed_passes_at_4x_resolution_meet_fp64_target(builder, oracle):
    p0 = Parameters(precision=PRECISION_MIXED).replace(**workloads.CLASSES["double"])
    b = {n: _build(builder, p0.replace(order=n)) for n in (1, 2, 3)}
    f64 = np.float64
    ntr, nir, nsc = p0.texel_counts()
    rng = np.random.default_rng(7)
    idx = np.sort(rng.choice(nsc, SAMPLES, replace=False)).astype(np.int64)

    def flat(a):
        return a.reshape(-1, 4)

    rows = []

    def check(name, gpu, ref):
        s = summary(gpu.astype(np.float64), ref)
        rows.append((name, s))
        assert np.isfinite(gpu).all(), name
        assert s["max"] <= MIXED_MAX, (name, s)

    tr = flat(b[1]["transmittance"]).astype(f64)
    check("transmittance (all texels)", flat(b[1]["transmittance"]), oracle.transmittance(p0, dtype=f64))
    d0 = flat(b[1]["delta_irradiance_0"]).astype(f64)
    check("direct irradiance (all)", d0, oracle.direct_irradiance(p0, tr, dtype=f64))
    dr, dm = flat(b[1]["delta_rayleigh"]).astype(f64), flat(b[1]["delta_mie"]).astype(f64)
    r, m = oracle.single_scattering(p0, tr, idx=idx, dtype=f64)
    check("single Rayleigh (sampled)", dr[idx], r)
    check("single Mie (sampled)", dm[idx], m)
    prev_ms, prev_e = None, d0
    for n in (2, 3):
        dens = flat(b[n]["scattering_density"]).astype(f64)
        if n == 2:
            ref = oracle.scattering_density(p0, 2, tr, dr, dm, None, prev_e, idx=idx, dtype=f64)
        else:
            ref = oracle.scattering_density(p0, n, tr, None, None, prev_ms, prev_e, idx=idx, dtype=f64)
        check("density order %d (sampled)" % n, dens[idx], ref)
        e_n = flat(b[n]["delta_irradiance_%d" % ((n + 1) & 1)]).astype(f64)
        if n == 2:
            ref = oracle.indirect_irradiance(p0, 1, dr, dm, None, dtype=f64)
        else:
            ref = oracle.indirect_irradiance(p0, n - 1, None, None, prev_ms, dtype=f64)
        check("indirect irradiance order %d (all)" % (n - 1), e_n, ref)
        ms = flat(b[n]["delta_multiple_scattering"]).astype(f64)
        ref, _ = oracle.multiple_scattering(p0, tr, dens, idx=idx, dtype=f64)
        check("multiple order %d (sampled)" % n, ms[idx], ref)
        prev_ms, prev_e = ms, e_n
    print()
    for name, s in rows:
        print("  %-36s max %.2e  rms %.2e  p99.9 %.2e" % (name, s["max"], s["rms"], s["p999"]))
