"""Seeded synthetic atmospheres for the batched and served benchmarks.

The reference publishes no dataset; these generators draw atmospheres from the
distributions its benchmark configurations name, converted to the crate's units
(km and 1/km; a coefficient in 1/m is multiplied by 1e3):

  bottom radius           uniform 3000-8000 km
  atmosphere thickness    uniform 40-120 km
  Rayleigh scale height   uniform 4-12 km     (exp_scale = -1/H)
  Mie scale height        uniform 0.5-3 km
  Rayleigh RGB scattering Earth value times ONE log-uniform factor in [0.2, 5]
  Mie scattering          log-uniform 1e-6-5e-5 /m; extinction = scattering / albedo,
                          albedo uniform 0.8-1.0
  Mie phase g             uniform 0.6-0.9
  ozone absorption        Earth value times uniform 0-3 (tent profile kept)
  sun, solar irradiance, ground albedo, mu_s_min: Parameters::default()

Draw order per atmosphere (fixed): R, thickness, H_R, H_M, rayleigh factor,
mie scattering, albedo, g, ozone factor. Table classes:
  "default"  Parameters::default() sizes (TR 256x64, IR 64x16, SC 32x128x32x8)
  "half"     TR 128x32, SC r16 mu64 mu_s16 nu4, IR 64x16
  "double"   TR 512x128 (2000 steps), IR 128x32, SC r64 mu256 mu_s64 nu16
"""
from __future__ import annotations

from typing import List

import numpy as np

from .params import DensityProfile, DensityProfileLayer, Parameters, PRECISION_MIXED

EARTH_RAYLEIGH = (0.005802, 0.013558, 0.033100)
EARTH_OZONE = (6.5e-4, 1.881e-3, 8.5e-5)

CLASSES = {
    "default": {},
    "half": dict(transmittance_mu_size=128, transmittance_r_size=32, scattering_r_size=16,
                 scattering_mu_size=64, scattering_mu_s_size=16, scattering_nu_size=4),
    "double": dict(transmittance_mu_size=512, transmittance_r_size=128, transmittance_steps=2000,
                   irradiance_mu_s_size=128, irradiance_r_size=32, scattering_r_size=64,
                   scattering_mu_size=256, scattering_mu_s_size=64, scattering_nu_size=16),
}


def _loguniform(rng, lo, hi):
    return float(np.exp(rng.uniform(np.log(lo), np.log(hi))))


def draw_atmosphere(rng: np.random.Generator, **overrides) -> Parameters:
    R = float(rng.uniform(3000.0, 8000.0))
    thickness = float(rng.uniform(40.0, 120.0))
    h_r = float(rng.uniform(4.0, 12.0))
    h_m = float(rng.uniform(0.5, 3.0))
    f_r = _loguniform(rng, 0.2, 5.0)
    mie = _loguniform(rng, 1e-6, 5e-5) * 1e3  # 1/m -> 1/km
    albedo = float(rng.uniform(0.8, 1.0))
    g = float(rng.uniform(0.6, 0.9))
    f_o = float(rng.uniform(0.0, 3.0))
    p = Parameters(
        bottom_radius=R, top_radius=R + thickness,
        rayleigh_density=DensityProfile([DensityProfileLayer(), DensityProfileLayer(exp_term=1.0, exp_scale=-1.0 / h_r)]),
        rayleigh_scattering=tuple(f_r * c for c in EARTH_RAYLEIGH),
        mie_density=DensityProfile([DensityProfileLayer(), DensityProfileLayer(exp_term=1.0, exp_scale=-1.0 / h_m)]),
        mie_scattering=(mie,) * 3, mie_extinction=(mie / albedo,) * 3, mie_phase_function_g=g,
        absorbtion_extinction=tuple(f_o * c for c in EARTH_OZONE),
    )
    return p.replace(**overrides) if overrides else p


def uniform_batch(n: int = 256, seed: int = 0, order: int = 4, precision: int = PRECISION_MIXED) -> List[Parameters]:
    """n atmospheres at the default table sizes, `order` bounces."""
    rng = np.random.default_rng(seed)
    return [draw_atmosphere(rng, order=order, precision=precision) for _ in range(n)]


def uneven_batch(n: int = 96, seed: int = 1, precision: int = PRECISION_MIXED) -> List[Parameters]:
    """n atmospheres split evenly over the three table classes, orders uniform in 2-8."""
    rng = np.random.default_rng(seed)
    names = ["default", "half", "double"]
    out = []
    for i in range(n):
        p = draw_atmosphere(rng, precision=precision)
        order = int(rng.integers(2, 9))
        out.append(p.replace(order=order, **CLASSES[names[i % 3]]))
    return out


def serving_request(rng: np.random.Generator, precision: int = PRECISION_MIXED) -> Parameters:
    """One request of the serving workload: class drawn 60/30/10 from
    default/half/double, orders uniform in 2-8."""
    p = draw_atmosphere(rng, precision=precision)
    u = float(rng.uniform())
    cls = "default" if u < 0.6 else ("half" if u < 0.9 else "double")
    return p.replace(order=int(rng.integers(2, 9)), **CLASSES[cls])
