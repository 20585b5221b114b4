"""Atmosphere parameters: the host-side mirror of the crate's parameter API.

`Parameters`, `DensityProfile` and `DensityProfileLayer` keep the field names,
units (km, 1/km) and defaults of src/precompute.rs:655-935, including the
reference's spelling `absorbtion_density` / `absorbtion_extinction`. The
Vulkan-only fields (`usage`, `dst_stage_mask`, `dst_access_mask`, `layout`,
src/precompute.rs:691-698) are accepted and ignored. Extra fields carry what
the reference fixes in its shaders (sample counts) plus the precision and
storage modes of this library.

`Parameters.to_c()` packs the 384-byte `fb_params` of include/fuzzyblue.h,
whose first 320 bytes are the ParamsRaw uniform block
(src/precompute.rs:937-1033).
"""
from __future__ import annotations

import ctypes
import dataclasses
from dataclasses import dataclass, field
from typing import List, Tuple

PRECISION_PLAIN = 0
PRECISION_MIXED = 1
STORAGE_F32 = 0
STORAGE_F16 = 1


class c_density_profile_layer(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_float),
        ("exp_term", ctypes.c_float),
        ("exp_scale", ctypes.c_float),
        ("linear_term", ctypes.c_float),
        ("constant_term", ctypes.c_float),
        ("_pad", ctypes.c_float * 3),
    ]


class c_density_profile(ctypes.Structure):
    _fields_ = [("layers", c_density_profile_layer * 2)]


class c_params_raw(ctypes.Structure):
    _fields_ = [
        ("solar_irradiance", ctypes.c_float * 3),
        ("sun_angular_radius", ctypes.c_float),
        ("rayleigh_scattering", ctypes.c_float * 3),
        ("bottom_radius", ctypes.c_float),
        ("mie_scattering", ctypes.c_float * 3),
        ("top_radius", ctypes.c_float),
        ("mie_extinction", ctypes.c_float * 3),
        ("mie_phase_function_g", ctypes.c_float),
        ("ground_albedo", ctypes.c_float * 3),
        ("mu_s_min", ctypes.c_float),
        ("absorption_extinction", ctypes.c_float * 3),
        ("transmittance_mu_size", ctypes.c_uint32),
        ("transmittance_r_size", ctypes.c_uint32),
        ("scattering_r_size", ctypes.c_uint32),
        ("scattering_mu_size", ctypes.c_uint32),
        ("scattering_mu_s_size", ctypes.c_uint32),
        ("scattering_nu_size", ctypes.c_uint32),
        ("irradiance_mu_s_size", ctypes.c_uint32),
        ("irradiance_r_size", ctypes.c_uint32),
        ("_pad0", ctypes.c_uint32),
        ("rayleigh_density", c_density_profile),
        ("mie_density", c_density_profile),
        ("absorption_density", c_density_profile),
    ]


class c_params(ctypes.Structure):
    _fields_ = [
        ("raw", c_params_raw),
        ("order", ctypes.c_uint32),
        ("transmittance_steps", ctypes.c_uint32),
        ("single_scattering_steps", ctypes.c_uint32),
        ("multiple_scattering_steps", ctypes.c_uint32),
        ("density_samples", ctypes.c_uint32),
        ("irradiance_samples", ctypes.c_uint32),
        ("precision", ctypes.c_uint32),
        ("storage", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32 * 8),
    ]


assert ctypes.sizeof(c_params_raw) == 320
assert ctypes.sizeof(c_params) == 384


@dataclass
class DensityProfileLayer:
    """One layer: clamp(exp_term*exp(exp_scale*h) + linear_term*h + constant_term, 0, 1)
    (src/precompute.rs:655-666, shaders/params.h:6-15)."""
    width: float = 0.0
    exp_term: float = 0.0
    exp_scale: float = 0.0
    linear_term: float = 0.0
    constant_term: float = 0.0


@dataclass
class DensityProfile:
    """Two layers, bottom to top (src/precompute.rs:668-676)."""
    layers: List[DensityProfileLayer] = field(
        default_factory=lambda: [DensityProfileLayer(), DensityProfileLayer()])


def _exp_profile(scale: float) -> DensityProfile:
    return DensityProfile([DensityProfileLayer(), DensityProfileLayer(exp_term=1.0, exp_scale=scale)])


def _ozone_profile() -> DensityProfile:
    return DensityProfile([
        DensityProfileLayer(width=25.0, linear_term=0.066667, constant_term=-0.666667),
        DensityProfileLayer(linear_term=-0.066667, constant_term=2.666667),
    ])


@dataclass
class Parameters:
    """Parameters governing generated skies; distances in km
    (src/precompute.rs:678-769, defaults src/precompute.rs:849-935)."""
    # Vulkan-only fields of the reference; no meaning here.
    usage: object = None
    dst_stage_mask: object = None
    dst_access_mask: object = None
    layout: object = None

    order: int = 4
    transmittance_mu_size: int = 256
    transmittance_r_size: int = 64
    scattering_r_size: int = 32
    scattering_mu_size: int = 128
    scattering_mu_s_size: int = 32
    scattering_nu_size: int = 8
    irradiance_mu_s_size: int = 64
    irradiance_r_size: int = 16

    solar_irradiance: Tuple[float, float, float] = (1.474, 1.850, 1.91198)
    sun_angular_radius: float = 0.004675
    bottom_radius: float = 6360.0
    top_radius: float = 6420.0
    rayleigh_density: DensityProfile = field(default_factory=lambda: _exp_profile(-0.125))
    rayleigh_scattering: Tuple[float, float, float] = (0.005802, 0.013558, 0.033100)
    mie_density: DensityProfile = field(default_factory=lambda: _exp_profile(-0.833333))
    mie_scattering: Tuple[float, float, float] = (0.003996, 0.003996, 0.003996)
    mie_extinction: Tuple[float, float, float] = (0.004440, 0.004440, 0.004440)
    mie_phase_function_g: float = 0.8
    absorbtion_density: DensityProfile = field(default_factory=_ozone_profile)
    absorbtion_extinction: Tuple[float, float, float] = (6.5e-4, 1.881e-3, 8.5e-5)
    ground_albedo: Tuple[float, float, float] = (0.1, 0.1, 0.1)
    mu_s_min: float = -0.207912

    # Fixed by the reference's shaders; runtime fields here.
    transmittance_steps: int = 500       # transmittance.comp:14
    single_scattering_steps: int = 50    # single_scattering.comp:42
    multiple_scattering_steps: int = 50  # multiple_scattering.comp:21
    density_samples: int = 16            # scattering_density.comp:34
    irradiance_samples: int = 32         # indirect_irradiance.comp:20
    precision: int = PRECISION_PLAIN
    storage: int = STORAGE_F32

    # Parameters::*_extent (src/precompute.rs:771-793)
    def transmittance_extent(self) -> Tuple[int, int]:
        return (self.transmittance_mu_size, self.transmittance_r_size)

    def irradiance_extent(self) -> Tuple[int, int]:
        return (self.irradiance_mu_s_size, self.irradiance_r_size)

    def scattering_extent(self) -> Tuple[int, int, int]:
        return (self.scattering_nu_size * self.scattering_mu_s_size, self.scattering_mu_size,
                self.scattering_r_size)

    # Spelling aliases.
    @property
    def absorption_density(self) -> DensityProfile:
        return self.absorbtion_density

    @property
    def absorption_extinction(self):
        return self.absorbtion_extinction

    def replace(self, **kw) -> "Parameters":
        return dataclasses.replace(self, **kw)

    def to_c(self) -> c_params:
        c = c_params()
        r = c.raw

        def put3(dst, v):
            for i in range(3):
                dst[i] = float(v[i])

        def put_profile(dst, prof):
            for i in range(2):
                L = prof.layers[i]
                d = dst.layers[i]
                d.width, d.exp_term, d.exp_scale = L.width, L.exp_term, L.exp_scale
                d.linear_term, d.constant_term = L.linear_term, L.constant_term

        put3(r.solar_irradiance, self.solar_irradiance)
        r.sun_angular_radius = self.sun_angular_radius
        put3(r.rayleigh_scattering, self.rayleigh_scattering)
        r.bottom_radius = self.bottom_radius
        put3(r.mie_scattering, self.mie_scattering)
        r.top_radius = self.top_radius
        put3(r.mie_extinction, self.mie_extinction)
        r.mie_phase_function_g = self.mie_phase_function_g
        put3(r.ground_albedo, self.ground_albedo)
        r.mu_s_min = self.mu_s_min
        put3(r.absorption_extinction, self.absorbtion_extinction)
        r.transmittance_mu_size = self.transmittance_mu_size
        r.transmittance_r_size = self.transmittance_r_size
        r.scattering_r_size = self.scattering_r_size
        r.scattering_mu_size = self.scattering_mu_size
        r.scattering_mu_s_size = self.scattering_mu_s_size
        r.scattering_nu_size = self.scattering_nu_size
        r.irradiance_mu_s_size = self.irradiance_mu_s_size
        r.irradiance_r_size = self.irradiance_r_size
        put_profile(r.rayleigh_density, self.rayleigh_density)
        put_profile(r.mie_density, self.mie_density)
        put_profile(r.absorption_density, self.absorbtion_density)
        c.order = self.order
        c.transmittance_steps = self.transmittance_steps
        c.single_scattering_steps = self.single_scattering_steps
        c.multiple_scattering_steps = self.multiple_scattering_steps
        c.density_samples = self.density_samples
        c.irradiance_samples = self.irradiance_samples
        c.precision = self.precision
        c.storage = self.storage
        return c

    def texel_counts(self) -> Tuple[int, int, int]:
        tw, th = self.transmittance_extent()
        iw, ih = self.irradiance_extent()
        sw, sh, sd = self.scattering_extent()
        return tw * th, iw * ih, sw * sh * sd


def smoke_parameters(**kw) -> Parameters:
    """The reduced atmosphere of the reference's integration test and bench:
    r=8, mu=32, mu_s=8, nu=2, defaults otherwise (tests/smoke.rs:132-143,
    benches/precompute.rs:123-134)."""
    return Parameters(scattering_r_size=8, scattering_mu_size=32, scattering_mu_s_size=8,
                      scattering_nu_size=2, **kw)


def dump_parameters(**kw) -> Parameters:
    """The table sizes of the reference's LUT dump example: r=16, mu=64,
    mu_s=16, nu=4, order 4 (examples/dump.rs:96-108)."""
    return Parameters(scattering_r_size=16, scattering_mu_size=64, scattering_mu_s_size=16,
                      scattering_nu_size=4, **kw)
