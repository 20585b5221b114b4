"""Generates the golden vectors in tests/golden/.

The vectors are outputs of the reference's OWN shader code: the six compute
shaders and their headers, compiled on the host through
oracle/ref_glsl/translate.py + glsl_shim.hpp (oracle/build.py), run in the
pass order of Atmosphere::build. The reference ships no golden vectors
(tests/smoke.rs only checks for validation-layer errors), so these fixtures are
the pin for the CPU oracle and, through it, for the CUDA library.

Fixtures (float32, npz):
  smoke_f32.npz  tests/smoke.rs:132-143 sizes (r8, mu32, mu_s8, nu2, order 4),
                 RGBA32F storage: final tables plus per-order tables
  smoke_f16.npz  the same with the reference's RGBA16F scattering-class
                 storage (src/precompute.rs:1215): final irradiance/scattering
  tiny_f32.npz   a small non-default atmosphere (other geometry and table
                 sizes, order 3): every table

Run: python tests/golden/make_golden.py   (needs the reference checkout)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fuzzyblue_gb300.params import Parameters, DensityProfile, DensityProfileLayer, smoke_parameters  # noqa
from oracle import py_oracle  # noqa


def tiny_parameters():
    return Parameters(
        order=3,
        transmittance_mu_size=32, transmittance_r_size=12,
        scattering_r_size=6, scattering_mu_size=16, scattering_mu_s_size=6, scattering_nu_size=3,
        irradiance_mu_s_size=16, irradiance_r_size=6,
        bottom_radius=3390.0, top_radius=3470.0,
        rayleigh_scattering=(0.0191, 0.0134, 0.0057),
        rayleigh_density=DensityProfile([DensityProfileLayer(), DensityProfileLayer(exp_term=1.0, exp_scale=-1 / 11.1)]),
        mie_scattering=(0.0085, 0.0085, 0.0085), mie_extinction=(0.0097, 0.0097, 0.0097),
        mie_density=DensityProfile([DensityProfileLayer(), DensityProfileLayer(exp_term=1.0, exp_scale=-1 / 2.5)]),
        mie_phase_function_g=0.7, ground_albedo=(0.3, 0.2, 0.1), mu_s_min=-0.35,
    )


FIXTURES = {
    "smoke_f32": (lambda: smoke_parameters(), True),
    "smoke_f16": (lambda: smoke_parameters(storage=1), False),
    "tiny_f32": (tiny_parameters, True),
}


def params_record(p: Parameters):
    return np.frombuffer(bytes(p.to_c()), dtype=np.uint8)


def main():
    if py_oracle.ref_lib() is None:
        raise SystemExit("the reference's shader build is unavailable (no reference checkout)")
    for name, (mk, full) in FIXTURES.items():
        p = mk()
        out = py_oracle.precompute(p, intermediates=full, reference=True)
        keep = dict(out) if full else {k: out[k] for k in ("irradiance", "scattering")}
        keep["params"] = params_record(p)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **keep)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
