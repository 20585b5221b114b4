"""Algorithmic FLOPs per texel of every pass of the reference's precompute.

Test and measurement infrastructure: counts the shader arithmetic of the
reference's algorithm (the oracle's restatement of shaders/*.comp, run with an
op-counting scalar, fbo_count_ops) per output texel, averaged over sampled
texels of the first atmospheres of a workload. Adds, subtracts, multiplies,
divides, square roots and transcendentals count one FLOP each; sampler
filtering (fixed-function in the reference) and operations on literals only
(including loop-counter expressions that a shader compiler folds once it
unrolls a fixed-trip-count loop) are not counted, so the figures are a lower
bound of the reference's arithmetic.

    python oracle/count_flops.py [--atmospheres 16] [--samples 256]

prints one JSON object: FLOPs per texel per pass (density and indirect
irradiance at the order their lookups read: order 2 density reads the single
scattering tables, higher orders one table), and FLOPs per atmosphere of the
default 4-order build.
"""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from fuzzyblue_gb300 import workloads  # noqa: E402
from oracle import py_oracle as O  # noqa: E402


def per_texel(p, samples, seed):
    out = {}
    out["transmittance"] = O.count_ops(p, "transmittance", 1, samples, seed)["flops"]
    out["direct_irradiance"] = O.count_ops(p, "direct_irradiance", 1, samples, seed)["flops"]
    out["single_scattering"] = O.count_ops(p, "single_scattering", 1, samples, seed)["flops"]
    out["density_order2"] = O.count_ops(p, "scattering_density", 2, samples, seed)["flops"]
    out["density_order3"] = O.count_ops(p, "scattering_density", 3, samples, seed)["flops"]
    out["indirect_order1"] = O.count_ops(p, "indirect_irradiance", 1, samples, seed)["flops"]
    out["indirect_order2"] = O.count_ops(p, "indirect_irradiance", 2, samples, seed)["flops"]
    out["multiple_scattering"] = O.count_ops(p, "multiple_scattering", 3, samples, seed)["flops"]
    return out


def per_atmosphere(p, f):
    ntr, nir, nsc = p.texel_counts()
    total = ntr * f["transmittance"] + nir * f["direct_irradiance"] + nsc * f["single_scattering"]
    for order in range(2, p.order + 1):
        total += nsc * (f["density_order2"] if order == 2 else f["density_order3"])
        total += nir * (f["indirect_order1"] if order == 2 else f["indirect_order2"])
        total += nsc * f["multiple_scattering"]
    return total


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--atmospheres", type=int, default=16)
    ap.add_argument("--samples", type=int, default=256)
    a = ap.parse_args()
    ps = workloads.uniform_batch(a.atmospheres, seed=0, order=4)
    acc = {}
    for i, p in enumerate(ps):
        f = per_texel(p, a.samples, seed=i + 1)
        for k, v in f.items():
            acc[k] = acc.get(k, 0.0) + v / len(ps)
    out = {"workload": "uniform batch, seed 0, first %d atmospheres, default sizes" % len(ps),
           "samples_per_pass": a.samples,
           "flop_per_texel": {k: round(v, 1) for k, v in acc.items()},
           "density_flop_per_direction_order3": round(acc["density_order3"] / (2 * ps[0].density_samples ** 2), 2),
           "flop_per_atmosphere_4_orders": per_atmosphere(ps[0], acc)}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
