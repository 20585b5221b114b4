"""Error metrics shared by the parity tests.

rel_err: |x - ref| / max(|ref|, tau * max|ref|) per channel (RGB), with the
floor tau = 1e-6 relative to the table's largest magnitude, so texels whose
reference value is ~0 are judged against a small absolute scale.
"""
import numpy as np

TAU = 1e-6


def rel_err(x, ref, tau=TAU):
    x = np.asarray(x, np.float64)[..., :3]
    ref = np.asarray(ref, np.float64)[..., :3]
    floor = tau * max(np.abs(ref).max(), 1e-300)
    return np.abs(x - ref) / np.maximum(np.abs(ref), floor)


def summary(x, ref, tau=TAU):
    e = rel_err(x, ref, tau)
    return {"max": float(e.max()), "rms": float(np.sqrt(np.mean(e * e))), "p999": float(np.quantile(e, 0.999))}
