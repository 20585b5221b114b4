"""Headless sky pass and surface lighting (fb_atmosphere_render_sky,
fb_atmosphere_sun_and_sky_irradiance) against the oracle's restatement of
render_sky.frag / render_sky.h / render_lighting.h, itself pinned bit for bit
to the reference's shading code, on the same tables.

Tolerance (relative error with the floor 1e-6 * max|ref|, tests/errors.py):
2e-3 for radiance toward the sky (depth 0) and for lighting; for aerial
perspective (finite depth), where the sky pass subtracts two nearly equal
lookups (render_sky.h:176-179), 2e-3 with the floor raised to 1e-4 * max|ref|.
NaN appears exactly where the reference gives NaN."""
import numpy as np
import pytest

from fuzzyblue_gb300.params import PRECISION_MIXED, smoke_parameters
from tests.errors import rel_err, summary

pytestmark = pytest.mark.gpu


def _tables(builder, p):
    from fuzzyblue_gb300.api import Atmosphere
    pend = Atmosphere.build(builder, p)
    pend.wait()
    atm = pend.take(0)
    pend.release()
    return atm, atm.to_host()


def _camera(seed, height_km=6361.0):
    from fuzzyblue_gb300.render import DrawParameters
    rng = np.random.default_rng(seed)
    fwd = rng.normal(size=3)
    fwd[1] = abs(fwd[1]) * 0.4
    return DrawParameters.look_at((0.0, height_km, 0.0), forward=fwd, up=(0, 1, 0), fov_y_deg=80, aspect=1.5,
                                  sun_direction=rng.normal(size=3))


def _compare(gpu, ref, floor):
    gpu, ref = np.asarray(gpu, np.float64), np.asarray(ref, np.float64)
    assert np.array_equal(np.isnan(gpu), np.isnan(ref))
    ok = np.isfinite(ref)
    g, r = np.where(ok, gpu, 0.0), np.where(ok, ref, 0.0)
    m = np.abs(r).max()
    return (np.abs(g - r) / np.maximum(np.abs(r), floor * m)).max()


@pytest.mark.parametrize("precision", [0, PRECISION_MIXED])
@pytest.mark.parametrize("seed", [0, 1])
def test_sky_pass_matches_oracle(builder, oracle, seed, precision):
    import torch
    from fuzzyblue_gb300.render import render_sky
    p = smoke_parameters(precision=precision)
    atm, t = _tables(builder, p)
    d = _camera(seed, 6361.0 + 20.0 * seed)
    w, h = 96, 64
    color, trans = render_sky(atm, d, w, h)
    torch.cuda.synchronize()
    c_ref, t_ref = oracle.render_sky(p, t["transmittance"], t["scattering"], d, w, h)
    assert _compare(color.cpu().numpy(), c_ref, 1e-6) <= 2e-3
    assert _compare(trans.cpu().numpy(), t_ref, 1e-6) <= 2e-3
    # aerial perspective: points at finite depth in part of the image
    rng = np.random.default_rng(seed + 10)
    depth = np.where(rng.random((h, w)) < 0.4, rng.uniform(2e-5, 5e-3, (h, w)), 0.0).astype(np.float32)
    color, trans = render_sky(atm, d, w, h, depth=torch.as_tensor(depth, device="cuda"))
    torch.cuda.synchronize()
    c_ref, t_ref = oracle.render_sky(p, t["transmittance"], t["scattering"], d, w, h, depth=depth)
    assert _compare(color.cpu().numpy(), c_ref, 1e-4) <= 2e-3
    assert _compare(trans.cpu().numpy(), t_ref, 1e-6) <= 2e-3
    atm.close()


def test_space_view_of_the_atmosphere(builder, oracle):
    """A camera outside the atmosphere: rays that miss give 0 radiance and
    transmittance 1; rays that enter are moved to the top boundary."""
    import torch
    from fuzzyblue_gb300.render import DrawParameters, render_sky
    p = smoke_parameters()
    atm, t = _tables(builder, p)
    d = DrawParameters.look_at((0.0, 0.0, 3.0 * p.top_radius), forward=(0, 0, -1), up=(0, 1, 0), fov_y_deg=50,
                               aspect=1.0, sun_direction=(0.3, 0.4, 0.8))
    color, trans = render_sky(atm, d, 64, 64)
    torch.cuda.synchronize()
    c_ref, t_ref = oracle.render_sky(p, t["transmittance"], t["scattering"], d, 64, 64)
    c = color.cpu().numpy()
    miss = np.all(t_ref[..., :3] == 1.0, axis=-1) & np.all(c_ref[..., :3] == 0.0, axis=-1)
    assert miss.any() and (~miss).any()
    assert np.all(c[miss][..., :3] == 0.0) and np.all(trans.cpu().numpy()[miss][..., :3] == 1.0)
    assert _compare(c, c_ref, 1e-6) <= 2e-3
    atm.close()


def test_sun_and_sky_irradiance_matches_oracle(builder, oracle):
    import torch
    from fuzzyblue_gb300.render import sun_and_sky_irradiance
    p = smoke_parameters()
    atm, t = _tables(builder, p)
    rng = np.random.default_rng(4)
    n = 4000
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    pts = (dirs * rng.uniform(p.bottom_radius, p.top_radius, (n, 1))).astype(np.float32)
    nrm = rng.normal(size=(n, 3))
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(np.float32)
    sun = np.array([0.3, 0.8, 0.2])
    sun = sun / np.linalg.norm(sun)
    s_gpu, k_gpu = sun_and_sky_irradiance(atm, torch.as_tensor(pts, device="cuda"),
                                          torch.as_tensor(nrm, device="cuda"), sun)
    torch.cuda.synchronize()
    s_ref, k_ref = oracle.sun_and_sky_irradiance(p, t["transmittance"], t["irradiance"], pts, nrm, sun)
    assert summary(s_gpu.cpu().numpy(), s_ref)["max"] <= 2e-3
    assert summary(k_gpu.cpu().numpy(), k_ref)["max"] <= 2e-3
    atm.close()
