"""Headless use of the precomputed tables: the crate's sky pass and surface
lighting (src/render.rs, shaders/render_sky.frag, render_sky.h,
render_lighting.h) evaluated by CUDA kernels into device memory.

`DrawParameters` mirrors the crate's push constants (src/render.rs:247-252):
(projection * view)^-1, the camera position in km and the sun direction.
`DrawParameters.look_at` builds them for a perspective camera with an
infinitely far, reversed depth range (depth 0 is at infinity, the value the
sky pass reads where nothing is in front of the sky); world positions of the
matrix are in metres, as the sky pass expects (it scales them by 1e-3).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _native as N


@dataclass
class DrawParameters:
    inverse_viewproj: np.ndarray          # 4x4, [column][row] (GLSL mat4 columns)
    camera_position: Tuple[float, float, float]  # km, planet frame
    sun_direction: Tuple[float, float, float]    # unit vector

    def to_c(self) -> N.c_draw_parameters:
        c = N.c_draw_parameters()
        m = np.asarray(self.inverse_viewproj, np.float32)
        for col in range(4):
            for row in range(4):
                c.inverse_viewproj[col][row] = float(m[col, row])
        for i in range(3):
            c.camera_position[i] = float(self.camera_position[i])
            c.sun_direction[i] = float(self.sun_direction[i])
        return c

    @staticmethod
    def look_at(camera_km: Sequence[float], forward: Sequence[float], up: Sequence[float], fov_y_deg: float,
                aspect: float, sun_direction: Sequence[float], near_m: float = 0.1) -> "DrawParameters":
        """A camera at `camera_km` looking along `forward`: view matrix in
        metres, reversed-depth infinite perspective (NDC depth near_m / distance),
        Vulkan clip space (y down)."""
        f = np.asarray(forward, np.float64)
        f = f / np.linalg.norm(f)
        s = np.cross(f, np.asarray(up, np.float64))
        s = s / np.linalg.norm(s)
        u = np.cross(s, f)
        eye = np.asarray(camera_km, np.float64) * 1e3
        view = np.eye(4)
        view[0, :3], view[1, :3], view[2, :3] = s, u, -f
        view[:3, 3] = -view[:3, :3] @ eye
        t = 1.0 / math.tan(math.radians(fov_y_deg) / 2.0)
        proj = np.zeros((4, 4))
        proj[0, 0] = t / aspect
        proj[1, 1] = -t
        proj[2, 3] = near_m
        proj[3, 2] = -1.0
        inv = np.linalg.inv(proj @ view)  # row-major: inv[row, col]
        sun = np.asarray(sun_direction, np.float64)
        sun = sun / np.linalg.norm(sun)
        return DrawParameters(inverse_viewproj=inv.T.astype(np.float32), camera_position=tuple(camera_km),
                              sun_direction=tuple(float(x) for x in sun))


def render_sky(atmosphere, draw: DrawParameters, width: int, height: int, depth=None, stream=None):
    """The sky pass for a width x height image: returns (radiance, transmittance)
    as torch tensors of shape (height, width, 4) on the atmosphere's device.
    `depth`: an optional (height, width) float32 CUDA tensor."""
    import torch
    from .api import _stream_handle
    color = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
    trans = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
    dptr = None
    if depth is not None:
        assert depth.is_cuda and depth.dtype == torch.float32 and tuple(depth.shape) == (height, width)
        dptr = depth.contiguous().data_ptr()
    c = draw.to_c()
    s = _stream_handle(stream) if stream is not None else torch.cuda.current_stream().cuda_stream
    N.check(N.lib().fb_atmosphere_render_sky(atmosphere._h, s, ctypes.byref(c), dptr, width, height,
                                             color.data_ptr(), trans.data_ptr()), "fb_atmosphere_render_sky")
    return color, trans


def sun_and_sky_irradiance(atmosphere, points, normals, sun_direction, stream=None):
    """GetSunAndSkyIrradiance at points (n, 3) with normals (n, 3), km, as
    CUDA tensors: returns (sun irradiance, sky irradiance), each (n, 3)."""
    import torch
    from .api import _stream_handle
    points = points.contiguous().float()
    normals = normals.contiguous().float()
    n = int(points.shape[0])
    sun_out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    sky_out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    sd = (ctypes.c_float * 3)(*[float(x) for x in sun_direction])
    s = _stream_handle(stream) if stream is not None else torch.cuda.current_stream().cuda_stream
    N.check(N.lib().fb_atmosphere_sun_and_sky_irradiance(atmosphere._h, s, points.data_ptr(), normals.data_ptr(),
                                                         sd, n, sun_out.data_ptr(), sky_out.data_ptr()),
            "fb_atmosphere_sun_and_sky_irradiance")
    return sun_out, sky_out
