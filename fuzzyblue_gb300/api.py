"""Python mirror of the crate's public API (src/lib.rs:9: Atmosphere, Builder,
Parameters, PendingAtmosphere), over the C ABI of include/fuzzyblue.h.

    builder = Builder(device=0)                      # Builder::new
    pending = Atmosphere.build(builder, Parameters()) # Atmosphere::build
    pending.wait(); pending.assert_ready()            # device_wait_idle + assert_ready
    atm = pending.atmosphere()                       # PendingAtmosphere::atmosphere
    atm.transmittance(), atm.scattering_extent() ...  # accessors, src/precompute.rs:2075-2101

Streams: any argument named `stream` accepts None (the builder's stream), a
torch.cuda.Stream, or a raw cudaStream_t as an int.
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _native as N
from .params import Parameters, c_params


def _stream_handle(stream) -> Optional[int]:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    h = getattr(stream, "cuda_stream", None)
    if h is not None:
        return int(h)
    raise TypeError("unsupported stream object %r" % (stream,))


class DeviceArray:
    """A view of device memory exposing __cuda_array_interface__ (float32),
    so torch.as_tensor(view, device='cuda') wraps it without a copy."""

    def __init__(self, ptr: int, shape, owner=None, typestr="<f4"):
        self.ptr = int(ptr)
        self.shape = tuple(int(s) for s in shape)
        self._owner = owner
        self.__cuda_array_interface__ = {"shape": self.shape, "typestr": typestr, "data": (self.ptr, False),
                                         "version": 3, "strides": None}

    def to_numpy(self) -> np.ndarray:
        import torch
        t = torch.as_tensor(self, device="cuda")
        return t.cpu().numpy()


def planes_to_rgba(planes: np.ndarray, width: int) -> np.ndarray:
    """(depth, height, 3, stride) float planes -> (depth, height, width, 4) RGBA
    with alpha 0 (the layout scattering_density.comp:155 writes)."""
    p = planes[..., :width]
    out = np.zeros(p.shape[:2] + (width, 4), np.float32)
    out[..., :3] = np.moveaxis(p, 2, 3)
    return out


class PlanarDensity(DeviceArray):
    """The scattering-density temporary, stored as three float planes (R, G, B)
    per (r, mu) row of `stride` floats; to_numpy() gives the RGBA layout of the
    other scattering-class tables."""

    def __init__(self, ptr: int, extent, stride: int, owner=None):
        sd, sh, sw = extent
        super().__init__(ptr, (sd, sh, 3, int(stride)), owner)
        self.width = int(sw)

    def to_numpy(self) -> np.ndarray:
        return planes_to_rgba(super().to_numpy(), self.width)


class Builder:
    """Builder::new (src/precompute.rs:61-68): one CUDA device and its kernels."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        N.check(N.lib().fb_builder_create(device, ctypes.byref(self._h)), "fb_builder_create")
        self._alloc_refs = None

    @property
    def handle(self):
        return self._h

    @property
    def sm_count(self) -> int:
        v = ctypes.c_int()
        N.check(N.lib().fb_builder_sm_count(self._h, ctypes.byref(v)), "fb_builder_sm_count")
        return v.value

    def set_profiling(self, enabled: bool = True):
        N.check(N.lib().fb_builder_set_profiling(self._h, 1 if enabled else 0), "fb_builder_set_profiling")

    def autotune(self, classes: Sequence[Parameters], batch: int = 8):
        """Times every candidate tile shape and kernel variant of each class
        (scattering sizes + precision) and keeps the fastest for later builds."""
        arr = (c_params * len(classes))(*[p.to_c() for p in classes])
        N.check(N.lib().fb_builder_autotune(self._h, arr, len(classes), batch), "fb_builder_autotune")

    def tuned_shape(self, params: Parameters) -> Optional[dict]:
        s = N.c_tile_shape()
        c = params.to_c()
        rc = N.lib().fb_builder_tuned_shape(self._h, ctypes.byref(c), ctypes.byref(s))
        if rc == N.FB_ERR_NOT_FOUND:
            return None
        N.check(rc, "fb_builder_tuned_shape")
        return {name: getattr(s, name) for name, _ in N.c_tile_shape._fields_}

    def save_tuning(self, path: str):
        N.check(N.lib().fb_builder_save_tuning(self._h, path.encode()), "fb_builder_save_tuning")

    def load_tuning(self, path: str):
        N.check(N.lib().fb_builder_load_tuning(self._h, path.encode()), "fb_builder_load_tuning")

    def set_allocator(self, alloc, release):
        """Routes the builder's device allocations through Python callables
        alloc(nbytes, stream) -> int pointer (0 = failure) and release(ptr, stream)."""
        if alloc is None:
            N.check(N.lib().fb_builder_set_allocator(self._h, N.ALLOC_FN(), N.FREE_FN(), None), "set_allocator")
            self._alloc_refs = None
            return
        a = N.ALLOC_FN(lambda user, n, s: alloc(n, s) or None)
        f = N.FREE_FN(lambda user, p, s: release(p, s))
        N.check(N.lib().fb_builder_set_allocator(self._h, a, f, None), "set_allocator")
        self._alloc_refs = (a, f)

    def close(self):
        if self._h:
            N.lib().fb_builder_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Atmosphere:
    """An atmosphere whose tables are ready (src/precompute.rs:1042-1101)."""

    def __init__(self, handle, params: Parameters, owned: bool, keepalive=None):
        self._h = handle
        self.params = params
        self._owned = owned
        self._keep = keepalive

    # -- Atmosphere::build ---------------------------------------------------
    @staticmethod
    def build(builder: Builder, params: Parameters, stream=None) -> "PendingAtmosphere":
        c = params.to_c()
        out = ctypes.c_void_p()
        N.check(N.lib().fb_atmosphere_build(builder.handle, _stream_handle(stream), ctypes.byref(c),
                                            ctypes.byref(out)), "fb_atmosphere_build")
        return PendingAtmosphere(out, [params], builder)

    # -- accessors (src/precompute.rs:2075-2101) ------------------------------
    def _tables(self) -> N.c_tables:
        t = N.c_tables()
        N.check(N.lib().fb_atmosphere_tables(self._h, ctypes.byref(t)), "fb_atmosphere_tables")
        return t

    def transmittance(self) -> int:
        return self._tables().transmittance

    def irradiance(self) -> int:
        return self._tables().irradiance

    def scattering(self) -> int:
        return self._tables().scattering

    def transmittance_extent(self):
        return self.params.transmittance_extent()

    def irradiance_extent(self):
        return self.params.irradiance_extent()

    def scattering_extent(self):
        return self.params.scattering_extent()

    def device_views(self) -> Dict[str, DeviceArray]:
        t = self._tables()
        tw, th = self.params.transmittance_extent()
        iw, ih = self.params.irradiance_extent()
        sw, sh, sd = self.params.scattering_extent()
        return {
            "transmittance": DeviceArray(t.transmittance, (th, tw, 4), self),
            "irradiance": DeviceArray(t.irradiance, (ih, iw, 4), self),
            "scattering": DeviceArray(t.scattering, (sd, sh, sw, 4), self),
        }

    def to_host(self, stream=None) -> Dict[str, np.ndarray]:
        """Copies the three tables to host memory: RGBA float32 arrays shaped
        (height, width, 4) and (depth, height, width, 4)."""
        tw, th = self.params.transmittance_extent()
        iw, ih = self.params.irradiance_extent()
        sw, sh, sd = self.params.scattering_extent()
        out = {
            "transmittance": np.empty((th, tw, 4), np.float32),
            "irradiance": np.empty((ih, iw, 4), np.float32),
            "scattering": np.empty((sd, sh, sw, 4), np.float32),
        }
        N.check(N.lib().fb_atmosphere_copy_to_host(self._h, _stream_handle(stream),
                                                   out["transmittance"].ctypes.data, out["irradiance"].ctypes.data,
                                                   out["scattering"].ctypes.data), "fb_atmosphere_copy_to_host")
        return out

    def copy_to_host_async(self, transmittance, irradiance, scattering, stream=None):
        """Enqueues the copies of the three tables into host buffers (any of
        them None to skip) on `stream` and returns at once; the buffers hold
        the tables once the stream has passed this point. Numpy arrays must be
        contiguous float32 of the table sizes; page-locked memory (e.g. a
        pinned torch tensor's numpy view) keeps the copies asynchronous."""
        def ptr(x):
            if x is None:
                return None
            assert x.dtype == np.float32 and x.flags["C_CONTIGUOUS"]
            return x.ctypes.data
        tw, th = self.params.transmittance_extent()
        iw, ih = self.params.irradiance_extent()
        sw, sh, sd = self.params.scattering_extent()
        for x, n in ((transmittance, tw * th), (irradiance, iw * ih), (scattering, sw * sh * sd)):
            assert x is None or x.size >= 4 * n, "host buffer too small"
        N.check(N.lib().fb_atmosphere_copy_to_host_async(self._h, _stream_handle(stream), ptr(transmittance),
                                                         ptr(irradiance), ptr(scattering)),
                "fb_atmosphere_copy_to_host_async")

    def render_sky(self, draw, width: int, height: int, depth=None, stream=None):
        """The crate's sky pass for a width x height image (fuzzyblue_gb300.render)."""
        from .render import render_sky
        return render_sky(self, draw, width, height, depth=depth, stream=stream)

    def sun_and_sky_irradiance(self, points, normals, sun_direction, stream=None):
        """GetSunAndSkyIrradiance at points (fuzzyblue_gb300.render)."""
        from .render import sun_and_sky_irradiance
        return sun_and_sky_irradiance(self, points, normals, sun_direction, stream=stream)

    def export_scattering_f16(self, stream=None) -> np.ndarray:
        """The scattering table as RGBA16F (np.float16), the reference's image format."""
        sw, sh, sd = self.params.scattering_extent()
        out = np.empty((sd, sh, sw, 4), np.float16)
        N.check(N.lib().fb_atmosphere_export_scattering_f16(self._h, _stream_handle(stream), out.ctypes.data),
                "fb_atmosphere_export_scattering_f16")
        return out

    def close(self):
        if self._owned and self._h:
            N.lib().fb_atmosphere_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PendingAtmosphere:
    """An atmosphere (or batch) being prepared by the GPU (src/precompute.rs:2103-2212)."""

    def __init__(self, handle, params: Sequence[Parameters], builder: Builder):
        self._h = handle
        self.params = list(params)
        self._builder = builder  # keeps the builder alive
        self._taken = set()

    def __len__(self):
        n = ctypes.c_uint32()
        N.check(N.lib().fb_pending_count(self._h, ctypes.byref(n)), "fb_pending_count")
        return n.value

    def query(self) -> bool:
        return N.check(N.lib().fb_pending_query(self._h), "fb_pending_query") == N.FB_OK

    def wait(self):
        N.check(N.lib().fb_pending_wait(self._h), "fb_pending_wait")

    def assert_ready(self):
        """PendingAtmosphere::assert_ready (src/precompute.rs:2209): the work
        must have completed."""
        if not self.query():
            raise RuntimeError("atmosphere build has not completed")

    def acquire(self, stream):
        """Makes `stream` wait for the build (acquire_ownership, src/precompute.rs:2147)."""
        N.check(N.lib().fb_pending_acquire(self._h, _stream_handle(stream)), "fb_pending_acquire")

    def atmosphere(self, index: int = 0) -> Atmosphere:
        h = ctypes.c_void_p()
        N.check(N.lib().fb_pending_atmosphere(self._h, index, ctypes.byref(h)), "fb_pending_atmosphere")
        return Atmosphere(h, self.params[index], owned=False, keepalive=self)

    def take(self, index: int = 0) -> Atmosphere:
        h = ctypes.c_void_p()
        N.check(N.lib().fb_pending_take(self._h, index, ctypes.byref(h)), "fb_pending_take")
        return Atmosphere(h, self.params[index], owned=True)

    def intermediates(self, index: int = 0) -> Dict[str, DeviceArray]:
        m = N.c_intermediates()
        N.check(N.lib().fb_pending_intermediates(self._h, index, ctypes.byref(m)), "fb_pending_intermediates")
        p = self.params[index]
        iw, ih = p.irradiance_extent()
        sw, sh, sd = p.scattering_extent()
        sc = (sd, sh, sw, 4)
        return {
            "delta_irradiance_0": DeviceArray(m.delta_irradiance[0], (ih, iw, 4), self),
            "delta_irradiance_1": DeviceArray(m.delta_irradiance[1], (ih, iw, 4), self),
            "delta_rayleigh": DeviceArray(m.delta_rayleigh, sc, self),
            "delta_mie": DeviceArray(m.delta_mie, sc, self),
            "delta_multiple_scattering": DeviceArray(m.delta_multiple_scattering, sc, self),
            "scattering_density": PlanarDensity(m.scattering_density, (sd, sh, sw), m.scattering_density_stride, self),
        }

    def profile(self) -> List[dict]:
        """Per-launch device times of the build (profiling must have been on)."""
        n = ctypes.c_uint32()
        N.check(N.lib().fb_pending_profile(self._h, None, 0, ctypes.byref(n)), "fb_pending_profile")
        arr = (N.c_launch_profile * max(n.value, 1))()
        N.check(N.lib().fb_pending_profile(self._h, arr, n.value, ctypes.byref(n)), "fb_pending_profile")
        return [{"kernel": N.KERNEL_NAMES[r.kernel], "order": r.order, "precision": r.precision, "grid": r.grid,
                 "items": r.items, "texels": r.texels, "ms": r.ms} for r in arr[:n.value]]

    def release(self):
        if self._h:
            N.lib().fb_pending_release(self._h)
            self._h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def build_batch(builder: Builder, params: Sequence[Parameters], stream=None) -> PendingAtmosphere:
    """Builds many atmospheres (any mix of table sizes, orders and precision
    modes) with one persistent launch per pass group, replayed from a CUDA graph."""
    arr = (c_params * len(params))(*[p.to_c() for p in params])
    out = ctypes.c_void_p()
    N.check(N.lib().fb_batch_build(builder.handle, _stream_handle(stream), arr, len(params), ctypes.byref(out)),
            "fb_batch_build")
    return PendingAtmosphere(out, params, builder)


def validate(params: Parameters) -> None:
    c = params.to_c()
    N.check(N.lib().fb_params_validate(ctypes.byref(c)), "fb_params_validate")


def device_bytes(params: Parameters):
    c = params.to_c()
    o = ctypes.c_uint64()
    t = ctypes.c_uint64()
    N.check(N.lib().fb_params_device_bytes(ctypes.byref(c), ctypes.byref(o), ctypes.byref(t)), "device_bytes")
    return o.value, t.value


class Server:
    """Request loop with HBM-budget admission, concurrent batches and a
    device-resident LRU cache of finished tables (fb_server_* in the C ABI)."""

    def __init__(self, builder: Builder, hbm_budget_bytes: Optional[int] = None, max_batch: Optional[int] = None,
                 max_inflight: Optional[int] = None, cache_entries: Optional[int] = None,
                 max_queue: Optional[int] = None):
        cfg = N.c_server_config()
        N.lib().fb_server_config_default(ctypes.byref(cfg))
        for name, v in (("hbm_budget_bytes", hbm_budget_bytes), ("max_batch", max_batch),
                        ("max_inflight", max_inflight), ("cache_entries", cache_entries), ("max_queue", max_queue)):
            if v is not None:
                setattr(cfg, name, v)
        self.config = cfg
        self._h = ctypes.c_void_p()
        N.check(N.lib().fb_server_create(builder.handle, ctypes.byref(cfg), ctypes.byref(self._h)), "fb_server_create")
        self._builder = builder
        self._params: Dict[int, Parameters] = {}

    def submit(self, params: Parameters) -> int:
        t = ctypes.c_uint64()
        c = params.to_c()
        N.check(N.lib().fb_server_submit(self._h, ctypes.byref(c), ctypes.byref(t)), "fb_server_submit")
        self._params[t.value] = params
        return t.value

    def _atm(self, ticket, h):
        return Atmosphere(h, self._params[ticket], owned=False, keepalive=self)

    def poll(self, ticket: int) -> Optional[Atmosphere]:
        h = ctypes.c_void_p()
        rc = N.check(N.lib().fb_server_poll(self._h, ticket, ctypes.byref(h)), "fb_server_poll")
        return None if rc == N.FB_NOT_READY else self._atm(ticket, h)

    def wait(self, ticket: int, timeout_ms: int = 0xFFFFFFFF) -> Optional[Atmosphere]:
        h = ctypes.c_void_p()
        rc = N.check(N.lib().fb_server_wait(self._h, ticket, timeout_ms, ctypes.byref(h)), "fb_server_wait")
        return None if rc == N.FB_NOT_READY else self._atm(ticket, h)

    def release(self, ticket: int):
        N.check(N.lib().fb_server_release(self._h, ticket), "fb_server_release")
        self._params.pop(ticket, None)

    def completed(self, timeout_ms: int = 0, capacity: int = 4096) -> List[int]:
        """Tickets that finished (ready or failed) since earlier calls, oldest
        first (fb_server_completed); waits up to timeout_ms for the first."""
        buf = (ctypes.c_uint64 * capacity)()
        n = ctypes.c_uint32()
        N.check(N.lib().fb_server_completed(self._h, buf, capacity, timeout_ms, ctypes.byref(n)),
                "fb_server_completed")
        return list(buf[:n.value])

    def cancel(self, ticket: int) -> bool:
        """True if the request was cancelled before it started."""
        return N.check(N.lib().fb_server_cancel(self._h, ticket), "fb_server_cancel") == N.FB_OK

    def stats(self) -> dict:
        s = N.c_server_stats()
        N.check(N.lib().fb_server_get_stats(self._h, ctypes.byref(s)), "fb_server_get_stats")
        return {name: getattr(s, name) for name, _ in N.c_server_stats._fields_}

    def close(self):
        if self._h:
            N.lib().fb_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
