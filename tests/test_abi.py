"""The C ABI: the library loads without a GPU, exports every symbol the
header declares, and its parameter handling matches the reference's layout and
defaults. No call here touches a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from fuzzyblue_gb300.params import Parameters, c_params, c_params_raw, smoke_parameters

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "fuzzyblue.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fb_[a-z0-9_]+)\s*\(", text)) - {"fb_alloc_fn", "fb_free_fn"})


def test_library_exports_every_declared_symbol(native_lib):
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(native_lib, s)]
    assert not missing, missing


def test_python_bindings_cover_header(native_lib):
    from fuzzyblue_gb300 import _native
    assert set(declared_symbols()) <= set(_native.SIGNATURES), set(declared_symbols()) - set(_native.SIGNATURES)


def test_params_raw_is_the_std140_block():
    # ParamsRaw, src/precompute.rs:937-964: 320 bytes, profiles at 128/192/256
    assert ctypes.sizeof(c_params_raw) == 320
    assert c_params_raw.transmittance_mu_size.offset == 92
    assert c_params_raw.rayleigh_density.offset == 128
    assert c_params_raw.mie_density.offset == 192
    assert c_params_raw.absorption_density.offset == 256
    assert ctypes.sizeof(c_params) == 384


def test_default_params_match_library(native_lib):
    c = c_params()
    native_lib.fb_params_default(ctypes.byref(c))
    assert bytes(c) == bytes(Parameters().to_c())


def test_extents_and_bytes(native_lib):
    from fuzzyblue_gb300 import _native as N
    p = Parameters()
    c = p.to_c()
    e = [N.c_extent() for _ in range(3)]
    assert native_lib.fb_params_extents(ctypes.byref(c), *[ctypes.byref(x) for x in e]) == 0
    assert (e[0].width, e[0].height) == p.transmittance_extent() == (256, 64)
    assert (e[1].width, e[1].height) == p.irradiance_extent() == (64, 16)
    assert (e[2].width, e[2].height, e[2].depth) == p.scattering_extent() == (256, 128, 32)
    o, t = ctypes.c_uint64(), ctypes.c_uint64()
    assert native_lib.fb_params_device_bytes(ctypes.byref(c), ctypes.byref(o), ctypes.byref(t)) == 0
    assert o.value >= 16 * (256 * 64 + 64 * 16 + 256 * 128 * 32)
    assert t.value >= 16 * 4 * 256 * 128 * 32


@pytest.mark.parametrize("bad", [
    dict(scattering_mu_size=31),            # odd mu size (the ground/sky split needs halves)
    dict(scattering_nu_size=1),             # nu decode divides by nu_size - 1
    dict(transmittance_mu_size=1),
    dict(top_radius=6000.0),                # top below bottom
    dict(order=0),
    dict(density_samples=15),
    dict(density_samples=34),
    dict(irradiance_samples=66),
    dict(single_scattering_steps=0),
    dict(multiple_scattering_steps=2000),
    dict(scattering_nu_size=64, scattering_mu_s_size=64),  # packed width > 2048
    dict(precision=7),
    dict(storage=3),
])
def test_validate_rejects_malformed(native_lib, bad):
    from fuzzyblue_gb300 import _native as N
    c = Parameters(**bad).to_c()
    assert native_lib.fb_params_validate(ctypes.byref(c)) == N.FB_ERR_INVALID_PARAMS
    assert native_lib.fb_last_error()


def test_validate_accepts_benchmark_classes(native_lib):
    for p in (Parameters(), smoke_parameters(),
              Parameters(transmittance_mu_size=512, transmittance_r_size=128, irradiance_mu_s_size=128,
                         irradiance_r_size=32, scattering_r_size=64, scattering_mu_size=256,
                         scattering_mu_s_size=64, scattering_nu_size=16, order=8, transmittance_steps=2000),
              Parameters(transmittance_mu_size=128, transmittance_r_size=32, scattering_r_size=16,
                         scattering_mu_size=64, scattering_mu_s_size=16, scattering_nu_size=4)):
        c = p.to_c()
        assert native_lib.fb_params_validate(ctypes.byref(c)) == 0, native_lib.fb_last_error()


def test_status_strings(native_lib):
    assert native_lib.fb_status_string(0) == b"ok"
    assert native_lib.fb_abi_version() == 1


def test_server_config_defaults(native_lib):
    from fuzzyblue_gb300 import _native as N
    c = N.c_server_config()
    native_lib.fb_server_config_default(ctypes.byref(c))
    assert c.hbm_budget_bytes == 120 << 30
    assert c.max_batch >= 1 and c.max_inflight >= 1 and c.cache_entries >= 1


def _rust_sys():
    return open(os.path.join(ROOT, "rust", "fuzzyblue-cuda-sys", "src", "lib.rs")).read()


def test_rust_sys_crate_declares_every_header_function():
    """The Rust binding (built only where cargo exists) declares every entry
    point of include/fuzzyblue.h."""
    import re
    header = open(os.path.join(ROOT, "include", "fuzzyblue.h")).read()
    declared = set(re.findall(r"^\s*(?:int|void|const char\*)\s+(fb_[a-z0-9_]+)\(", header, re.M))
    rust = set(re.findall(r"pub fn (fb_[a-z0-9_]+)\(", _rust_sys()))
    assert declared and declared == rust, (declared - rust, rust - declared)


def test_rust_sys_params_layout_matches_header():
    """Field order of fb_params_raw / fb_params in the Rust structs is the
    header's (both are #[repr(C)] / C structs of the same types)."""
    import re
    header = open(os.path.join(ROOT, "include", "fuzzyblue.h")).read()
    rust = _rust_sys()
    for name in ("fb_params_raw", "fb_params"):
        hb = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), header, re.S).group(1)
        hf = re.findall(r"\b(?:float|uint32_t|fb_density_profile|fb_params_raw)\s+(\w+)", hb)
        rb = re.search(r"pub struct %s \{(.*?)\n\}" % name, rust, re.S).group(1)
        rf = re.findall(r"pub (\w+):", rb)
        assert hf == rf, (name, hf, rf)


def test_intermediates_struct_matches_bindings():
    """fb_intermediates: the Python ctypes struct and the Rust struct list the
    header's fields in its order."""
    import re
    from fuzzyblue_gb300 import _native as N
    header = open(os.path.join(ROOT, "include", "fuzzyblue.h")).read()
    hb = re.search(r"typedef struct fb_intermediates \{(.*?)\} fb_intermediates;", header, re.S).group(1)
    hb = re.sub(r"/\*.*?\*/", "", hb, flags=re.S)
    hf = re.findall(r"\b(?:void\*|uint32_t)\s+(\w+)", hb)
    assert hf == [f[0] for f in N.c_intermediates._fields_]
    rb = re.search(r"pub struct fb_intermediates \{(.*?)\n\}", _rust_sys(), re.S).group(1)
    assert hf == re.findall(r"pub (\w+):", rb)


def test_planar_density_to_rgba():
    """The planar density temporary (R, G, B planes of `stride` floats per
    (r, mu) row) reads back as the RGBA layout of the other tables."""
    from fuzzyblue_gb300.api import planes_to_rgba
    depth, height, width, stride = 2, 3, 5, 8
    rng = np.random.default_rng(0)
    rgba = rng.random((depth, height, width, 4), dtype=np.float32)
    rgba[..., 3] = 0.0
    planes = np.full((depth, height, 3, stride), np.nan, np.float32)  # padding never read
    planes[..., :width] = np.moveaxis(rgba[..., :3], 3, 2)
    assert np.array_equal(planes_to_rgba(planes, width), rgba)
