//! Raw declarations of include/fuzzyblue.h (the C ABI of the CUDA
//! atmosphere precompute). Struct layouts match the header field for field;
//! `fb_params_raw` is byte-for-byte the 320-byte std140 `ParamsRaw` block.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const FB_OK: c_int = 0;
pub const FB_NOT_READY: c_int = 1;
pub const FB_ERR_INVALID_ARGUMENT: c_int = -1;
pub const FB_ERR_INVALID_PARAMS: c_int = -2;
pub const FB_ERR_OUT_OF_MEMORY: c_int = -3;
pub const FB_ERR_CUDA: c_int = -4;
pub const FB_ERR_BUDGET: c_int = -5;
pub const FB_ERR_CANCELLED: c_int = -6;
pub const FB_ERR_NOT_FOUND: c_int = -7;
pub const FB_ERR_SHUTDOWN: c_int = -8;
pub const FB_ERR_NO_KERNEL: c_int = -9;

pub const FB_PRECISION_PLAIN: u32 = 0;
pub const FB_PRECISION_MIXED: u32 = 1;
pub const FB_STORAGE_F32: u32 = 0;
pub const FB_STORAGE_F16: u32 = 1;

#[repr(C)]
pub struct fb_builder {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct fb_pending {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct fb_atmosphere {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct fb_server {
    _opaque: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct fb_density_profile_layer {
    pub width: f32,
    pub exp_term: f32,
    pub exp_scale: f32,
    pub linear_term: f32,
    pub constant_term: f32,
    pub _pad: [f32; 3],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct fb_density_profile {
    pub layers: [fb_density_profile_layer; 2],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct fb_params_raw {
    pub solar_irradiance: [f32; 3],
    pub sun_angular_radius: f32,
    pub rayleigh_scattering: [f32; 3],
    pub bottom_radius: f32,
    pub mie_scattering: [f32; 3],
    pub top_radius: f32,
    pub mie_extinction: [f32; 3],
    pub mie_phase_function_g: f32,
    pub ground_albedo: [f32; 3],
    pub mu_s_min: f32,
    pub absorption_extinction: [f32; 3],
    pub transmittance_mu_size: u32,
    pub transmittance_r_size: u32,
    pub scattering_r_size: u32,
    pub scattering_mu_size: u32,
    pub scattering_mu_s_size: u32,
    pub scattering_nu_size: u32,
    pub irradiance_mu_s_size: u32,
    pub irradiance_r_size: u32,
    pub _pad0: u32,
    pub rayleigh_density: fb_density_profile,
    pub mie_density: fb_density_profile,
    pub absorption_density: fb_density_profile,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct fb_params {
    pub raw: fb_params_raw,
    pub order: u32,
    pub transmittance_steps: u32,
    pub single_scattering_steps: u32,
    pub multiple_scattering_steps: u32,
    pub density_samples: u32,
    pub irradiance_samples: u32,
    pub precision: u32,
    pub storage: u32,
    pub reserved: [u32; 8],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq, Eq)]
pub struct fb_extent {
    pub width: u32,
    pub height: u32,
    pub depth: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct fb_tables {
    pub transmittance: *mut c_void,
    pub irradiance: *mut c_void,
    pub scattering: *mut c_void,
    pub transmittance_extent: fb_extent,
    pub irradiance_extent: fb_extent,
    pub scattering_extent: fb_extent,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct fb_intermediates {
    pub delta_irradiance: [*mut c_void; 2],
    pub delta_rayleigh: *mut c_void,
    pub delta_mie: *mut c_void,
    pub delta_multiple_scattering: *mut c_void,
    pub scattering_density: *mut c_void,
    pub scattering_density_stride: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct fb_tile_shape {
    pub density_columns: u32,
    pub density_rows: u32,
    pub density_variant: u32,
    pub multiple_variant: u32,
    pub density_ms: f32,
    pub multiple_ms: f32,
}

pub const FB_KERNEL_TRANSMITTANCE: u32 = 0;
pub const FB_KERNEL_SINGLE: u32 = 1;
pub const FB_KERNEL_DENSITY: u32 = 2;
pub const FB_KERNEL_MULTIPLE: u32 = 3;

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct fb_launch_profile {
    pub kernel: u32,
    pub order: u32,
    pub precision: u32,
    pub grid: u32,
    pub items: u64,
    pub texels: u64,
    pub ms: f32,
    pub _pad: f32,
}

/// Device allocation hook of `fb_builder_set_allocator` (NULL on failure).
pub type fb_alloc_fn = Option<unsafe extern "C" fn(user: *mut c_void, bytes: usize, stream: *mut c_void) -> *mut c_void>;
pub type fb_free_fn = Option<unsafe extern "C" fn(user: *mut c_void, ptr: *mut c_void, stream: *mut c_void)>;

/// Push constants of the crate's sky pass: inverse_viewproj[column][row].
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct fb_draw_parameters {
    pub inverse_viewproj: [[f32; 4]; 4],
    pub camera_position: [f32; 3],
    pub _pad0: f32,
    pub sun_direction: [f32; 3],
    pub _pad1: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct fb_server_config {
    pub hbm_budget_bytes: u64,
    pub max_batch: u32,
    pub max_inflight: u32,
    pub cache_entries: u32,
    pub max_queue: u32,
    pub reserved: [u32; 6],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct fb_server_stats {
    pub submitted: u64,
    pub completed: u64,
    pub rejected: u64,
    pub cancelled: u64,
    pub cache_hits: u64,
    pub evictions: u64,
    pub batches: u64,
    pub resident_bytes: u64,
    pub inflight_bytes: u64,
    pub queued: u64,
    pub p50_ms: f64,
    pub p99_ms: f64,
    pub mean_ms: f64,
    pub mean_batch: f64,
}

#[link(name = "fuzzyblue_cuda")]
extern "C" {
    pub fn fb_params_default(out: *mut fb_params);
    pub fn fb_params_validate(p: *const fb_params) -> c_int;
    pub fn fb_params_extents(p: *const fb_params, tr: *mut fb_extent, ir: *mut fb_extent,
                             sc: *mut fb_extent) -> c_int;
    pub fn fb_params_device_bytes(p: *const fb_params, output_bytes: *mut u64,
                                  temporary_bytes: *mut u64) -> c_int;

    pub fn fb_builder_create(device: c_int, out: *mut *mut fb_builder) -> c_int;
    pub fn fb_builder_destroy(b: *mut fb_builder);
    pub fn fb_builder_device(b: *const fb_builder, device: *mut c_int) -> c_int;
    pub fn fb_builder_sm_count(b: *const fb_builder, sms: *mut c_int) -> c_int;
    pub fn fb_builder_set_allocator(b: *mut fb_builder, alloc: fb_alloc_fn, release: fb_free_fn,
                                    user: *mut c_void) -> c_int;
    pub fn fb_builder_set_profiling(b: *mut fb_builder, enabled: c_int) -> c_int;
    pub fn fb_builder_tuned_shape(b: *const fb_builder, cls: *const fb_params, out: *mut fb_tile_shape) -> c_int;
    pub fn fb_builder_autotune(b: *mut fb_builder, classes: *const fb_params, count: u32, batch: u32) -> c_int;
    pub fn fb_builder_save_tuning(b: *mut fb_builder, path: *const c_char) -> c_int;
    pub fn fb_builder_load_tuning(b: *mut fb_builder, path: *const c_char) -> c_int;

    pub fn fb_atmosphere_build(b: *mut fb_builder, stream: *mut c_void, p: *const fb_params,
                               out: *mut *mut fb_pending) -> c_int;
    pub fn fb_batch_build(b: *mut fb_builder, stream: *mut c_void, p: *const fb_params, count: u32,
                          out: *mut *mut fb_pending) -> c_int;
    pub fn fb_pending_query(p: *mut fb_pending) -> c_int;
    pub fn fb_pending_wait(p: *mut fb_pending) -> c_int;
    pub fn fb_pending_acquire(p: *mut fb_pending, consumer_stream: *mut c_void) -> c_int;
    pub fn fb_pending_count(p: *const fb_pending, count: *mut u32) -> c_int;
    pub fn fb_pending_atmosphere(p: *mut fb_pending, index: u32, out: *mut *mut fb_atmosphere) -> c_int;
    pub fn fb_pending_take(p: *mut fb_pending, index: u32, out: *mut *mut fb_atmosphere) -> c_int;
    pub fn fb_pending_intermediates(p: *mut fb_pending, index: u32, out: *mut fb_intermediates) -> c_int;
    pub fn fb_pending_profile(p: *mut fb_pending, out: *mut fb_launch_profile, capacity: u32,
                              count: *mut u32) -> c_int;
    pub fn fb_pending_release(p: *mut fb_pending);

    pub fn fb_atmosphere_tables(a: *const fb_atmosphere, out: *mut fb_tables) -> c_int;
    pub fn fb_atmosphere_copy_to_host(a: *const fb_atmosphere, stream: *mut c_void, tr: *mut f32,
                                      ir: *mut f32, sc: *mut f32) -> c_int;
    pub fn fb_atmosphere_copy_to_host_async(a: *const fb_atmosphere, stream: *mut c_void, tr: *mut f32,
                                            ir: *mut f32, sc: *mut f32) -> c_int;
    pub fn fb_atmosphere_export_scattering_f16(a: *const fb_atmosphere, stream: *mut c_void,
                                               out: *mut u16) -> c_int;
    pub fn fb_atmosphere_params(a: *const fb_atmosphere, out: *mut fb_params) -> c_int;
    pub fn fb_atmosphere_destroy(a: *mut fb_atmosphere);
    pub fn fb_atmosphere_build_noalloc(stream: *mut c_void, p: *const fb_params, transmittance: *mut c_void,
                                       irradiance: *mut c_void, scattering: *mut c_void) -> c_int;

    pub fn fb_atmosphere_render_sky(a: *const fb_atmosphere, stream: *mut c_void, d: *const fb_draw_parameters,
                                    depth: *const f32, width: u32, height: u32, color: *mut f32,
                                    transmittance: *mut f32) -> c_int;
    pub fn fb_atmosphere_sun_and_sky_irradiance(a: *const fb_atmosphere, stream: *mut c_void, points: *const f32,
                                                normals: *const f32, sun_direction: *const f32, n: u32,
                                                sun_irradiance: *mut f32, sky_irradiance: *mut f32) -> c_int;

    pub fn fb_server_config_default(out: *mut fb_server_config);
    pub fn fb_server_create(b: *mut fb_builder, cfg: *const fb_server_config, out: *mut *mut fb_server) -> c_int;
    pub fn fb_server_submit(s: *mut fb_server, p: *const fb_params, ticket: *mut u64) -> c_int;
    pub fn fb_server_poll(s: *mut fb_server, ticket: u64, out: *mut *mut fb_atmosphere) -> c_int;
    pub fn fb_server_wait(s: *mut fb_server, ticket: u64, timeout_ms: u32, out: *mut *mut fb_atmosphere) -> c_int;
    pub fn fb_server_release(s: *mut fb_server, ticket: u64) -> c_int;
    pub fn fb_server_completed(s: *mut fb_server, tickets: *mut u64, capacity: u32, timeout_ms: u32,
                               count: *mut u32) -> c_int;
    pub fn fb_server_cancel(s: *mut fb_server, ticket: u64) -> c_int;
    pub fn fb_server_get_stats(s: *mut fb_server, out: *mut fb_server_stats) -> c_int;
    pub fn fb_server_destroy(s: *mut fb_server);

    pub fn fb_status_string(status: c_int) -> *const c_char;
    pub fn fb_last_error() -> *const c_char;
    pub fn fb_abi_version() -> c_int;
}
