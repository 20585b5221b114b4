//! The precompute half of the `fuzzyblue` crate (`Builder`, `Parameters`,
//! `Atmosphere::build`, `PendingAtmosphere`) on the CUDA library of this
//! repository. Names and fields follow `src/precompute.rs` of the crate; the
//! Vulkan-only fields of `Parameters` (usage, stage and access masks, layout)
//! have no counterpart, and a CUDA stream takes the place of the command
//! buffer. Failures are returned as `Error` where the crate panics.

use std::ffi::CStr;
use std::fmt;
use std::marker::PhantomData;
use std::ops::Deref;
use std::os::raw::c_void;
use std::ptr;
use std::sync::Arc;

use fuzzyblue_cuda_sys as sys;

/// A failed call: the library's status code and message.
#[derive(Clone, Debug)]
pub struct Error {
    pub status: i32,
    pub message: String,
}

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "fuzzyblue-cuda error {}: {}", self.status, self.message)
    }
}

impl std::error::Error for Error {}

fn check(status: i32) -> Result<i32, Error> {
    if status >= 0 {
        return Ok(status);
    }
    let message = unsafe { CStr::from_ptr(sys::fb_last_error()) }.to_string_lossy().into_owned();
    Err(Error { status, message })
}

/// A CUDA stream handle (`cudaStream_t`); null is the builder's own stream.
#[derive(Clone, Copy, Debug)]
pub struct Stream(pub *mut c_void);

impl Stream {
    pub fn builder_default() -> Self {
        Stream(ptr::null_mut())
    }
}

#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct DensityProfileLayer {
    pub width: f32,
    pub exp_term: f32,
    pub exp_scale: f32,
    pub linear_term: f32,
    pub constant_term: f32,
}

#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct DensityProfile {
    pub layers: [DensityProfileLayer; 2],
}

impl DensityProfile {
    fn raw(&self) -> sys::fb_density_profile {
        let mut o = sys::fb_density_profile::default();
        for (d, s) in o.layers.iter_mut().zip(self.layers.iter()) {
            d.width = s.width;
            d.exp_term = s.exp_term;
            d.exp_scale = s.exp_scale;
            d.linear_term = s.linear_term;
            d.constant_term = s.constant_term;
        }
        o
    }
    fn from_raw(r: &sys::fb_density_profile) -> Self {
        let mut o = DensityProfile::default();
        for (d, s) in o.layers.iter_mut().zip(r.layers.iter()) {
            *d = DensityProfileLayer {
                width: s.width,
                exp_term: s.exp_term,
                exp_scale: s.exp_scale,
                linear_term: s.linear_term,
                constant_term: s.constant_term,
            };
        }
        o
    }
}

/// Arithmetic of a build: `Plain` is FP32 as the crate's shaders compute;
/// `Mixed` keeps FP64 where the horizon and the order sums need it.
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Precision {
    Plain,
    Mixed,
}

/// Parameters governing generated skies, distances in km (the crate's
/// `Parameters`, with the sample counts of its shaders as fields).
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct Parameters {
    pub order: u32,
    pub transmittance_mu_size: u32,
    pub transmittance_r_size: u32,
    pub scattering_r_size: u32,
    pub scattering_mu_size: u32,
    pub scattering_mu_s_size: u32,
    pub scattering_nu_size: u32,
    pub irradiance_mu_s_size: u32,
    pub irradiance_r_size: u32,
    pub solar_irradiance: [f32; 3],
    pub sun_angular_radius: f32,
    pub bottom_radius: f32,
    pub top_radius: f32,
    pub rayleigh_density: DensityProfile,
    pub rayleigh_scattering: [f32; 3],
    pub mie_density: DensityProfile,
    pub mie_scattering: [f32; 3],
    pub mie_extinction: [f32; 3],
    pub mie_phase_function_g: f32,
    pub absorbtion_density: DensityProfile,
    pub absorbtion_extinction: [f32; 3],
    pub ground_albedo: [f32; 3],
    pub mu_s_min: f32,
    pub transmittance_steps: u32,
    pub single_scattering_steps: u32,
    pub multiple_scattering_steps: u32,
    pub density_samples: u32,
    pub irradiance_samples: u32,
    pub precision: Precision,
    /// Round the scattering-class tables to half precision as they are stored
    /// (the crate's RGBA16F images).
    pub store_f16: bool,
}

impl Default for Parameters {
    fn default() -> Self {
        let mut raw = sys::fb_params::default();
        unsafe { sys::fb_params_default(&mut raw) };
        Parameters::from_raw(&raw)
    }
}

impl Parameters {
    fn from_raw(p: &sys::fb_params) -> Self {
        let r = &p.raw;
        Parameters {
            order: p.order,
            transmittance_mu_size: r.transmittance_mu_size,
            transmittance_r_size: r.transmittance_r_size,
            scattering_r_size: r.scattering_r_size,
            scattering_mu_size: r.scattering_mu_size,
            scattering_mu_s_size: r.scattering_mu_s_size,
            scattering_nu_size: r.scattering_nu_size,
            irradiance_mu_s_size: r.irradiance_mu_s_size,
            irradiance_r_size: r.irradiance_r_size,
            solar_irradiance: r.solar_irradiance,
            sun_angular_radius: r.sun_angular_radius,
            bottom_radius: r.bottom_radius,
            top_radius: r.top_radius,
            rayleigh_density: DensityProfile::from_raw(&r.rayleigh_density),
            rayleigh_scattering: r.rayleigh_scattering,
            mie_density: DensityProfile::from_raw(&r.mie_density),
            mie_scattering: r.mie_scattering,
            mie_extinction: r.mie_extinction,
            mie_phase_function_g: r.mie_phase_function_g,
            absorbtion_density: DensityProfile::from_raw(&r.absorption_density),
            absorbtion_extinction: r.absorption_extinction,
            ground_albedo: r.ground_albedo,
            mu_s_min: r.mu_s_min,
            transmittance_steps: p.transmittance_steps,
            single_scattering_steps: p.single_scattering_steps,
            multiple_scattering_steps: p.multiple_scattering_steps,
            density_samples: p.density_samples,
            irradiance_samples: p.irradiance_samples,
            precision: if p.precision == sys::FB_PRECISION_MIXED { Precision::Mixed } else { Precision::Plain },
            store_f16: p.storage == sys::FB_STORAGE_F16,
        }
    }

    /// The C record: the crate's 320-byte `ParamsRaw` plus the extension block.
    pub fn to_raw(&self) -> sys::fb_params {
        let mut p = sys::fb_params::default();
        unsafe { sys::fb_params_default(&mut p) };
        let r = &mut p.raw;
        r.solar_irradiance = self.solar_irradiance;
        r.sun_angular_radius = self.sun_angular_radius;
        r.rayleigh_scattering = self.rayleigh_scattering;
        r.bottom_radius = self.bottom_radius;
        r.mie_scattering = self.mie_scattering;
        r.top_radius = self.top_radius;
        r.mie_extinction = self.mie_extinction;
        r.mie_phase_function_g = self.mie_phase_function_g;
        r.ground_albedo = self.ground_albedo;
        r.mu_s_min = self.mu_s_min;
        r.absorption_extinction = self.absorbtion_extinction;
        r.transmittance_mu_size = self.transmittance_mu_size;
        r.transmittance_r_size = self.transmittance_r_size;
        r.scattering_r_size = self.scattering_r_size;
        r.scattering_mu_size = self.scattering_mu_size;
        r.scattering_mu_s_size = self.scattering_mu_s_size;
        r.scattering_nu_size = self.scattering_nu_size;
        r.irradiance_mu_s_size = self.irradiance_mu_s_size;
        r.irradiance_r_size = self.irradiance_r_size;
        r.rayleigh_density = self.rayleigh_density.raw();
        r.mie_density = self.mie_density.raw();
        r.absorption_density = self.absorbtion_density.raw();
        p.order = self.order;
        p.transmittance_steps = self.transmittance_steps;
        p.single_scattering_steps = self.single_scattering_steps;
        p.multiple_scattering_steps = self.multiple_scattering_steps;
        p.density_samples = self.density_samples;
        p.irradiance_samples = self.irradiance_samples;
        p.precision = match self.precision {
            Precision::Plain => sys::FB_PRECISION_PLAIN,
            Precision::Mixed => sys::FB_PRECISION_MIXED,
        };
        p.storage = if self.store_f16 { sys::FB_STORAGE_F16 } else { sys::FB_STORAGE_F32 };
        p
    }

    pub fn validate(&self) -> Result<(), Error> {
        let p = self.to_raw();
        check(unsafe { sys::fb_params_validate(&p) }).map(|_| ())
    }

    fn extents(&self) -> (sys::fb_extent, sys::fb_extent, sys::fb_extent) {
        let p = self.to_raw();
        let (mut t, mut i, mut s) = Default::default();
        unsafe { sys::fb_params_extents(&p, &mut t, &mut i, &mut s) };
        (t, i, s)
    }
    /// (width, height) of the transmittance table.
    pub fn transmittance_extent(&self) -> (u32, u32) {
        let e = self.extents().0;
        (e.width, e.height)
    }
    /// (width, height) of the irradiance table.
    pub fn irradiance_extent(&self) -> (u32, u32) {
        let e = self.extents().1;
        (e.width, e.height)
    }
    /// (width, height, depth) of the packed scattering table.
    pub fn scattering_extent(&self) -> (u32, u32, u32) {
        let e = self.extents().2;
        (e.width, e.height, e.depth)
    }
}

/// The crate's `DrawParameters` (src/render.rs:247-252).
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct DrawParameters {
    /// (projection * view)^-1
    pub inverse_viewproj: [[f32; 4]; 4],
    pub camera_position: [f32; 3],
    pub sun_direction: [f32; 3],
}

/// A CUDA device with the precompute kernels loaded (the crate's `Builder`).
pub struct Builder {
    raw: *mut sys::fb_builder,
}

unsafe impl Send for Builder {}
unsafe impl Sync for Builder {}

impl Builder {
    pub fn new(device: i32) -> Result<Self, Error> {
        let mut raw = ptr::null_mut();
        check(unsafe { sys::fb_builder_create(device, &mut raw) })?;
        Ok(Builder { raw })
    }

    /// Picks tile shapes for the table classes of `classes` by timing them.
    pub fn autotune(&self, classes: &[Parameters]) -> Result<(), Error> {
        let raw: Vec<sys::fb_params> = classes.iter().map(Parameters::to_raw).collect();
        check(unsafe { sys::fb_builder_autotune(self.raw, raw.as_ptr(), raw.len() as u32, 0) }).map(|_| ())
    }
}

impl Drop for Builder {
    fn drop(&mut self) {
        unsafe { sys::fb_builder_destroy(self.raw) }
    }
}

/// Device tables of one atmosphere (the crate's `Atmosphere`): float4
/// texels, x fastest, as the crate's images are laid out.
pub struct Atmosphere {
    raw: *mut sys::fb_atmosphere,
    owned: bool,
    _builder: Arc<Builder>,
}

unsafe impl Send for Atmosphere {}

impl Atmosphere {
    /// Enqueues the precompute on `stream` and returns at once (the crate's
    /// `Atmosphere::build`, which records into a command buffer).
    pub fn build(builder: Arc<Builder>, stream: Stream, params: &Parameters) -> Result<PendingAtmosphere, Error> {
        let p = params.to_raw();
        let mut raw = ptr::null_mut();
        check(unsafe { sys::fb_atmosphere_build(builder.raw, stream.0, &p, &mut raw) })?;
        Ok(PendingAtmosphere { raw, builder })
    }

    /// Many atmospheres of any table sizes and orders in one batch build.
    pub fn build_batch(builder: Arc<Builder>, stream: Stream, params: &[Parameters])
                       -> Result<PendingAtmosphere, Error> {
        let p: Vec<sys::fb_params> = params.iter().map(Parameters::to_raw).collect();
        let mut raw = ptr::null_mut();
        check(unsafe { sys::fb_batch_build(builder.raw, stream.0, p.as_ptr(), p.len() as u32, &mut raw) })?;
        Ok(PendingAtmosphere { raw, builder })
    }

    fn tables(&self) -> sys::fb_tables {
        let mut t = sys::fb_tables {
            transmittance: ptr::null_mut(),
            irradiance: ptr::null_mut(),
            scattering: ptr::null_mut(),
            transmittance_extent: Default::default(),
            irradiance_extent: Default::default(),
            scattering_extent: Default::default(),
        };
        unsafe { sys::fb_atmosphere_tables(self.raw, &mut t) };
        t
    }
    /// Device pointer of the transmittance table.
    pub fn transmittance(&self) -> *mut c_void {
        self.tables().transmittance
    }
    pub fn transmittance_extent(&self) -> (u32, u32) {
        let e = self.tables().transmittance_extent;
        (e.width, e.height)
    }
    /// Device pointer of the packed scattering table.
    pub fn scattering(&self) -> *mut c_void {
        self.tables().scattering
    }
    pub fn scattering_extent(&self) -> (u32, u32, u32) {
        let e = self.tables().scattering_extent;
        (e.width, e.height, e.depth)
    }
    /// Device pointer of the irradiance table.
    pub fn irradiance(&self) -> *mut c_void {
        self.tables().irradiance
    }
    pub fn irradiance_extent(&self) -> (u32, u32) {
        let e = self.tables().irradiance_extent;
        (e.width, e.height)
    }

    /// Copies the three tables into host memory (RGBA f32 each).
    pub fn to_host(&self) -> Result<(Vec<f32>, Vec<f32>, Vec<f32>), Error> {
        let (tw, th) = self.transmittance_extent();
        let (iw, ih) = self.irradiance_extent();
        let (sw, sh, sd) = self.scattering_extent();
        let mut t = vec![0f32; 4 * (tw * th) as usize];
        let mut i = vec![0f32; 4 * (iw * ih) as usize];
        let mut s = vec![0f32; 4 * (sw * sh * sd) as usize];
        check(unsafe {
            sys::fb_atmosphere_copy_to_host(self.raw, ptr::null_mut(), t.as_mut_ptr(), i.as_mut_ptr(), s.as_mut_ptr())
        })?;
        Ok((t, i, s))
    }

    /// Enqueues the copies of the three tables into caller-owned host buffers
    /// on `stream` without waiting; the buffers hold the tables once the
    /// stream has passed this point (page-locked buffers for the copies to be
    /// asynchronous). Any pointer may be null.
    pub unsafe fn copy_to_host_async(&self, stream: Stream, transmittance: *mut f32, irradiance: *mut f32,
                                     scattering: *mut f32) -> Result<(), Error> {
        check(sys::fb_atmosphere_copy_to_host_async(self.raw, stream.0, transmittance, irradiance, scattering))
    }

    /// The crate's sky pass (render_sky.frag) for a width x height image into
    /// device buffers of RGBA f32 (`transmittance` may be null); `depth` is a
    /// device buffer of width * height floats or null (nothing in front of the sky).
    pub unsafe fn render_sky(&self, stream: Stream, draw: &DrawParameters, depth: *const f32, width: u32,
                             height: u32, color: *mut f32, transmittance: *mut f32) -> Result<(), Error> {
        let d = sys::fb_draw_parameters {
            inverse_viewproj: draw.inverse_viewproj,
            camera_position: draw.camera_position,
            _pad0: 0.0,
            sun_direction: draw.sun_direction,
            _pad1: 0.0,
        };
        check(sys::fb_atmosphere_render_sky(self.raw, stream.0, &d, depth, width, height, color, transmittance))
            .map(|_| ())
    }

    /// The scattering table as RGBA16F bits (the crate's image format).
    pub fn scattering_f16(&self) -> Result<Vec<u16>, Error> {
        let (sw, sh, sd) = self.scattering_extent();
        let mut out = vec![0u16; 4 * (sw * sh * sd) as usize];
        check(unsafe { sys::fb_atmosphere_export_scattering_f16(self.raw, ptr::null_mut(), out.as_mut_ptr()) })?;
        Ok(out)
    }
}

impl Drop for Atmosphere {
    fn drop(&mut self) {
        if self.owned {
            unsafe { sys::fb_atmosphere_destroy(self.raw) }
        }
    }
}

/// An enqueued build (the crate's `PendingAtmosphere`): its temporaries live
/// until it is dropped.
pub struct PendingAtmosphere {
    raw: *mut sys::fb_pending,
    builder: Arc<Builder>,
}

unsafe impl Send for PendingAtmosphere {}

impl PendingAtmosphere {
    /// True once the build has completed on the device.
    pub fn is_ready(&self) -> Result<bool, Error> {
        Ok(check(unsafe { sys::fb_pending_query(self.raw) })? == sys::FB_OK)
    }
    /// Blocks until the build has completed.
    pub fn wait(&self) -> Result<(), Error> {
        check(unsafe { sys::fb_pending_wait(self.raw) }).map(|_| ())
    }
    /// Makes `consumer` wait for the build on the device (the crate's
    /// `acquire_ownership`, a queue-family transfer there).
    pub fn acquire_ownership(&self, consumer: Stream) -> Result<(), Error> {
        check(unsafe { sys::fb_pending_acquire(self.raw, consumer.0) }).map(|_| ())
    }
    /// Number of atmospheres of the build (1, or the batch size).
    pub fn len(&self) -> usize {
        let mut n = 0u32;
        unsafe { sys::fb_pending_count(self.raw, &mut n) };
        n as usize
    }
    pub fn is_empty(&self) -> bool {
        self.len() == 0
    }
    /// Atmosphere `index`, borrowed from the pending build (the crate's
    /// `atmosphere`): it cannot outlive the build.
    pub fn atmosphere(&self, index: usize) -> Result<BorrowedAtmosphere<'_>, Error> {
        let mut a = ptr::null_mut();
        check(unsafe { sys::fb_pending_atmosphere(self.raw, index as u32, &mut a) })?;
        Ok(BorrowedAtmosphere {
            inner: Atmosphere { raw: a, owned: false, _builder: self.builder.clone() },
            _pending: PhantomData,
        })
    }
    /// Waits for the build and takes atmosphere `index` out of it (the
    /// crate's `assert_ready`).
    pub fn take(&self, index: usize) -> Result<Atmosphere, Error> {
        let mut a = ptr::null_mut();
        check(unsafe { sys::fb_pending_take(self.raw, index as u32, &mut a) })?;
        Ok(Atmosphere { raw: a, owned: true, _builder: self.builder.clone() })
    }
}

/// An atmosphere that still belongs to its pending build.
pub struct BorrowedAtmosphere<'a> {
    inner: Atmosphere,
    _pending: PhantomData<&'a PendingAtmosphere>,
}

impl<'a> Deref for BorrowedAtmosphere<'a> {
    type Target = Atmosphere;
    fn deref(&self) -> &Atmosphere {
        &self.inner
    }
}

impl Drop for PendingAtmosphere {
    fn drop(&mut self) {
        unsafe { sys::fb_pending_release(self.raw) }
    }
}
