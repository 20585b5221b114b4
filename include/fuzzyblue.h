/*
 * fuzzyblue.h — C ABI of the GB300 (sm_103a) atmosphere look-up-table precompute.
 *
 * This library replaces the Vulkan precompute path of the fuzzyblue crate
 * (src/precompute.rs): the same parameters (km, 1/km), the same six passes
 * (transmittance, direct irradiance, single scattering, scattering density,
 * indirect irradiance, multiple scattering) and the same three output tables:
 *
 *   transmittance  2D  width = transmittance_mu_size, height = transmittance_r_size
 *   irradiance     2D  width = irradiance_mu_s_size,  height = irradiance_r_size
 *   scattering     3D  width = scattering_nu_size * scattering_mu_s_size,
 *                      height = scattering_mu_size, depth = scattering_r_size
 *
 * Every table is RGBA, tightly packed, x fastest then y then z: the host layout
 * that examples/dump.rs:150-194 obtains with vkCmdCopyImageToBuffer. Tables are
 * RGBA32F in device memory (the scattering table can additionally be exported
 * as RGBA16F, the format the reference allocates at src/precompute.rs:1215).
 *
 * Conventions: every entry point returns an int status (FB_OK = 0, negative on
 * error) and never throws; handles are opaque; a handle may be used from one
 * thread at a time; `stream` arguments are cudaStream_t passed as void*
 * (NULL selects the builder's own stream). Work is enqueued asynchronously on
 * the stream, the way Atmosphere::build records into a caller's command buffer.
 */
#ifndef FUZZYBLUE_H_
#define FUZZYBLUE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FB_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------- */
#define FB_OK 0
#define FB_NOT_READY 1            /* work still in flight (query/poll) */
#define FB_ERR_INVALID_ARGUMENT (-1)
#define FB_ERR_INVALID_PARAMS (-2) /* rejected by fb_params_validate */
#define FB_ERR_OUT_OF_MEMORY (-3)
#define FB_ERR_CUDA (-4)
#define FB_ERR_BUDGET (-5)         /* request larger than the serving HBM budget */
#define FB_ERR_CANCELLED (-6)
#define FB_ERR_NOT_FOUND (-7)
#define FB_ERR_SHUTDOWN (-8)
#define FB_ERR_NO_KERNEL (-9)      /* no sm_103a image for the current device */

/* ---- parameters ----------------------------------------------------------- */

/* One layer of a density profile: clamp(exp_term*exp(exp_scale*h) +
 * linear_term*h + constant_term, 0, 1). Replaces DensityProfileLayer
 * (src/precompute.rs:660-666); padded to the 32-byte std140 array stride of
 * DensityProfileLayerRaw (src/precompute.rs:1012-1021). */
typedef struct fb_density_profile_layer {
    float width;
    float exp_term;
    float exp_scale;
    float linear_term;
    float constant_term;
    float _pad[3];
} fb_density_profile_layer;

/* Two layers, bottom to top; the width of the last one is ignored.
 * Replaces DensityProfile (src/precompute.rs:674-676). */
typedef struct fb_density_profile {
    fb_density_profile_layer layers[2];
} fb_density_profile;

/* Byte-for-byte the 320-byte ParamsRaw uniform block
 * (src/precompute.rs:937-964 == shaders/params.h:26-87 in std140). */
typedef struct fb_params_raw {
    float solar_irradiance[3];
    float sun_angular_radius;
    float rayleigh_scattering[3];
    float bottom_radius;
    float mie_scattering[3];
    float top_radius;
    float mie_extinction[3];
    float mie_phase_function_g;
    float ground_albedo[3];
    float mu_s_min;
    float absorption_extinction[3];
    uint32_t transmittance_mu_size;
    uint32_t transmittance_r_size;
    uint32_t scattering_r_size;
    uint32_t scattering_mu_size;
    uint32_t scattering_mu_s_size;
    uint32_t scattering_nu_size;
    uint32_t irradiance_mu_s_size;
    uint32_t irradiance_r_size;
    uint32_t _pad0;
    fb_density_profile rayleigh_density;
    fb_density_profile mie_density;
    fb_density_profile absorption_density;
} fb_params_raw;

/* Arithmetic of the passes. PLAIN is one FP32 atmosphere exactly as the
 * reference's shaders compute it. MIXED keeps FP32 bulk work but uses
 * compensated (Kahan) quadrature sums and FP64 for the ray/sphere
 * discriminants, the texture-coordinate mappings at the horizon seam and the
 * accumulation of orders into the final tables. */
#define FB_PRECISION_PLAIN 0u
#define FB_PRECISION_MIXED 1u

/* Storage of the five scattering-class tables. F32 keeps every table RGBA32F.
 * F16 rounds every scattering-class texel to half precision when it is
 * stored, as the reference's RGBA16F images do (src/precompute.rs:1215). */
#define FB_STORAGE_F32 0u
#define FB_STORAGE_F16 1u

/* Parameters of one atmosphere: the ParamsRaw block plus the fields the
 * reference keeps elsewhere (Parameters::order, src/precompute.rs:700) or as
 * shader constants (sample counts). Vulkan-only fields of Parameters (usage,
 * stage/access masks, layout) have no counterpart. 384 bytes. */
typedef struct fb_params {
    fb_params_raw raw;
    uint32_t order;                     /* number of bounces, >= 1 (default 4) */
    uint32_t transmittance_steps;       /* transmittance.comp:14, default 500 */
    uint32_t single_scattering_steps;   /* single_scattering.comp:42, default 50 */
    uint32_t multiple_scattering_steps; /* multiple_scattering.comp:21, default 50 */
    uint32_t density_samples;           /* scattering_density.comp:34, default 16
                                           (16 theta x 32 phi directions) */
    uint32_t irradiance_samples;        /* indirect_irradiance.comp:20, default 32
                                           (16 theta x 64 phi directions) */
    uint32_t precision;                 /* FB_PRECISION_* */
    uint32_t storage;                   /* FB_STORAGE_* */
    uint32_t reserved[8];
} fb_params;

typedef struct fb_extent {
    uint32_t width;
    uint32_t height;
    uint32_t depth;
} fb_extent;

/* Parameters::default() (src/precompute.rs:849-935) plus the default
 * extension fields. */
void fb_params_default(fb_params* out);

/* Checks sizes and geometry; FB_OK or FB_ERR_INVALID_PARAMS (the reason is in
 * fb_last_error). Rules: every table size in [2, 65536]; scattering_mu_size
 * even; scattering_nu_size <= 64; nu_size * mu_s_size <= 2048; irradiance
 * mu_s size <= 4096; 0 < bottom_radius < top_radius; order in [1, 64];
 * transmittance_steps in [1, 1e6]; single/multiple scattering steps in
 * [1, 1024]; density_samples even in [2, 32]; irradiance_samples even in
 * [2, 64]; known precision and storage modes. The reference silently leaves
 * texels unwritten for sizes that are not multiples of its workgroup size
 * (src/precompute.rs:1742,1797); every size accepted here is computed fully. */
int fb_params_validate(const fb_params* p);

/* Parameters::{transmittance,irradiance,scattering}_extent
 * (src/precompute.rs:771-793). Any pointer may be NULL. */
int fb_params_extents(const fb_params* p, fb_extent* transmittance,
                      fb_extent* irradiance, fb_extent* scattering);

/* Device bytes one build needs: the three outputs plus the temporaries. */
int fb_params_device_bytes(const fb_params* p, uint64_t* output_bytes,
                           uint64_t* temporary_bytes);

/* ---- builder ------------------------------------------------------------- */

typedef struct fb_builder fb_builder;
typedef struct fb_atmosphere fb_atmosphere;
typedef struct fb_pending fb_pending;

/* Replaces Builder::new (src/precompute.rs:61-68): binds a CUDA device, creates
 * the builder's stream and checks that the sm_103a kernels load. */
int fb_builder_create(int device, fb_builder** out);
void fb_builder_destroy(fb_builder* b);
int fb_builder_device(const fb_builder* b, int* device);
/* Number of SMs, used to size persistent launches. */
int fb_builder_sm_count(const fb_builder* b, int* sms);

/* Host-side allocation hook: when set, every device allocation the builder
 * makes goes through `alloc` (return NULL to report failure) and `release`.
 * Used to inject allocation failures in tests; NULL restores the builder's own
 * stream-ordered memory pool (cudaMallocFromPoolAsync on a pool that keeps
 * freed memory for reuse). */
typedef void* (*fb_alloc_fn)(void* user, size_t bytes, void* stream);
typedef void (*fb_free_fn)(void* user, void* ptr, void* stream);
int fb_builder_set_allocator(fb_builder* b, fb_alloc_fn alloc, fb_free_fn release,
                             void* user);

/* ---- one atmosphere ------------------------------------------------------ */

/* Replaces Atmosphere::build (src/precompute.rs:1077-2073): allocates the
 * outputs and temporaries and enqueues every pass on `stream`. Returns at once;
 * the tables are ready when the pending handle reports FB_OK. */
int fb_atmosphere_build(fb_builder* b, void* stream, const fb_params* p,
                        fb_pending** out);

/* FB_OK when all work of the build has completed, FB_NOT_READY otherwise. */
int fb_pending_query(fb_pending* p);
/* Blocks until the build completed (PendingAtmosphere::assert_ready,
 * src/precompute.rs:2209, after the caller's wait). */
int fb_pending_wait(fb_pending* p);
/* Makes `consumer_stream` wait for the build (an event wait): the stream
 * analogue of PendingAtmosphere::acquire_ownership (src/precompute.rs:2147). */
int fb_pending_acquire(fb_pending* p, void* consumer_stream);
/* Number of atmospheres the pending handle carries (1, or the batch size). */
int fb_pending_count(const fb_pending* p, uint32_t* count);
/* PendingAtmosphere::atmosphere (src/precompute.rs:2204): borrows atmosphere
 * `index`; it stays owned by the pending handle until fb_pending_take. */
int fb_pending_atmosphere(fb_pending* p, uint32_t index, fb_atmosphere** out);
/* Transfers ownership of atmosphere `index` to the caller (who then calls
 * fb_atmosphere_destroy). Waits for completion first. */
int fb_pending_take(fb_pending* p, uint32_t index, fb_atmosphere** out);
/* Device pointers of the temporaries of atmosphere `index` (the images
 * PendingAtmosphere owns, src/precompute.rs:2111-2121), valid until
 * fb_pending_release. After the build they hold the values of the last order:
 * delta_irradiance[n & 1] the irradiance read by order n's density,
 * delta_irradiance[(n+1) & 1] the indirect irradiance of order n-1. */
typedef struct fb_intermediates {
    void* delta_irradiance[2];
    void* delta_rayleigh;
    void* delta_mie;
    void* delta_multiple_scattering;
    /* float planes: for each (r, mu) row of the scattering extent, R then G
     * then B, each scattering_density_stride floats of which the first
     * width (nu_size * mu_s_size) hold values */
    void* scattering_density;
    uint32_t scattering_density_stride;
} fb_intermediates;
int fb_pending_intermediates(fb_pending* p, uint32_t index, fb_intermediates* out);
/* Drop for PendingAtmosphere (src/precompute.rs:2122-2140): frees the
 * temporaries (stream-ordered) and every atmosphere not taken. */
void fb_pending_release(fb_pending* p);

typedef struct fb_tables {
    void* transmittance; /* float4, transmittance extent */
    void* irradiance;    /* float4, irradiance extent */
    void* scattering;    /* float4, scattering extent */
    fb_extent transmittance_extent;
    fb_extent irradiance_extent;
    fb_extent scattering_extent;
} fb_tables;

/* Device pointers and extents: the accessors of src/precompute.rs:2075-2101. */
int fb_atmosphere_tables(const fb_atmosphere* a, fb_tables* out);
/* Enqueues device->host copies of the three tables (any pointer may be NULL)
 * on `stream` and waits for them. Host buffers hold width*height*depth*4
 * floats each. */
int fb_atmosphere_copy_to_host(const fb_atmosphere* a, void* stream,
                               float* transmittance, float* irradiance,
                               float* scattering);
/* The same copies, enqueued on `stream` without waiting: the host buffers
 * hold the tables once the stream has passed this point (synchronize the
 * stream, or wait on an event recorded after the call). Asynchronous with
 * respect to the host only for page-locked host buffers. Lets a caller
 * overlap the copies of one build with the kernels of the next. */
int fb_atmosphere_copy_to_host_async(const fb_atmosphere* a, void* stream,
                                     float* transmittance, float* irradiance,
                                     float* scattering);
/* RGBA16F copy of the scattering table (the reference's image format,
 * src/precompute.rs:1215; examples/dump.rs:120): `out` holds
 * width*height*depth*4 uint16 half floats, round to nearest even. */
int fb_atmosphere_export_scattering_f16(const fb_atmosphere* a, void* stream,
                                        uint16_t* out);
int fb_atmosphere_params(const fb_atmosphere* a, fb_params* out);
/* Drop for Atmosphere (src/precompute.rs:1059-1075). */
void fb_atmosphere_destroy(fb_atmosphere* a);

/* Builds one atmosphere without allocating any device memory. No counterpart
 * in the reference: it exists for callers that may not allocate, directly or
 * through a library, such as an engine that owns every device allocation in
 * its own pool, or a render loop where an allocation's implicit device
 * synchronisation would stall frames. The caller passes the three output
 * tables (device pointers, 16-byte aligned, laid out as fb_tables describes);
 * every temporary lives in a fixed 16 MiB device array that each GPU loading
 * this library holds until the process exits. Builds needing more (beyond the
 * r16 mu64 mu_s16 nu4 class) are refused with FB_ERR_BUDGET. The work is
 * enqueued on `stream` for the current device. All calls share that array
 * and it keeps the last call's contents: calls whose GPU work overlaps race on
 * it, so serialise them. The first call on a device sets the device up; make
 * it before any stream capture. Every check runs before anything is enqueued:
 * a call that returns an error has enqueued nothing and left the tables
 * untouched. */
int fb_atmosphere_build_noalloc(void* stream, const fb_params* p,
                                void* transmittance, void* irradiance,
                                void* scattering);

/* ---- batches ------------------------------------------------------------- */

/* Builds `count` atmospheres with one persistent launch per pass group,
 * whatever their table sizes, orders and precision; the order iteration is
 * replayed from a CUDA graph. Atmospheres are read with
 * fb_pending_atmosphere(p, i, ...). */
int fb_batch_build(fb_builder* b, void* stream, const fb_params* params,
                   uint32_t count, fb_pending** out);

/* ---- tile-shape autotuning ----------------------------------------------- */

/* The tuned launch shapes of one table class (scattering sizes + precision). */
typedef struct fb_tile_shape {
    uint32_t density_columns;  /* mu_s columns per scattering-density tile */
    uint32_t density_rows;     /* mu rows per scattering-density tile */
    uint32_t density_variant;  /* density kernel: 0, 1, 2 = registers for 4, 3, 5 blocks per SM;
                                  3-5: the same with exact-size interval tables */
    uint32_t multiple_variant; /* multiple-scattering kernel: 0, 1 = registers for 4, 3 blocks
                                  per SM (rows of the default layout, 32 mu_s x 8 nu, run
                                  the same variant compiled for that layout) */
    float density_ms;          /* measured time of the chosen density launch */
    float multiple_ms;         /* measured time of the chosen multiple-scattering launch */
} fb_tile_shape;

/* Times every candidate tile shape and kernel variant of each class in
 * `classes` (its scattering sizes and precision count; `batch` atmospheres per
 * measurement) on the builder's device and keeps the fastest for builds of
 * that class. */
int fb_builder_autotune(fb_builder* b, const fb_params* classes, uint32_t count,
                        uint32_t batch);
/* The shape builds of this class use; FB_ERR_NOT_FOUND if never tuned. */
int fb_builder_tuned_shape(const fb_builder* b, const fb_params* cls,
                           fb_tile_shape* out);
/* JSON cache of the tuned shapes (one object per class). */
int fb_builder_save_tuning(fb_builder* b, const char* path);
int fb_builder_load_tuning(fb_builder* b, const char* path);

/* ---- serving ------------------------------------------------------------- */

/* A request loop over one builder: precompute requests arrive at any time and
 * are admitted while the device-memory budget allows (in-flight builds plus
 * resident tables), several batches run at once on separate streams (requests
 * that arrive while others are on the GPU start without waiting for them),
 * and finished tables stay resident on the device for renderers, evicted in
 * least-recently-used order when the budget needs the room. A request for
 * parameters that are already resident (or in flight) shares that result. */
typedef struct fb_server fb_server;

typedef struct fb_server_config {
    uint64_t hbm_budget_bytes; /* device bytes for in-flight builds + resident tables (default 120 GB) */
    uint32_t max_batch;        /* atmospheres per batch launch (default 64) */
    uint32_t max_inflight;     /* batches running at once, one stream each (default 4) */
    uint32_t cache_entries;    /* finished atmospheres kept resident at most (default 4096) */
    uint32_t max_queue;        /* queued requests beyond which submit refuses (default 65536) */
    uint32_t reserved[6];
} fb_server_config;

typedef struct fb_server_stats {
    uint64_t submitted;      /* requests accepted */
    uint64_t completed;      /* requests whose tables are ready (built or shared) */
    uint64_t rejected;       /* refused: over budget alone or queue full */
    uint64_t cancelled;
    uint64_t cache_hits;     /* requests answered by resident or in-flight tables */
    uint64_t evictions;      /* resident atmospheres freed to make room */
    uint64_t batches;        /* batch launches */
    uint64_t resident_bytes; /* finished tables on the device */
    uint64_t inflight_bytes; /* outputs + temporaries of running batches */
    uint64_t queued;         /* requests waiting for admission */
    double p50_ms;           /* submit-to-ready latency of completed requests */
    double p99_ms;
    double mean_ms;
    double mean_batch;       /* atmospheres per batch launch */
} fb_server_stats;

void fb_server_config_default(fb_server_config* out);
int fb_server_create(fb_builder* b, const fb_server_config* cfg, fb_server** out);
/* Queues a request; FB_ERR_BUDGET if its tables alone exceed the budget,
 * FB_ERR_SHUTDOWN after destroy began. */
int fb_server_submit(fb_server* s, const fb_params* p, uint64_t* ticket);
/* FB_OK (and *out) when the request's tables are ready, FB_NOT_READY while it
 * is queued or running, FB_ERR_CANCELLED / FB_ERR_NOT_FOUND otherwise. The
 * atmosphere stays owned by the server and is not evicted until
 * fb_server_release(ticket). */
int fb_server_poll(fb_server* s, uint64_t ticket, fb_atmosphere** out);
/* As fb_server_poll, blocking up to timeout_ms (UINT32_MAX: no limit). */
int fb_server_wait(fb_server* s, uint64_t ticket, uint32_t timeout_ms, fb_atmosphere** out);
/* Copies into `tickets` up to `capacity` tickets of requests that finished
 * (ready or failed) since earlier calls, oldest first, and sets *count; the
 * rest stay for the next call. With none waiting it blocks up to timeout_ms
 * (0: return at once, UINT32_MAX: until one finishes or the server stops).
 * One call replaces polling every outstanding ticket; fb_server_poll then
 * gives each ticket's tables or status. */
int fb_server_completed(fb_server* s, uint64_t* tickets, uint32_t capacity, uint32_t timeout_ms,
                        uint32_t* count);
/* The caller is done with the ticket's tables; they may now be evicted. */
int fb_server_release(fb_server* s, uint64_t ticket);
/* Cancels a request that has not started; FB_NOT_READY if it is running. */
int fb_server_cancel(fb_server* s, uint64_t ticket);
int fb_server_get_stats(fb_server* s, fb_server_stats* out);
/* Waits for running batches, frees every resident table, stops the loop. */
void fb_server_destroy(fb_server* s);

/* ---- headless sky rendering ---------------------------------------------- */

/* The push constants of the crate's sky pass (DrawParameters,
 * src/render.rs:247-270): (projection * view)^-1 as the columns of a GLSL
 * mat4 (inverse_viewproj[column][row]), camera position in km and the
 * direction towards the sun (unit length), in the planet's frame. */
typedef struct fb_draw_parameters {
    float inverse_viewproj[4][4];
    float camera_position[3];
    float _pad0;
    float sun_direction[3];
    float _pad1;
} fb_draw_parameters;

/* The sky pass of the crate's renderer (render_sky.frag:24-34 over
 * render_sky.h:111-191) for every pixel of a width x height image, without
 * a graphics API: pixel (x, y) has screen coordinates ((x + 1/2) / width,
 * (y + 1/2) / height), `depth` (device, width * height floats, NULL for 0
 * everywhere: nothing in front of the sky) is the depth the sky pass reads,
 * world positions are in metres as there and scaled to km. Writes RGBA
 * float4 per pixel to `color` (radiance, A = 0) and, when not NULL, to
 * `transmittance` (A = 1), both device memory, rows of `width` pixels. The
 * tables are sampled as the crate's sampler does (LINEAR, CLAMP_TO_EDGE). */
int fb_atmosphere_render_sky(const fb_atmosphere* a, void* stream, const fb_draw_parameters* d,
                             const float* depth, uint32_t width, uint32_t height,
                             float* color, float* transmittance);

/* GetSunAndSkyIrradiance (render_lighting.h:10-28) at `n` points (km, planet
 * frame) with surface normals: sun_irradiance and sky_irradiance receive 3
 * floats per point. All arrays are device memory; sun_direction is 3 floats
 * of host memory. */
int fb_atmosphere_sun_and_sky_irradiance(const fb_atmosphere* a, void* stream, const float* points,
                                         const float* normals, const float* sun_direction, uint32_t n,
                                         float* sun_irradiance, float* sky_irradiance);

/* ---- profiling ----------------------------------------------------------- */

/* When enabled, builds record a CUDA timing event around every kernel launch
 * (batches then launch directly instead of replaying their CUDA graph: events
 * inside a graph cannot be read back); fb_pending_profile then reports the
 * device time of each launch once the build has completed. */
int fb_builder_set_profiling(fb_builder* b, int enabled);

#define FB_KERNEL_TRANSMITTANCE 0 /* transmittance.comp */
#define FB_KERNEL_SINGLE 1        /* single_scattering + direct_irradiance */
#define FB_KERNEL_DENSITY 2       /* scattering_density + indirect_irradiance */
#define FB_KERNEL_MULTIPLE 3      /* multiple_scattering */

typedef struct fb_launch_profile {
    uint32_t kernel;     /* FB_KERNEL_* */
    uint32_t order;      /* scattering order of the launch (0 for the first two) */
    uint32_t precision;  /* FB_PRECISION_* */
    uint32_t grid;       /* CTAs launched (persistent) */
    uint64_t items;      /* work items (tiles) processed */
    uint64_t texels;     /* output texels written by the launch */
    float ms;            /* device time */
    float _pad;
} fb_launch_profile;

/* Copies up to `capacity` launch records into `out` and sets *count to the
 * number of launches of the build. Waits for the build. FB_ERR_NOT_FOUND if
 * profiling was off when the build was enqueued. */
int fb_pending_profile(fb_pending* p, fb_launch_profile* out, uint32_t capacity,
                       uint32_t* count);

/* ---- diagnostics --------------------------------------------------------- */

const char* fb_status_string(int status);
/* Message of the last error on the calling thread ("" if none). */
const char* fb_last_error(void);
int fb_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FUZZYBLUE_H_ */
