/*
 * raydar_cuda.h -- C ABI of the GB300 (sm_103a) path-tracing backend for Raydar.
 *
 * This library replaces the hot path of Raydar's CPU renderer
 * (src/renderer/cpu.rs:193-394 with src/utils/mod.rs:6-55 and
 * src/scene/world.rs:17-31): camera ray generation, sphere/cube closest hit,
 * Diffuse/Specular/Metal/Glass scattering, the bounce loop and per-pixel
 * sample accumulation.  It sits behind Raydar's `trait Renderer`
 * (src/renderer/mod.rs:25-35); a Rust `CudaRenderer` binds these symbols.
 *
 * Conventions
 *   - Every entry point returns rdc_status (0 = RDC_OK).  No exception or
 *     panic crosses the ABI.  The message of the last failure on a context is
 *     returned by rdc_last_error(ctx); failures of rdc_create (no context yet)
 *     are reported by rdc_last_error(NULL) on the calling thread.
 *   - The caller owns every host buffer; the context owns all device memory.
 *     Host arrays passed in are copied during the call.
 *   - A context is used from one thread at a time (the reference trait takes
 *     `&mut self`).  The context serialises its work on its own CUDA stream.
 *   - Matrices are column-major 4x4 float (x column first), exactly as
 *     serialised in `.rscn` files (src/scene/camera.rs:26-29).
 *   - Randomness is a counter-based Philox4x32-10 stream keyed by
 *     (seed, pixel, sample, bounce), so a render is deterministic, progressive
 *     rendering in any split of the sample range gives bit-identical results,
 *     and the CPU oracle can replay any path.
 */
#ifndef RAYDAR_CUDA_H
#define RAYDAR_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RDC_ABI_VERSION 1

typedef enum rdc_status {
    RDC_OK = 0,
    RDC_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, malformed scene */
    RDC_ERR_UNSUPPORTED = 2,      /* e.g. World::Transparent (a todo!() panic in the reference) */
    RDC_ERR_LIMIT = 3,            /* a size above the documented maxima below */
    RDC_ERR_NO_SCENE = 4,         /* render/read before rdc_scene_upload */
    RDC_ERR_CUDA = 5,             /* a CUDA runtime call failed; see rdc_last_error */
    RDC_ERR_OUT_OF_MEMORY = 6,
    RDC_ERR_DEVICE = 7            /* a kernel reported an error flag (bounds/step cap) */
} rdc_status;

/* Geometry kinds: src/scene/objects.rs:6-10. */
enum { RDC_GEOMETRY_SPHERE = 0, RDC_GEOMETRY_CUBE = 1 };
/* World kinds: src/scene/world.rs:6-14. */
enum { RDC_WORLD_SKY_COLOR = 0, RDC_WORLD_SOLID_COLOR = 1, RDC_WORLD_TRANSPARENT = 2 };
/* Projection kinds: src/scene/camera.rs:8-11. */
enum { RDC_PROJECTION_PERSPECTIVE = 0, RDC_PROJECTION_ORTHOGRAPHIC = 1 };

/* Documented maxima (checked on upload; RDC_ERR_LIMIT above them). */
#define RDC_MAX_RESOLUTION 16384u     /* per axis */
#define RDC_MAX_OBJECTS (1u << 24)    /* objects per scene */
#define RDC_MAX_BRUTE_OBJECTS 4096u   /* brute-force render: records staged in shared memory */
#define RDC_MAX_BOUNCES 1024u

/* Closest-hit acceleration (rdc_set_accel).  Both give the reference's
 * result bit for bit; the LBVH is built on the device on upload. */
enum { RDC_ACCEL_AUTO = 0, RDC_ACCEL_BRUTE_FORCE = 1, RDC_ACCEL_LBVH = 2 };
#define RDC_ACCEL_AUTO_LBVH_ABOVE 512u /* AUTO uses the LBVH above this many objects */

/* The form rdc_render runs in (rdc_set_render_form).  Both give the same
 * accumulator bit for bit. */
enum { RDC_FORM_AUTO = 0, RDC_FORM_MEGAKERNEL = 1, RDC_FORM_WAVEFRONT = 2 };
#define RDC_FORM_AUTO_WAVE_SAMPLES 4u /* AUTO: LBVH renders whose wave holds this many samples run as wavefront */

/* Camera, field for field as src/scene/camera.rs:13-30.  The renderer uses
 * `position`, the resolution and the two inverse matrices as stored; the
 * remaining fields are carried so a caller can round-trip a Camera. */
typedef struct rdc_camera {
    float position[3];
    float target[3];
    float up[3];
    uint32_t resolution_x;
    uint32_t resolution_y;
    uint32_t projection;      /* RDC_PROJECTION_* */
    float fov_degrees;        /* Projection::Perspective { fov } */
    float ortho_size;         /* Projection::Orthographic { size } */
    float near_clip;
    float far_clip;
    float view_matrix[16];
    float proj_matrix[16];
    float inverse_view_matrix[16];
    float inverse_proj_matrix[16];
} rdc_camera;

/* World, src/scene/world.rs:6-14.  SkyColor uses top/bottom; SolidColor uses
 * solid_color; Transparent is rejected with RDC_ERR_UNSUPPORTED. */
typedef struct rdc_world {
    uint32_t kind;            /* RDC_WORLD_* */
    float top_color[3];
    float bottom_color[3];
    float solid_color[3];
} rdc_world;

/* Material, src/scene/material.rs:4-13. */
typedef struct rdc_material {
    float albedo[3];
    float roughness;
    float metallic;
    float emission_color[3];
    float emission_strength;
    float transmission;
    float ior;
} rdc_material;

/* Object, src/scene/objects.rs:12-16 with Geometry::{Sphere,Cube} (40-50). */
typedef struct rdc_object {
    uint32_t geometry;        /* RDC_GEOMETRY_* */
    float center[3];
    float radius;             /* Sphere::radius (ignored for cubes) */
    float side_length;        /* Cube::side_length (ignored for spheres) */
    rdc_material material;
} rdc_object;

/* Scene, src/scene/mod.rs:13-18.  `objects` keeps the scene's own order: the
 * closest-hit tie rule (first minimum wins, src/renderer/cpu.rs:345-349)
 * depends on it. */
typedef struct rdc_scene_desc {
    rdc_camera camera;
    rdc_world world;
    const rdc_object* objects;
    uint32_t object_count;
} rdc_scene_desc;

typedef struct rdc_stats {
    uint64_t segments;        /* trace_ray calls (src/renderer/cpu.rs:257) in the last render */
    uint64_t paths;           /* pixels x samples in the last render */
    float device_ms;          /* CUDA-event time of the last render's kernels */
    uint32_t sample_count;    /* samples accumulated since the last reset */
    uint32_t kernel_launches; /* kernels launched by the last render */
    uint64_t h2d_bytes;       /* host->device bytes the context has copied since creation */
    uint64_t d2h_bytes;       /* device->host bytes the context has copied since creation */
    uint64_t node_visits;     /* LBVH interior nodes visited by the last render (0 for brute force) */
    uint64_t prim_tests;      /* LBVH object tests of the last render (0 for brute force) */
    uint32_t accel;           /* RDC_ACCEL_BRUTE_FORCE or RDC_ACCEL_LBVH: what the current scene uses */
    uint32_t bvh_depth;       /* deepest LBVH leaf of the current scene (0 without an LBVH) */
} rdc_stats;

typedef struct rdc_ctx rdc_ctx;

/* ---- lifetime --------------------------------------------------------- */

/* Library version string. */
const char* rdc_version(void);

/* Create a context on CUDA device `device`.  Replaces constructing a renderer
 * (CpuRenderer::new, src/renderer/cpu.rs:186; src/cli/mod.rs:50-54). */
rdc_status rdc_create(rdc_ctx** out, int device);

/* Destroy a context and free its device memory.  NULL is accepted. */
void rdc_destroy(rdc_ctx* ctx);

/* Message of the last failure on `ctx` ("" if none).  With ctx == NULL:
 * the last failure of a call without a context (rdc_create, the .rscn
 * reader and writer) on the calling thread. */
const char* rdc_last_error(const rdc_ctx* ctx);

/* The CUDA stream (cudaStream_t) all of the context's work is ordered on. */
rdc_status rdc_get_stream(rdc_ctx* ctx, void** stream_out);

/* Block until all work queued on the context has finished. */
rdc_status rdc_synchronize(rdc_ctx* ctx);

/* ---- scene ------------------------------------------------------------ */

/* Read a .rscn scene -- the serde JSON the reference loads and saves
 * (src/cli/mod.rs:32-40; layout src/scene/mod.rs:13-18, camera.rs:13-30,
 * objects.rs:12-50, material.rs:4-13, world.rs:6-14) -- from `length` bytes of
 * text.  The camera matrices are taken as stored.  With objects_out NULL and
 * capacity 0 it only validates and sets *count_out; otherwise capacity must
 * be at least the object count, and scene_out->objects = objects_out.
 * Errors: RDC_ERR_INVALID_ARGUMENT (malformed; message in
 * rdc_last_error(NULL)), RDC_ERR_LIMIT (capacity too small). */
rdc_status rdc_scene_parse_rscn(const char* text, size_t length, rdc_scene_desc* scene_out,
                                rdc_object* objects_out, uint32_t capacity, uint32_t* count_out);

/* Write a scene as .rscn JSON into buf (capacity bytes, NUL-terminated);
 * *length_out = the JSON's length without the NUL (buf NULL: length only).
 * Floats are written with the fewest digits that read back to the same f32. */
rdc_status rdc_scene_write_rscn(const rdc_scene_desc* scene, char* buf, size_t capacity, size_t* length_out);

/* Copy a scene to the device: validates it, flattens the objects into
 * structure-of-arrays records and precomputes per-object constants.
 * Replaces the `&Scene` each Renderer method receives (src/renderer/mod.rs:26-28).
 * If the resolution changed, the accumulator is reallocated and zeroed, as
 * CpuRenderer::frame_buffer does (src/renderer/cpu.rs:400-417). */
rdc_status rdc_scene_upload(rdc_ctx* ctx, const rdc_scene_desc* scene);

/* Choose the closest-hit acceleration (RDC_ACCEL_*) for this and later
 * uploads; with a scene already uploaded, builds or drops its LBVH now.  The
 * reference always tests every object (src/renderer/cpu.rs:344-352). */
rdc_status rdc_set_accel(rdc_ctx* ctx, uint32_t mode);

/* Replace the materials of the uploaded scene's objects (count = its object
 * count, in scene order) without re-uploading geometry or rebuilding the
 * LBVH: the per-step update of an inverse-rendering loop, or of the editor's
 * material inspector (src/widgets/inspector.rs:433-531).  The accumulator is
 * kept; a later rdc_backward needs a new rdc_forward. */
rdc_status rdc_update_materials(rdc_ctx* ctx, const rdc_material* materials, uint32_t count);

/* ---- rendering -------------------------------------------------------- */

/* Zero the RGBA accumulator and the sample count: Renderer::new_frame
 * (src/renderer/cpu.rs:135-140, 419-423). */
rdc_status rdc_reset(rdc_ctx* ctx);

/* Trace samples [spp_begin, spp_begin + spp_count) of every pixel with at
 * most `max_bounces` segments per path and add them, in sample order, to
 * the accumulator: the body of CpuRenderer::render_next_sample
 * (src/renderer/cpu.rs:193-219) repeated spp_count times, with per_pixel
 * (233-342), trace_ray (344-352) and closest_hit (354-394).  Queued on the
 * context stream; returns once launched.  render_frame is
 * rdc_reset + rdc_render(0, max_sample_count); render_sample is
 * rdc_render(sample_count, 1). */
rdc_status rdc_render(rdc_ctx* ctx, uint32_t spp_begin, uint32_t spp_count,
                      uint32_t max_bounces, uint64_t seed);

/* Choose the form of later rdc_render calls (RDC_FORM_*): the megakernel
 * (each path in one lane's registers, each lane owning whole pixels), the
 * wavefront form of rdc_render_wavefront, or AUTO (the default): the
 * wavefront when one wave holds at least RDC_FORM_AUTO_WAVE_SAMPLES samples
 * of every pixel (spp_count >= 4 and at most 2^23 pixels) and the scene
 * uses the LBVH or the image has at most 1.5 pixels per resident megakernel
 * lane (1.5 x SMs x 768: 175,104 on 152 SMs), else the megakernel.
 * Measured, wavefront / megakernel time: 110k-object LBVH scene at 1080p 16
 * spp 0.92, 4 spp 0.93, 1 spp 1.22, at 512x512 64 spp 0.69, at 480x270 32
 * spp 0.55; 81-object brute-force scene at 1080p 64 spp 1.46, 960x540 1.06,
 * 480x270 0.63, 320x180 0.48, 128x72 at 512 spp 0.31.
 * RDC_ERR_INVALID_ARGUMENT for another value.  Affects speed and device
 * memory (the wavefront's state, up to 2.9 GB) only, never results. */
rdc_status rdc_set_render_form(rdc_ctx* ctx, uint32_t form);

/* Render without allocating any GPU memory.  For callers that cannot call
 * cudaMalloc -- an application whose device memory belongs to another
 * allocator (a game engine, a Vulkan or OpenGL interop layer), a real-time
 * loop that forbids allocation after start-up, a plugin with a fixed memory
 * budget.  It does what rdc_scene_upload + rdc_render do on a context, but
 * the caller passes `accum_device`, a device pointer to its own
 * width*height*4-float RGBA accumulator (added to in sample order, exactly as
 * rdc_render adds), and the scene is copied into a fixed-size device array
 * inside the library (RDC_STATIC_SCRATCH_BYTES, held by every GPU that loads
 * the library until exit) together with the counters the kernel works from.
 * Limits: at most RDC_STATIC_MAX_OBJECTS objects (RDC_ERR_LIMIT above).
 * Work is queued on `stream` (a cudaStream_t, NULL = legacy default stream)
 * of the calling thread's current device.  The first call on a device looks
 * up the array's device address; make it before any stream capture.  Every
 * call on a device shares the array: calls that overlap on the GPU race and
 * must be serialised by the caller.  If `segments_out` is non-NULL the call
 * waits for the render, stores its segment count and reports a device error
 * (a block that could not stage the scene into shared memory) as
 * RDC_ERR_DEVICE; with segments_out NULL it returns once the work is queued
 * and device errors are not reported, so pass it wherever they must be
 * checked.  A message for a non-OK status is written to `error_out`
 * (capacity bytes, may be NULL).
 * No counterpart in the reference: it has no allocation-free entry point. */
#define RDC_STATIC_MAX_OBJECTS 1024u
/* 256 B of counters + 160 B per object slot: up to 4 intersection records
 * of 16 B (a one-cube run takes 4), 16 B of hit data, a 64 B material and a
 * 16 B run entry. */
#define RDC_STATIC_SCRATCH_BYTES 164096u
rdc_status rdc_render_static(const rdc_scene_desc* scene, float* accum_device, uint32_t spp_begin,
                             uint32_t spp_count, uint32_t max_bounces, uint64_t seed, void* stream,
                             uint64_t* segments_out, char* error_out, size_t error_capacity);

/* Copy the float RGBA accumulator (width*height*4 floats, row-major, alpha =
 * sample count) to host memory.  `count` is the capacity of rgba_out in
 * floats.  Synchronises the context stream. */
rdc_status rdc_read_accum(rdc_ctx* ctx, float* rgba_out, size_t count);

/* Overwrite the accumulator from host memory (checkpoint resume) and set the
 * sample count. */
rdc_status rdc_write_accum(rdc_ctx* ctx, const float* rgba_in, size_t count,
                           uint32_t sample_count);

/* Tone-map the accumulator into 8-bit RGBA on the device and copy it to host
 * memory: CpuRenderer::print_frame_buffer (src/renderer/cpu.rs:221-230),
 * trunc(clamp(sum / sample_count, 0, 1) * 255).  `count` is the capacity of
 * rgba_out in bytes.  Synchronises the context stream. */
rdc_status rdc_read_rgba8(rdc_ctx* ctx, uint32_t sample_count, uint8_t* rgba_out,
                          size_t count);

/* Counters of the last render (synchronises the context stream). */
rdc_status rdc_stats_get(rdc_ctx* ctx, rdc_stats* out);

/* ---- batched rendering: many scenes in one persistent launch ---------- */

/* One scene of a batch: samples [0, spp) of every pixel, at most max_bounces
 * segments per path, RNG key `seed` and RNG stream = the item's index. */
typedef struct rdc_batch_item {
    const rdc_scene_desc* scene;
    uint32_t spp;
    uint32_t max_bounces;
    uint64_t seed;
} rdc_batch_item;

/* Launch shape of the persistent kernels. */
typedef struct rdc_launch_config {
    uint32_t block_size;      /* threads per block: 64, 128 or 256 */
    uint32_t blocks_per_sm;   /* resident blocks per SM, i.e. paths in flight per SM; 0 = as many as fit */
    uint32_t refill_min_idle; /* idle lanes of a warp before it takes new pixels (1..32) */
} rdc_launch_config;

/* Copy `count` scenes to the device as one batch (replacing any previous
 * batch of the context), allocate one accumulator per scene, and capture the
 * batch's launch (clear + persistent kernel) in a CUDA graph.  The reference
 * renders one scene per process run (src/main.rs:10-24); a batch is N such
 * render_frame calls (src/renderer/cpu.rs:119-133) fused into one launch. */
rdc_status rdc_batch_upload(rdc_ctx* ctx, const rdc_batch_item* items, uint32_t count);

/* Render every scene of the batch from cleared accumulators: one graph
 * launch on the context stream (returns once launched). */
rdc_status rdc_batch_render(rdc_ctx* ctx);

/* Copy scene `index`'s accumulator (its width*height*4 floats) to host memory. */
rdc_status rdc_batch_read_accum(rdc_ctx* ctx, uint32_t index, float* rgba_out, size_t count);

/* Set / get the batch launch shape (re-captures the graph). */
rdc_status rdc_batch_set_config(rdc_ctx* ctx, const rdc_launch_config* config);
rdc_status rdc_batch_get_config(rdc_ctx* ctx, rdc_launch_config* config);

/* Time the batch under a grid of launch shapes (block size x blocks per SM x
 * refill threshold), keep the fastest and return it with its device time.
 * Leaves the accumulators of the last trial; render again for results. */
rdc_status rdc_batch_autotune(rdc_ctx* ctx, rdc_launch_config* best_out, float* best_ms_out);

/* The same render as rdc_render, bit for bit, in wavefront form: per-path
 * state in device memory, one launch per bounce for the closest hits of all
 * queued rays and one for shading them, regrouped by material class
 * (diffuse/specular mix, metal, glass, miss) so each warp shades one class.
 * One wave is up to 16 consecutive samples of every pixel, at most 2^25
 * paths (88 bytes of device memory each: 2.9 GB at 1080p), a CUDA graph
 * replayed per wave; each pixel adds its samples in sample order, as
 * src/renderer/cpu.rs:198-210 does.
 * With an LBVH the closest hits come from a persistent kernel whose lanes
 * take queued rays as they finish their traversals (refill_min_idle of
 * rdc_set_render_config sets how many idle lanes trigger a refill).
 * Provided for the megakernel / wavefront comparison. */
rdc_status rdc_render_wavefront(rdc_ctx* ctx, uint32_t spp_begin, uint32_t spp_count, uint32_t max_bounces,
                                uint64_t seed);

/* ---- differentiation (path-replay adjoint) ------------------------------
 * The reference renderer is not differentiable; these two calls add the
 * gradient of an image loss with respect to per-object material parameters,
 * for the same estimator rdc_render evaluates (src/renderer/cpu.rs:253-341).
 * The image is the mean radiance, RGB per pixel, row-major (W*H*3 floats). */
#define RDC_MAX_ADJOINT_BOUNCES 16u

/* Render samples [spp_begin, spp_begin+spp_count) of every pixel from a
 * cleared accumulator (rdc_reset + rdc_render) and write the mean-radiance
 * image to image_out (W*H*3 floats; NULL to skip).  Remembers the sample
 * range, bounce limit and seed for rdc_backward. */
rdc_status rdc_forward(rdc_ctx* ctx, uint32_t spp_begin, uint32_t spp_count, uint32_t max_bounces,
                       uint64_t seed, float* image_out);

/* Gradient of L with respect to every object's parameters, given dl_dimage =
 * dL/dimage (W*H*3 floats) for the image of the last rdc_forward.  Outputs
 * (NULL to skip): grad_albedo (N*3), grad_roughness (N, w.r.t.
 * Material::roughness), grad_emission (N*3, w.r.t. the emitted radiance
 * emission_color * emission_strength).  Each path is replayed from its
 * random-number counter; nothing from the forward pass is stored.  The
 * roughness gradient has a pathwise part (roughness bends scatter directions)
 * and a lobe-choice part: where a coin whose probability depends on the
 * parameters picked the lobe -- U < roughness^2 for diffuse over specular
 * (src/renderer/cpu.rs:309), Schlick's reflectance for reflection over
 * refraction (cpu.rs:296-297) -- the path adds the radiance it gathers after
 * that choice times d log P (a score-function term, unbiased for
 * 0 < roughness < 1).  Not included: changes of which object a ray hits
 * (silhouette crossings) and the total-internal-reflection edge. */
rdc_status rdc_backward(rdc_ctx* ctx, const float* dl_dimage, float* grad_albedo, float* grad_roughness,
                        float* grad_emission);

/* Set / get the launch shape of rdc_render.  block_size and blocks_per_sm as
 * for a batch (default 256, 0); LBVH renders use blocks of at most 128
 * threads (their kernel is compiled for 5 such blocks per SM).
 * refill_min_idle applies to LBVH renders: a
 * warp keeps stepping its lanes' traversals until this many have finished,
 * then shades those together (default 16).  Brute-force renders refill each
 * idle lane at once.  Affects results never, speed only. */
rdc_status rdc_set_render_config(rdc_ctx* ctx, const rdc_launch_config* config);
rdc_status rdc_get_render_config(rdc_ctx* ctx, rdc_launch_config* config);

/* ---- fixed-input entry points (parity checks of single stages) -------- */

/* Closest hit of n rays against the uploaded scene: Ray::hit / trace_ray /
 * closest_hit (src/renderer/cpu.rs:23-98, 344-394).  origins and directions
 * are n*3 floats.  Outputs: t (n), object index (n, -1 on a miss), world
 * normal after the front-face flip (n*3), front-face flag (n). */
rdc_status rdc_intersect_rays(rdc_ctx* ctx, const float* origins, const float* directions,
                              uint32_t n, float* t_out, int32_t* index_out,
                              float* normal_out, uint8_t* front_out);

/* One scatter step with given random words: the hit branch of per_pixel
 * (src/renderer/cpu.rs:257-333) for n hits.  Per hit: the ray direction
 * (3 floats), object index, and 12 raw 32-bit random words (slots 0..10 are
 * used; their conversion to uniforms is part of the step).  The hit point,
 * normal and front face are recomputed from the ray origin + t.  Inputs:
 * origins/directions n*3, t n, index n, words n*12.  Outputs: new origin
 * n*3, new direction n*3. */
rdc_status rdc_scatter_fixed(rdc_ctx* ctx, const float* origins, const float* directions,
                             const float* t, const int32_t* index, const uint32_t* words,
                             uint32_t n, float* origin_out, float* direction_out);

/* ---- measurement ------------------------------------------------------ */

/* Measure the FP32 issue rate of the context's GPU: every SM runs
 * independent FFMA chains for a few milliseconds.  Reports FP32 lane
 * operations per second counting one per lane per clock (SMs x 128 x clock,
 * the bound of non-contracted FP32 code) and the SM clock that implies.
 * This is the denominator of the path tracer's roofline; the reference has no
 * counterpart (it reports wall-clock timers only, src/renderer/timing.rs). */
rdc_status rdc_measure_fp32_issue(rdc_ctx* ctx, double* lane_ops_per_second, double* sm_mhz);

/* The same with packed FP32x2 FMA chains (fma.rn.f32x2), counting both
 * components: the FP32 rate the packed two-sphere tests can reach. */
rdc_status rdc_measure_fp32x2_issue(rdc_ctx* ctx, double* lane_ops_per_second);

/* Self-test of the device-error path: runs one block whose shared-memory
 * staging wait cannot complete (the barrier expects bytes no copy delivers),
 * so the wait gives up after its bounded polls.  Returns RDC_ERR_DEVICE with
 * the message a render would give; the context stays usable. */
rdc_status rdc_selftest_staging_timeout(rdc_ctx* ctx);

/* Self-tests of the device sort and prefix sum the LBVH build runs (no
 * counterpart in the reference, which builds no hierarchy).  On n host
 * values: rdc_selftest_radix_sort sorts the pairs (keys, vals) by key,
 * stably, into keys_out / vals_out, for keys below 2^key_bits (key_bits
 * 1..32; passes of 10 bits); rdc_selftest_exclusive_scan writes out[i] =
 * in[0] + ... + in[i-1] (mod 2^32).  n <= RDC_MAX_OBJECTS. */
rdc_status rdc_selftest_radix_sort(rdc_ctx* ctx, const uint32_t* keys, const uint32_t* vals, uint32_t n,
                                   uint32_t key_bits, uint32_t* keys_out, uint32_t* vals_out);
rdc_status rdc_selftest_exclusive_scan(rdc_ctx* ctx, const uint32_t* in, uint32_t n, uint32_t* out);

/* ---- host-only helpers (no GPU needed) -------------------------------- */

/* Recompute a camera's view, projection and inverse matrices from its
 * position/target/up/resolution/projection/clip fields:
 * Camera::update_matrices (src/scene/camera.rs:210-231). */
rdc_status rdc_camera_update_matrices(rdc_camera* camera);

#ifdef __cplusplus
}
#endif

#endif /* RAYDAR_CUDA_H */
