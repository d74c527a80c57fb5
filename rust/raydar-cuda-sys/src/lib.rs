//! FFI declarations of libraydar_cuda, one per entry point of
//! include/raydar_cuda.h, with the header's structures in repr(C) layout.
//! Raydar's `CudaRenderer` (src/renderer/cuda.rs) is the only user; it maps a
//! non-OK status to a panic carrying rdc_last_error's message, since the
//! reference's `trait Renderer` (src/renderer/mod.rs:25-35) returns no Result.
#![allow(non_camel_case_types)]
use std::mem::size_of;
use std::os::raw::{c_char, c_int, c_void};

pub type rdc_status = c_int;
pub const RDC_OK: rdc_status = 0;
pub const RDC_ERR_INVALID_ARGUMENT: rdc_status = 1;
pub const RDC_ERR_UNSUPPORTED: rdc_status = 2;
pub const RDC_ERR_LIMIT: rdc_status = 3;
pub const RDC_ERR_NO_SCENE: rdc_status = 4;
pub const RDC_ERR_CUDA: rdc_status = 5;
pub const RDC_ERR_OUT_OF_MEMORY: rdc_status = 6;
pub const RDC_ERR_DEVICE: rdc_status = 7;

pub const RDC_GEOMETRY_SPHERE: u32 = 0;
pub const RDC_GEOMETRY_CUBE: u32 = 1;
pub const RDC_WORLD_SKY_COLOR: u32 = 0;
pub const RDC_WORLD_SOLID_COLOR: u32 = 1;
pub const RDC_WORLD_TRANSPARENT: u32 = 2;
pub const RDC_PROJECTION_PERSPECTIVE: u32 = 0;
pub const RDC_PROJECTION_ORTHOGRAPHIC: u32 = 1;
pub const RDC_ACCEL_AUTO: u32 = 0;
pub const RDC_ACCEL_BRUTE_FORCE: u32 = 1;
pub const RDC_ACCEL_LBVH: u32 = 2;
pub const RDC_FORM_AUTO: u32 = 0;
pub const RDC_FORM_MEGAKERNEL: u32 = 1;
pub const RDC_FORM_WAVEFRONT: u32 = 2;
pub const RDC_FORM_AUTO_WAVE_SAMPLES: u32 = 4;

pub const RDC_MAX_RESOLUTION: u32 = 16384;
pub const RDC_MAX_OBJECTS: u32 = 1 << 24;
pub const RDC_MAX_BRUTE_OBJECTS: u32 = 4096;
pub const RDC_MAX_BOUNCES: u32 = 1024;
pub const RDC_MAX_ADJOINT_BOUNCES: u32 = 16;
pub const RDC_STATIC_MAX_OBJECTS: u32 = 1024;
pub const RDC_STATIC_SCRATCH_BYTES: u32 = 164096;

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct rdc_camera {
    pub position: [f32; 3],
    pub target: [f32; 3],
    pub up: [f32; 3],
    pub resolution_x: u32,
    pub resolution_y: u32,
    pub projection: u32,
    pub fov_degrees: f32,
    pub ortho_size: f32,
    pub near_clip: f32,
    pub far_clip: f32,
    pub view_matrix: [f32; 16],
    pub proj_matrix: [f32; 16],
    pub inverse_view_matrix: [f32; 16],
    pub inverse_proj_matrix: [f32; 16],
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct rdc_world {
    pub kind: u32,
    pub top_color: [f32; 3],
    pub bottom_color: [f32; 3],
    pub solid_color: [f32; 3],
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct rdc_material {
    pub albedo: [f32; 3],
    pub roughness: f32,
    pub metallic: f32,
    pub emission_color: [f32; 3],
    pub emission_strength: f32,
    pub transmission: f32,
    pub ior: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct rdc_object {
    pub geometry: u32,
    pub center: [f32; 3],
    pub radius: f32,
    pub side_length: f32,
    pub material: rdc_material,
}

#[repr(C)]
pub struct rdc_scene_desc {
    pub camera: rdc_camera,
    pub world: rdc_world,
    pub objects: *const rdc_object,
    pub object_count: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct rdc_stats {
    pub segments: u64,
    pub paths: u64,
    pub device_ms: f32,
    pub sample_count: u32,
    pub kernel_launches: u32,
    pub h2d_bytes: u64,
    pub d2h_bytes: u64,
    pub node_visits: u64,
    pub prim_tests: u64,
    pub accel: u32,
    pub bvh_depth: u32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct rdc_batch_item {
    pub scene: *const rdc_scene_desc,
    pub spp: u32,
    pub max_bounces: u32,
    pub seed: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct rdc_launch_config {
    pub block_size: u32,
    pub blocks_per_sm: u32,
    pub refill_min_idle: u32,
}

/// Opaque context (one per thread at a time, as `&mut self` implies).
pub enum rdc_ctx {}

// The header's layouts on a 64-bit target.
const _: () = assert!(size_of::<rdc_camera>() == 320);
const _: () = assert!(size_of::<rdc_world>() == 40);
const _: () = assert!(size_of::<rdc_material>() == 44);
const _: () = assert!(size_of::<rdc_object>() == 68);
const _: () = assert!(size_of::<rdc_scene_desc>() == 376);
const _: () = assert!(size_of::<rdc_stats>() == 72);
const _: () = assert!(size_of::<rdc_batch_item>() == 24);
const _: () = assert!(size_of::<rdc_launch_config>() == 12);

extern "C" {
    // lifetime
    pub fn rdc_version() -> *const c_char;
    pub fn rdc_create(out: *mut *mut rdc_ctx, device: c_int) -> rdc_status;
    pub fn rdc_destroy(ctx: *mut rdc_ctx);
    pub fn rdc_last_error(ctx: *const rdc_ctx) -> *const c_char;
    pub fn rdc_get_stream(ctx: *mut rdc_ctx, stream_out: *mut *mut c_void) -> rdc_status;
    pub fn rdc_synchronize(ctx: *mut rdc_ctx) -> rdc_status;

    // scene
    pub fn rdc_scene_parse_rscn(text: *const c_char, length: usize, scene_out: *mut rdc_scene_desc,
                                objects_out: *mut rdc_object, capacity: u32, count_out: *mut u32) -> rdc_status;
    pub fn rdc_scene_write_rscn(scene: *const rdc_scene_desc, buf: *mut c_char, capacity: usize,
                                length_out: *mut usize) -> rdc_status;
    pub fn rdc_scene_upload(ctx: *mut rdc_ctx, scene: *const rdc_scene_desc) -> rdc_status;
    pub fn rdc_set_accel(ctx: *mut rdc_ctx, mode: u32) -> rdc_status;
    pub fn rdc_set_render_form(ctx: *mut rdc_ctx, form: u32) -> rdc_status;
    pub fn rdc_update_materials(ctx: *mut rdc_ctx, materials: *const rdc_material, count: u32) -> rdc_status;

    // rendering
    pub fn rdc_reset(ctx: *mut rdc_ctx) -> rdc_status;
    pub fn rdc_render(ctx: *mut rdc_ctx, spp_begin: u32, spp_count: u32, max_bounces: u32, seed: u64) -> rdc_status;
    pub fn rdc_render_static(scene: *const rdc_scene_desc, accum_device: *mut f32, spp_begin: u32, spp_count: u32,
                             max_bounces: u32, seed: u64, stream: *mut c_void, segments_out: *mut u64,
                             error_out: *mut c_char, error_capacity: usize) -> rdc_status;
    pub fn rdc_read_accum(ctx: *mut rdc_ctx, rgba_out: *mut f32, count: usize) -> rdc_status;
    pub fn rdc_write_accum(ctx: *mut rdc_ctx, rgba_in: *const f32, count: usize, sample_count: u32) -> rdc_status;
    pub fn rdc_read_rgba8(ctx: *mut rdc_ctx, sample_count: u32, rgba_out: *mut u8, count: usize) -> rdc_status;
    pub fn rdc_stats_get(ctx: *mut rdc_ctx, out: *mut rdc_stats) -> rdc_status;
    pub fn rdc_render_wavefront(ctx: *mut rdc_ctx, spp_begin: u32, spp_count: u32, max_bounces: u32,
                                seed: u64) -> rdc_status;
    pub fn rdc_set_render_config(ctx: *mut rdc_ctx, config: *const rdc_launch_config) -> rdc_status;
    pub fn rdc_get_render_config(ctx: *mut rdc_ctx, config: *mut rdc_launch_config) -> rdc_status;

    // many scenes in one persistent launch (a CUDA graph)
    pub fn rdc_batch_upload(ctx: *mut rdc_ctx, items: *const rdc_batch_item, count: u32) -> rdc_status;
    pub fn rdc_batch_render(ctx: *mut rdc_ctx) -> rdc_status;
    pub fn rdc_batch_read_accum(ctx: *mut rdc_ctx, index: u32, rgba_out: *mut f32, count: usize) -> rdc_status;
    pub fn rdc_batch_set_config(ctx: *mut rdc_ctx, config: *const rdc_launch_config) -> rdc_status;
    pub fn rdc_batch_get_config(ctx: *mut rdc_ctx, config: *mut rdc_launch_config) -> rdc_status;
    pub fn rdc_batch_autotune(ctx: *mut rdc_ctx, best_out: *mut rdc_launch_config, best_ms_out: *mut f32)
                              -> rdc_status;

    // differentiation: image = mean radiance (W*H*3); gradients per object
    pub fn rdc_forward(ctx: *mut rdc_ctx, spp_begin: u32, spp_count: u32, max_bounces: u32, seed: u64,
                       image_out: *mut f32) -> rdc_status;
    pub fn rdc_backward(ctx: *mut rdc_ctx, dl_dimage: *const f32, grad_albedo: *mut f32, grad_roughness: *mut f32,
                        grad_emission: *mut f32) -> rdc_status;

    // single-stage checks and measurement
    pub fn rdc_intersect_rays(ctx: *mut rdc_ctx, origins: *const f32, directions: *const f32, n: u32,
                              t_out: *mut f32, index_out: *mut i32, normal_out: *mut f32, front_out: *mut u8)
                              -> rdc_status;
    pub fn rdc_scatter_fixed(ctx: *mut rdc_ctx, origins: *const f32, directions: *const f32, t: *const f32,
                             index: *const i32, words: *const u32, n: u32, origin_out: *mut f32,
                             direction_out: *mut f32) -> rdc_status;
    pub fn rdc_measure_fp32_issue(ctx: *mut rdc_ctx, lane_ops_per_second: *mut f64, sm_mhz: *mut f64)
                                  -> rdc_status;
    pub fn rdc_measure_fp32x2_issue(ctx: *mut rdc_ctx, lane_ops_per_second: *mut f64) -> rdc_status;
    pub fn rdc_selftest_staging_timeout(ctx: *mut rdc_ctx) -> rdc_status;
    pub fn rdc_selftest_radix_sort(ctx: *mut rdc_ctx, keys: *const u32, vals: *const u32, n: u32, key_bits: u32,
                                   keys_out: *mut u32, vals_out: *mut u32) -> rdc_status;
    pub fn rdc_selftest_exclusive_scan(ctx: *mut rdc_ctx, input: *const u32, n: u32, out: *mut u32)
                                       -> rdc_status;

    // host only
    pub fn rdc_camera_update_matrices(camera: *mut rdc_camera) -> rdc_status;
}
