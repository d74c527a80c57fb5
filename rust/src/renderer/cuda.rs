//! The `--cuda` backend: Raydar's `trait Renderer` (src/renderer/mod.rs:25-35)
//! over libraydar_cuda, a drop-in for `CpuRenderer` (src/renderer/cpu.rs).
//! Lives in the reference's src/renderer/ beside cpu.rs and vulkan.rs, because
//! Profiler's timers are pub(super) (src/renderer/timing.rs:10-19); the
//! rust/raydar-cuda.patch adds `pub mod cuda;`, the `--cuda` flag and the
//! dependency on raydar-cuda-sys.
//!
//! Every library call returns a status; the trait returns no Result, so a
//! failure panics with the library's message (the Vulkan backend unwraps in
//! the same places).  The scene is uploaded on `new_frame` and on every
//! `render_sample`, which reads the `&Scene` it is given each call as
//! CpuRenderer::render_sample does (src/renderer/cpu.rs:142-158).
use image::{ImageBuffer, RgbaImage};
use raydar_cuda_sys as ffi;
use std::ffi::CStr;

use crate::scene::{camera::Projection, objects::Geometry, world::World, Scene};
use super::{timing::Profiler, Renderer, RendererConfig};

pub struct CudaRenderer {
    ctx: *mut ffi::rdc_ctx,
    profiler: Profiler,
    sample_count: u32,
    config: RendererConfig,
    seed: u64,
}

fn check(ctx: *mut ffi::rdc_ctx, st: ffi::rdc_status, what: &str) {
    if st != ffi::RDC_OK {
        // trait Renderer returns no Result: surface the library's message as a panic, as the Vulkan backend does.
        let msg = unsafe { CStr::from_ptr(ffi::rdc_last_error(ctx)) }.to_string_lossy();
        panic!("{what} failed ({st}): {msg}");
    }
}

fn v3(v: cgmath::Vector3<f32>) -> [f32; 3] { [v.x, v.y, v.z] }
fn p3(p: cgmath::Point3<f32>) -> [f32; 3] { [p.x, p.y, p.z] }
fn m4(m: cgmath::Matrix4<f32>) -> [f32; 16] { let a: &[f32; 16] = m.as_ref(); *a }

impl CudaRenderer {
    pub fn new(config: RendererConfig) -> Self {
        let mut ctx = std::ptr::null_mut();
        check(std::ptr::null_mut(), unsafe { ffi::rdc_create(&mut ctx, 0) }, "rdc_create");
        Self { ctx, profiler: Profiler::default(), sample_count: 0, config, seed: 0 }
    }

    // Flatten the Scene (src/scene/mod.rs:13-18) in object order and copy it to the device.
    fn upload(&mut self, scene: &Scene) {
        let c = &scene.camera;
        let (projection, fov, size) = match c.projection() {
            Projection::Perspective { fov } => (ffi::RDC_PROJECTION_PERSPECTIVE, fov.0, 0.0),
            Projection::Orthographic { size } => (ffi::RDC_PROJECTION_ORTHOGRAPHIC, 0.0, size),
        };
        let camera = ffi::rdc_camera {
            position: p3(c.position()), target: p3(c.target()), up: v3(c.up()),
            resolution_x: c.resolution_x(), resolution_y: c.resolution_y(),
            projection, fov_degrees: fov, ortho_size: size, near_clip: c.near_clip(), far_clip: c.far_clip(),
            view_matrix: m4(c.view_matrix()), proj_matrix: m4(c.proj_matrix()),
            inverse_view_matrix: m4(c.inverse_view_matrix()), inverse_proj_matrix: m4(c.inverse_proj_matrix()),
        };
        let mut world = ffi::rdc_world::default();
        match &scene.world {
            World::SkyColor { top_color, bottom_color } => {
                world.kind = ffi::RDC_WORLD_SKY_COLOR; world.top_color = v3(*top_color); world.bottom_color = v3(*bottom_color);
            }
            World::SolidColor(col) => { world.kind = ffi::RDC_WORLD_SOLID_COLOR; world.solid_color = v3(*col); }
            World::Transparent => world.kind = ffi::RDC_WORLD_TRANSPARENT, // rejected: RDC_ERR_UNSUPPORTED
        }
        let objects: Vec<ffi::rdc_object> = scene.objects.iter().map(|o| {
            let m = &o.material;
            let material = ffi::rdc_material {
                albedo: v3(m.albedo), roughness: m.roughness, metallic: m.metallic,
                emission_color: v3(m.emission_color), emission_strength: m.emission_strength,
                transmission: m.transmission, ior: m.ior,
            };
            match &o.geometry {
                Geometry::Sphere(s) => ffi::rdc_object { geometry: ffi::RDC_GEOMETRY_SPHERE, center: p3(s.center),
                                                         radius: s.radius, side_length: 0.0, material },
                Geometry::Cube(q) => ffi::rdc_object { geometry: ffi::RDC_GEOMETRY_CUBE, center: p3(q.center),
                                                       radius: 0.0, side_length: q.side_length, material },
            }
        }).collect();
        let desc = ffi::rdc_scene_desc { camera, world, objects: objects.as_ptr(), object_count: objects.len() as u32 };
        check(self.ctx, unsafe { ffi::rdc_scene_upload(self.ctx, &desc) }, "rdc_scene_upload");
    }

    fn image(&self, scene: &Scene) -> RgbaImage {
        let (w, h) = (scene.camera.resolution_x(), scene.camera.resolution_y());
        let mut buf = vec![0u8; (w * h * 4) as usize];
        check(self.ctx, unsafe { ffi::rdc_read_rgba8(self.ctx, self.sample_count, buf.as_mut_ptr(), buf.len()) },
              "rdc_read_rgba8");
        ImageBuffer::from_raw(w, h, buf).unwrap()
    }

    fn device_ms(&self) -> f32 {
        let mut s = ffi::rdc_stats::default();
        check(self.ctx, unsafe { ffi::rdc_stats_get(self.ctx, &mut s) }, "rdc_stats_get");
        s.device_ms
    }
}

impl Drop for CudaRenderer {
    fn drop(&mut self) { unsafe { ffi::rdc_destroy(self.ctx) } }
}

impl Renderer for CudaRenderer {
    fn render_frame(&mut self, scene: &Scene) -> RgbaImage {
        self.new_frame(scene);
        self.profiler.prepare_timer.end_if_not_ended();
        self.profiler.render_timer.start_if_not_started();
        self.profiler.sample_timer.start();
        let n = self.config.max_sample_count;
        check(self.ctx, unsafe { ffi::rdc_render(self.ctx, 0, n, self.config.max_bounces, self.seed) }, "rdc_render");
        self.device_ms(); // waits for the frame
        self.sample_count = n;
        self.profiler.sample_timer.end_multiple(n.max(1)); // all samples in one launch, as the Vulkan backend does
        self.profiler.render_timer.end();
        self.profiler.frame_timer.end();
        self.image(scene)
    }

    fn render_sample(&mut self, scene: &Scene) -> Option<RgbaImage> {
        if self.sample_count >= self.config.max_sample_count { return None; }
        self.upload(scene);
        self.profiler.prepare_timer.end_if_not_ended();
        self.profiler.render_timer.start_if_not_started();
        self.profiler.sample_timer.start();
        check(self.ctx, unsafe { ffi::rdc_render(self.ctx, self.sample_count, 1, self.config.max_bounces, self.seed) },
              "rdc_render");
        self.device_ms();
        self.sample_count += 1;
        if self.sample_count == self.config.max_sample_count {
            self.profiler.render_timer.end();
            self.profiler.frame_timer.end();
        }
        self.profiler.sample_timer.end();
        Some(self.image(scene))
    }

    fn new_frame(&mut self, scene: &Scene) {
        self.profiler.frame_timer.start();
        self.profiler.prepare_timer.start();
        self.upload(scene);
        check(self.ctx, unsafe { ffi::rdc_reset(self.ctx) }, "rdc_reset");
        self.sample_count = 0;
    }

    fn profiler(&self) -> &Profiler { &self.profiler }
    fn sample_count(&self) -> u32 { self.sample_count }
    fn max_sample_count(&self) -> u32 { self.config.max_sample_count }
    fn max_bounces(&self) -> u32 { self.config.max_bounces }
    fn set_max_sample_count(&mut self, count: u32) { self.config.max_sample_count = count; }
    fn set_max_bounces(&mut self, bounces: u32) { self.config.max_bounces = bounces; }
}
