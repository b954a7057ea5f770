//! Raw bindings to libsoftrender_gb300 (the C ABI of include/sr.h): the
//! rendering path of softrender (src/pipeline) on a GB300 GPU.  Every
//! function mirrors one declaration of the header; tests/test_abi.py checks
//! the two against each other.  The safe wrapper is the softrender-cuda crate.
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_int, c_void};

// ---- status codes and enumerations of include/sr.h
pub const SR_OK: c_int = 0;
pub const SR_EINVAL: c_int = 1;
pub const SR_ENOMEM: c_int = 2;
pub const SR_EBUDGET: c_int = 3;
pub const SR_EOVERFLOW: c_int = 4;
pub const SR_ETIMEOUT: c_int = 5;
pub const SR_ECUDA: c_int = 6;
pub const SR_ENAN: c_int = 7;
pub const SR_ENOTFOUND: c_int = 8;
pub const SR_EBUSY: c_int = 9;

pub const SR_COLOR_NONE: u32 = 0;
pub const SR_COLOR_RGBA32F: u32 = 1;
pub const SR_COLOR_RGBA8: u32 = 2;
pub const SR_PRIM_POINT: u32 = 1;
pub const SR_PRIM_LINE: u32 = 2;
pub const SR_PRIM_TRIANGLE: u32 = 3;
pub const SR_GS_NONE: u32 = 0;
pub const SR_GS_CLIP: u32 = 1;
pub const SR_GS_NAMED: u32 = 2;
pub const SR_CULL_NONE: u32 = 0;
pub const SR_CULL_CLOCKWISE: u32 = 1;
pub const SR_CULL_COUNTER_CLOCKWISE: u32 = 2;
pub const SR_STENCIL_ALWAYS: c_int = 0;
pub const SR_STENCIL_NEVER: c_int = 1;
pub const SR_STENCIL_LESS_THAN: c_int = 2;
pub const SR_STENCIL_GREATER_THAN: c_int = 3;
pub const SR_STENCIL_LESS_THAN_EQ: c_int = 4;
pub const SR_STENCIL_GREATER_THAN_EQ: c_int = 5;
pub const SR_STENCIL_EQUAL: c_int = 6;
pub const SR_STENCIL_NOT_EQUAL: c_int = 7;
pub const SR_STENCIL_KEEP: c_int = 0;
pub const SR_STENCIL_INVERT: c_int = 1;
pub const SR_STENCIL_ZERO: c_int = 2;
pub const SR_STENCIL_REPLACE: c_int = 3;
pub const SR_STENCIL_INCREMENT: c_int = 4;
pub const SR_STENCIL_DECREMENT: c_int = 5;
pub const SR_STAGE_VERTEX: c_int = 0;
pub const SR_STAGE_GEOMETRY: c_int = 1;
pub const SR_STAGE_FRAGMENT: c_int = 2;
pub const SR_STAGE_BLEND: c_int = 3;
pub const SR_SAMPLE_NEAREST: u32 = 0;
pub const SR_SAMPLE_BILINEAR: u32 = 1;
pub const SR_SAMPLE_CLAMP: u32 = 0;
pub const SR_SAMPLE_WRAP: u32 = 1;
pub const SR_SAMPLE_BORDER: u32 = 2;
pub const SR_REUSE_NONE: u32 = 0;
pub const SR_REUSE_VERTICES: u32 = 1;
pub const SR_REUSE_GEOMETRY: u32 = 2;
pub const SR_STATIC_MAX_PIXELS: u32 = 1 << 20;
pub const SR_STATIC_MAX_TRIANGLES: u32 = 1 << 16;
pub const SR_STATIC_MAX_VERTICES: u32 = 1 << 16;

#[repr(C)] pub struct sr_pipeline { _p: [u8; 0] }
#[repr(C)] pub struct sr_mesh { _p: [u8; 0] }
#[repr(C)] pub struct sr_texture { _p: [u8; 0] }
#[repr(C)] pub struct sr_batch { _p: [u8; 0] }
#[repr(C)] pub struct sr_server { _p: [u8; 0] }

#[repr(C)] #[derive(Clone, Copy)]
pub struct sr_fb_desc { pub width: u32, pub height: u32, pub color_format: u32, pub depth: u32, pub stencil: u32 }
#[repr(C)] #[derive(Clone, Copy)]
pub struct sr_viewport { pub x: f32, pub y: f32, pub width: f32, pub height: f32, pub near: f32, pub far: f32 }
#[repr(C)] #[derive(Clone, Copy)]
pub struct sr_draw {
    pub mesh: *const sr_mesh, pub prim: u32, pub vs: i32, pub gs_mode: u32, pub gs: i32,
    pub viewport: sr_viewport, pub cull: u32, pub fs: i32, pub blend: i32, pub aa_lines: u32,
    pub tile_w: u32, pub tile_h: u32, pub stencil_ref: u32, pub texture: *const sr_texture,
    pub tex_filter: u32, pub tex_edge: u32, pub reuse: u32,
}
#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct sr_stats {
    pub triangles_in: u64, pub triangles_generated: u64, pub triangles_raster: u64,
    pub unsafe_triangles: u64, pub bin_entries: u64, pub fragments: u64,
    pub nan_bbox: u32, pub overflow: u32, pub kernel_launches: u32, pub profiled: u32,
    pub stage_ms: [f32; 6],
}
#[repr(C)] #[derive(Clone, Copy)]
pub struct sr_batch_item { pub target: *mut sr_pipeline, pub draw: sr_draw, pub clear: u32, pub clear_color: [u8; 16] }
#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct sr_server_config { pub hbm_budget: u64, pub max_inflight: u32, pub max_batch: u32, pub plain: u32 }
#[repr(C)] #[derive(Clone, Copy)]
pub struct sr_request {
    pub draw: sr_draw, pub uniforms: *const c_void, pub uniforms_size: usize,
    pub width: u32, pub height: u32, pub color_format: u32, pub clear_color: [u8; 16],
}
#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct sr_server_stats {
    pub submitted: u64, pub completed: u64, pub batches: u64, pub mean_batch: f64,
    pub p50_ms: f64, pub p99_ms: f64, pub mean_ms: f64, pub max_ms: f64,
    pub throughput_rps: f64, pub peak_bytes: u64,
}

/// The uniforms of the shaders compiled into the library (sr_uniforms of
/// include/sr_shaders.h); the library fills `pv` and `mvp` itself.
#[repr(C)] #[derive(Clone, Copy)]
pub struct sr_uniforms {
    pub model: [f32; 16], pub mit: [f32; 16], pub view: [f32; 16], pub projection: [f32; 16],
    pub camera: [f32; 4], pub light_dir: [f32; 4], pub light_pos: [f32; 4], pub color: [f32; 4],
    pub intensity: f32, pub shininess: f32, pub ior: f32, pub gamma: f32,
    pub light_color: [[f32; 4]; 4], pub light_pos4: [[f32; 4]; 4], pub light_int4: [f32; 4],
    pub pv: [f32; 16], pub mvp: [f32; 16],
}

#[link(name = "softrender_gb300")]
extern "C" {
    // pipeline (Pipeline::from_framebuffer, uniforms_mut, stencil_config_mut, threadpool_mut)
    pub fn sr_pipeline_create(fb: *const sr_fb_desc, u: *const c_void, usz: usize, out: *mut *mut sr_pipeline) -> c_int;
    pub fn sr_pipeline_set_uniforms(p: *mut sr_pipeline, u: *const c_void, usz: usize) -> c_int;
    pub fn sr_pipeline_set_stencil(p: *mut sr_pipeline, test: c_int, op: c_int, wrap: c_int) -> c_int;
    pub fn sr_pipeline_set_stream(p: *mut sr_pipeline, stream: *mut c_void) -> c_int;
    pub fn sr_pipeline_destroy(p: *mut sr_pipeline) -> c_int;
    pub fn sr_pipeline_set_profiling(p: *mut sr_pipeline, enable: c_int) -> c_int;

    // framebuffer (Framebuffer::clear, the pixel getters and setters)
    pub fn sr_framebuffer_clear(p: *mut sr_pipeline, color: *const c_void) -> c_int;
    pub fn sr_framebuffer_read(p: *mut sr_pipeline, color: *mut c_void, depth: *mut f32, stencil: *mut u8) -> c_int;
    pub fn sr_framebuffer_read_async(p: *mut sr_pipeline, color: *mut c_void, depth: *mut f32, stencil: *mut u8) -> c_int;
    pub fn sr_framebuffer_write(p: *mut sr_pipeline, color: *const c_void, depth: *const f32, stencil: *const u8) -> c_int;
    pub fn sr_framebuffer_device_ptrs(p: *mut sr_pipeline, color: *mut *mut c_void, depth: *mut *mut f32,
                                      stencil: *mut *mut u8) -> c_int;

    // meshes (Arc<Mesh<V>>) and textures
    pub fn sr_mesh_upload(planes: *const *const f32, n_planes: u32, n_verts: u32,
                          idx: *const u32, n_idx: u64, out: *mut *mut sr_mesh) -> c_int;
    pub fn sr_mesh_update(m: *mut sr_mesh, planes: *const *const f32, n_planes: u32, n_verts: u32,
                          idx: *const u32, n_idx: u64, stream: *mut c_void) -> c_int;
    pub fn sr_mesh_free(m: *mut sr_mesh) -> c_int;
    pub fn sr_mesh_bytes(m: *const sr_mesh) -> u64;
    pub fn sr_texture_upload(rgba8: *const u32, w: u32, h: u32, out: *mut *mut sr_texture) -> c_int;
    pub fn sr_texture_update(t: *mut sr_texture, rgba8: *const u32, w: u32, h: u32, stream: *mut c_void) -> c_int;
    pub fn sr_texture_free(t: *mut sr_texture) -> c_int;
    pub fn sr_texture_upload_rgba32f(rgba: *const f32, w: u32, h: u32, out: *mut *mut sr_texture) -> c_int;
    pub fn sr_texture_from_framebuffer(p: *mut sr_pipeline, t: *mut sr_texture) -> c_int;
    pub fn sr_texture_view_framebuffer(p: *mut sr_pipeline, out: *mut *mut sr_texture) -> c_int;

    // shaders by name, one draw, completion
    pub fn sr_shader_lookup(name: *const c_char, stage: c_int, id: *mut c_int) -> c_int;
    pub fn sr_draw_init(d: *mut sr_draw);
    pub fn sr_render(p: *mut sr_pipeline, d: *const sr_draw) -> c_int;
    pub fn sr_sync(p: *mut sr_pipeline) -> c_int;
    pub fn sr_get_stats(p: *mut sr_pipeline, out: *mut sr_stats) -> c_int;

    // batched draws (section 4)
    pub fn sr_batch_create(out: *mut *mut sr_batch) -> c_int;
    pub fn sr_batch_destroy(b: *mut sr_batch) -> c_int;
    pub fn sr_batch_set_stream(b: *mut sr_batch, stream: *mut c_void) -> c_int;
    pub fn sr_batch_set_options(b: *mut sr_batch, use_graphs: c_int, autotune: c_int) -> c_int;
    pub fn sr_batch_set_config(b: *mut sr_batch, bins_per_primitive: u32, big_threshold: u32, ctas_per_sm: u32) -> c_int;
    pub fn sr_batch_get_config(b: *mut sr_batch, bins_per_primitive: *mut u32, big_threshold: *mut u32,
                               ctas_per_sm: *mut u32) -> c_int;
    pub fn sr_batch_render(b: *mut sr_batch, items: *const sr_batch_item, n: u32) -> c_int;
    pub fn sr_batch_sync(b: *mut sr_batch) -> c_int;
    pub fn sr_batch_get_stats(b: *mut sr_batch, out: *mut sr_stats) -> c_int;

    // the serving loop (section 4)
    pub fn sr_server_create(cfg: *const sr_server_config, out: *mut *mut sr_server) -> c_int;
    pub fn sr_server_submit(s: *mut sr_server, r: *const sr_request, ticket: *mut u64) -> c_int;
    pub fn sr_server_wait(s: *mut sr_server, ticket: u64, timeout_ms: u32) -> c_int;
    pub fn sr_server_read(s: *mut sr_server, ticket: u64, color: *mut c_void, depth: *mut f32) -> c_int;
    pub fn sr_server_release(s: *mut sr_server, ticket: u64) -> c_int;
    pub fn sr_server_drain(s: *mut sr_server, timeout_ms: u32) -> c_int;
    pub fn sr_server_get_stats(s: *mut sr_server, out: *mut sr_server_stats) -> c_int;
    pub fn sr_server_reset_stats(s: *mut sr_server) -> c_int;
    pub fn sr_server_destroy(s: *mut sr_server) -> c_int;

    // allocation-free draw (section 5)
    pub fn sr_render_static(d: *const sr_draw, uniforms: *const c_void, usz: usize, planes: *const f32,
                            n_planes: u32, plane_stride: u32, n_verts: u32, indices: *const u32, n_triangles: u32,
                            texture: *const u32, tex_w: u32, tex_h: u32, fb: *const sr_fb_desc,
                            color: *mut c_void, depth: *mut f32, stream: *mut c_void) -> c_int;

    // status names and version
    pub fn sr_status_string(status: c_int) -> *const c_char;
    pub fn sr_version() -> *const c_char;
}
