//! softrender's `Pipeline` builder chain (src/pipeline/mod.rs:110-155,
//! stages/vertex.rs:87-160, stages/geometry.rs:40-336,
//! stages/fragment.rs:82-318) over libsoftrender_gb300.
//!
//! The reference monomorphises Rust closures per call; here the stages carry
//! shader *names* (the library's registry of compiled device functions) and
//! the chain fills one `sr_draw` as it advances.  `FragmentShader::run` is the
//! only call that crosses the FFI: it enqueues the draw on the pipeline's
//! stream and returns; `Pipeline::sync` waits (the reference's `Pool::scoped`
//! returned when every tile was done).
use softrender_cuda_sys as sys;
use std::ffi::{CStr, CString};
use std::os::raw::{c_int, c_void};
use std::ptr;

/// A status code of the library (the reference panicked where most of these
/// are returned: `mod.rs:129-130,148`, `triangle.rs:70`).
#[derive(Debug, Clone, Copy, PartialEq, Eq)]
pub struct SrError(pub c_int);

impl std::fmt::Display for SrError {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
        let s = unsafe { CStr::from_ptr(sys::sr_status_string(self.0)) };
        write!(f, "{}", s.to_string_lossy())
    }
}
impl std::error::Error for SrError {}

pub type Result<T> = std::result::Result<T, SrError>;

fn check(st: c_int) -> Result<()> {
    if st == sys::SR_OK { Ok(()) } else { Err(SrError(st)) }
}

#[derive(Clone, Copy, Debug)]
pub enum Stage { Vertex, Geometry, Fragment, Blend }

/// The id of a shader compiled into the library ("mvp_pos_nrm",
/// "textured_blinn_phong", "over", ...).
pub fn shader_id(name: &str, stage: Stage) -> Result<c_int> {
    let st = match stage {
        Stage::Vertex => sys::SR_STAGE_VERTEX,
        Stage::Geometry => sys::SR_STAGE_GEOMETRY,
        Stage::Fragment => sys::SR_STAGE_FRAGMENT,
        Stage::Blend => sys::SR_STAGE_BLEND,
    };
    let c = CString::new(name).map_err(|_| SrError(sys::SR_EINVAL))?;
    let mut id = 0;
    check(unsafe { sys::sr_shader_lookup(c.as_ptr(), st, &mut id) })?;
    Ok(id)
}

#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Primitive { Point = 1, Line = 2, Triangle = 3 }

/// src/geometry/winding.rs:11-44
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum FaceWinding { Clockwise = 1, CounterClockwise = 2 }

#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum ColorFormat { None = 0, Rgba32f = 1, Rgba8 = 2 }

/// src/geometry/clipvertex.rs:50-59 (x, y, width, height, near, far)
#[derive(Clone, Copy, Debug)]
pub struct Viewport { pub x: f32, pub y: f32, pub width: f32, pub height: f32, pub near: f32, pub far: f32 }

impl Viewport {
    pub fn from_dimensions(width: u32, height: u32) -> Viewport {
        Viewport { x: 0.0, y: 0.0, width: width as f32, height: height as f32, near: 0.0, far: 1.0 }
    }
}

impl From<Viewport> for sys::sr_viewport {
    fn from(v: Viewport) -> sys::sr_viewport {
        sys::sr_viewport { x: v.x, y: v.y, width: v.width, height: v.height, near: v.near, far: v.far }
    }
}

/// src/stencil.rs:162-199: the stencil test, operation and wrap mode.
#[derive(Clone, Copy, Debug)]
pub struct StencilConfig { pub test: c_int, pub op: c_int, pub wrap: bool }

/// A mesh uploaded once as SoA f32 attribute planes and u32 indices.  The
/// library counts references like the reference's `Arc<Mesh>`: draws still
/// pending on a pipeline and queued server requests keep it alive, so the
/// handle may be dropped at any time.
pub struct GpuMesh { raw: *mut sys::sr_mesh }

impl GpuMesh {
    pub fn upload(planes: &[&[f32]], indices: &[u32]) -> Result<GpuMesh> {
        let n_verts = planes.first().map_or(0, |p| p.len());
        if planes.iter().any(|p| p.len() != n_verts) {
            return Err(SrError(sys::SR_EINVAL));
        }
        let ptrs: Vec<*const f32> = planes.iter().map(|p| p.as_ptr()).collect();
        let mut raw = ptr::null_mut();
        check(unsafe {
            sys::sr_mesh_upload(ptrs.as_ptr(), ptrs.len() as u32, n_verts as u32, indices.as_ptr(),
                                indices.len() as u64, &mut raw)
        })?;
        Ok(GpuMesh { raw })
    }
}

impl Drop for GpuMesh {
    fn drop(&mut self) { unsafe { sys::sr_mesh_free(self.raw); } }
}

/// An RGBA8 texture for the textured shaders (full_example/src/texture.rs).
pub struct GpuTexture { raw: *mut sys::sr_texture }

impl GpuTexture {
    pub fn upload_rgba8(texels: &[u32], width: u32, height: u32) -> Result<GpuTexture> {
        if texels.len() != (width as usize) * (height as usize) {
            return Err(SrError(sys::SR_EINVAL));
        }
        let mut raw = ptr::null_mut();
        check(unsafe { sys::sr_texture_upload(texels.as_ptr(), width, height, &mut raw) })?;
        Ok(GpuTexture { raw })
    }
}

impl Drop for GpuTexture {
    fn drop(&mut self) { unsafe { sys::sr_texture_free(self.raw); } }
}

/// Pipeline::from_framebuffer (src/pipeline/mod.rs:110-140): the framebuffer
/// (colour, depth, stencil planes) lives on the GPU, owned by the pipeline.
pub struct Pipeline { raw: *mut sys::sr_pipeline, width: u32, height: u32, format: ColorFormat }

impl Pipeline {
    pub fn from_framebuffer(width: u32, height: u32, format: ColorFormat, depth: bool, stencil: bool,
                            uniforms: &sys::sr_uniforms) -> Result<Pipeline> {
        let fb = sys::sr_fb_desc { width, height, color_format: format as u32, depth: depth as u32,
                                   stencil: stencil as u32 };
        let mut raw = ptr::null_mut();
        check(unsafe {
            sys::sr_pipeline_create(&fb, uniforms as *const _ as *const c_void,
                                    std::mem::size_of::<sys::sr_uniforms>(), &mut raw)
        })?;
        Ok(Pipeline { raw, width, height, format })
    }

    /// uniforms_mut() (mod.rs:43-45): the values later draws use.
    pub fn set_uniforms(&mut self, uniforms: &sys::sr_uniforms) -> Result<()> {
        check(unsafe {
            sys::sr_pipeline_set_uniforms(self.raw, uniforms as *const _ as *const c_void,
                                          std::mem::size_of::<sys::sr_uniforms>())
        })
    }

    /// stencil_config_mut() (mod.rs:86-88)
    pub fn set_stencil(&mut self, cfg: StencilConfig) -> Result<()> {
        check(unsafe { sys::sr_pipeline_set_stencil(self.raw, cfg.test, cfg.op, cfg.wrap as c_int) })
    }

    /// threadpool_mut() (mod.rs:78) becomes the CUDA stream draws run on
    /// (null: the pipeline's own stream).
    pub unsafe fn set_stream(&mut self, stream: *mut c_void) -> Result<()> {
        check(sys::sr_pipeline_set_stream(self.raw, stream))
    }

    /// Framebuffer::clear (src/framebuffer/renderbuffer/mod.rs:125-133):
    /// colour to `color` (16 bytes of RGBA f32, or 4 of RGBA8), depth to
    /// f32::MIN, stencil to 0.
    pub fn clear(&mut self, color: &[u8]) -> Result<()> {
        let need = match self.format { ColorFormat::Rgba32f => 16, ColorFormat::Rgba8 => 4, ColorFormat::None => 0 };
        if color.len() < need {
            return Err(SrError(sys::SR_EINVAL));
        }
        check(unsafe { sys::sr_framebuffer_clear(self.raw, color.as_ptr() as *const c_void) })
    }

    /// render_mesh (mod.rs:146-155): the start of one draw's chain.
    pub fn render_mesh<'a>(&'a mut self, prim: Primitive, mesh: &'a GpuMesh, stencil: Option<u8>)
                           -> VertexShader<'a> {
        let mut d: sys::sr_draw = unsafe { std::mem::zeroed() };
        unsafe { sys::sr_draw_init(&mut d) };
        d.mesh = mesh.raw;
        d.prim = prim as u32;
        d.stencil_ref = stencil.unwrap_or_default() as u32;
        d.viewport = Viewport::from_dimensions(self.width, self.height).into();
        VertexShader { p: self, d, err: None }
    }

    /// Waits for the pipeline's draws; reports their device-recorded errors.
    pub fn sync(&mut self) -> Result<()> { check(unsafe { sys::sr_sync(self.raw) }) }

    /// The colour plane (RGBA8 words, r in the low byte) and depth plane.
    pub fn read_rgba8(&mut self) -> Result<(Vec<u32>, Vec<f32>)> {
        let n = (self.width as usize) * (self.height as usize);
        let mut color = vec![0u32; n];
        let mut depth = vec![0f32; n];
        check(unsafe {
            sys::sr_framebuffer_read(self.raw, color.as_mut_ptr() as *mut c_void, depth.as_mut_ptr(),
                                     ptr::null_mut())
        })?;
        Ok((color, depth))
    }
}

impl Drop for Pipeline {
    fn drop(&mut self) { unsafe { sys::sr_pipeline_destroy(self.raw); } }
}

/// stages/vertex.rs: `run(vs)` leads to the geometry stage,
/// `run_to_fragment(vs)` straight to the fragment stage (no geometry shader,
/// vertices normalised with the viewport).
pub struct VertexShader<'a> { p: &'a mut Pipeline, d: sys::sr_draw, err: Option<SrError> }

impl<'a> VertexShader<'a> {
    fn set_vs(&mut self, vs: &str) {
        match shader_id(vs, Stage::Vertex) { Ok(id) => self.d.vs = id, Err(e) => self.err = Some(e) }
    }
    pub fn run(mut self, vs: &str) -> GeometryShader<'a> {
        self.set_vs(vs);
        GeometryShader { p: self.p, d: self.d, err: self.err }
    }
    pub fn run_to_fragment(mut self, vs: &str, viewport: Viewport) -> FragmentShader<'a> {
        self.set_vs(vs);
        self.d.gs_mode = sys::SR_GS_NONE;
        self.d.viewport = viewport.into();
        FragmentShader { p: self.p, d: self.d, err: self.err }
    }
    /// VertexShader::duplicate (vertex.rs:44): this draw re-renders the
    /// previous draw's vertex outputs (same mesh contents, shader, viewport).
    pub fn reuse_vertices(mut self) -> Self { self.d.reuse = sys::SR_REUSE_VERTICES; self }
}

/// stages/geometry.rs: `clip_primitives` (the clipping shader, geometry.rs:261)
/// or a named geometry shader, then `finish(viewport)`.
pub struct GeometryShader<'a> { p: &'a mut Pipeline, d: sys::sr_draw, err: Option<SrError> }

impl<'a> GeometryShader<'a> {
    pub fn clip_primitives(mut self) -> Self { self.d.gs_mode = sys::SR_GS_CLIP; self }
    pub fn run(mut self, gs: &str) -> Self {
        match shader_id(gs, Stage::Geometry) {
            Ok(id) => { self.d.gs_mode = sys::SR_GS_NAMED; self.d.gs = id; }
            Err(e) => self.err = Some(e),
        }
        self
    }
    pub fn finish(mut self, viewport: Viewport) -> FragmentShader<'a> {
        self.d.viewport = viewport.into();
        FragmentShader { p: self.p, d: self.d, err: self.err }
    }
}

/// stages/fragment.rs:82-168: blend, culling, line anti-aliasing, semantic
/// tile size, then `run(fs)`.
pub struct FragmentShader<'a> { p: &'a mut Pipeline, d: sys::sr_draw, err: Option<SrError> }

impl<'a> FragmentShader<'a> {
    pub fn with_blend(mut self, blend: &str) -> Self {
        match shader_id(blend, Stage::Blend) { Ok(id) => self.d.blend = id, Err(e) => self.err = Some(e) }
        self
    }
    pub fn with_default_blend(self) -> Self { self.with_blend("replace") }
    pub fn cull_faces(mut self, cull: Option<FaceWinding>) -> Self {
        self.d.cull = cull.map_or(sys::SR_CULL_NONE, |w| w as u32);
        self
    }
    pub fn antialiased_lines(mut self, enable: bool) -> Self { self.d.aa_lines = enable as u32; self }
    pub fn tile_size(mut self, width: u32, height: u32) -> Self { self.d.tile_w = width; self.d.tile_h = height; self }
    pub fn with_texture(mut self, tex: &'a GpuTexture, filter: u32, edge: u32) -> Self {
        self.d.texture = tex.raw;
        self.d.tex_filter = filter;
        self.d.tex_edge = edge;
        self
    }
    /// FragmentShader::duplicate (fragment.rs:118-135): this draw re-renders
    /// the previous draw's geometry outputs with its own fragment state.
    pub fn reuse_geometry(mut self) -> Self { self.d.reuse = sys::SR_REUSE_GEOMETRY; self }
    /// FragmentShader::run: enqueues the draw; `Pipeline::sync` waits for it.
    pub fn run(mut self, fs: &str) -> Result<()> {
        if let Some(e) = self.err {
            return Err(e);
        }
        self.d.fs = shader_id(fs, Stage::Fragment)?;
        check(unsafe { sys::sr_render(self.p.raw, &self.d) })
    }
}
