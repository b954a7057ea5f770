/*
 * sr.h — C ABI of softrender-gb300, the GB300 (sm_103a) rendering hot path of
 * softrender (novacrazy/rust-softrender).
 *
 * The reference exposes a typestate builder chain (src/pipeline):
 *
 *   Pipeline::from_framebuffer(fb, uniforms)                 mod.rs:120-122
 *     .render_mesh(Triangle, mesh, Some(stencil_ref))        mod.rs:146-155
 *     -> VertexShader::run(vs) | run_to_fragment(vp, vs)     stages/vertex.rs:87,123
 *     -> GeometryShader::clip_primitives() / run(gs)         stages/geometry.rs:261,132
 *        .finish(viewport)                                   stages/geometry.rs:60
 *     -> FragmentShader.with_blend(b).cull_faces(c)
 *        .tile_size(t).run(fs)                               stages/fragment.rs:82-168
 *
 * Across this ABI the chain collapses into one sr_draw descriptor handed to
 * sr_render().  Shader stages are device functions compiled into the library
 * and selected by name (sr_shader_lookup).  All calls return an sr_status;
 * nothing aborts or traps.  Rendering calls are stream-ordered: sr_render
 * returns after enqueue and sr_sync() reports completion and any error the
 * device recorded (the reference panics at those points instead).
 *
 * Plain C types only: pointers, sizes and the POD structs below.
 */
#ifndef SR_H
#define SR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define SR_API
#else
#define SR_API __attribute__((visibility("default")))
#endif

/* ------------------------------------------------------------ status codes */
typedef enum sr_status {
    SR_OK = 0,
    SR_EINVAL = 1,     /* invalid argument (reference: assert!/panic)            */
    SR_ENOMEM = 2,     /* device or host allocation failed                      */
    SR_EBUDGET = 3,    /* request exceeds the HBM admission budget              */
    SR_EOVERFLOW = 4,  /* a fixed-capacity device buffer overflowed             */
    SR_ETIMEOUT = 5,   /* a bounded device or host wait gave up                 */
    SR_ECUDA = 6,      /* a CUDA runtime call failed                            */
    SR_ENAN = 7,       /* a triangle had an all-NaN bounding box, or a line NaN
                          end points after clipping; the reference panics in
                          clamp_as_int (triangle.rs:66-78) or in the i64 cast of
                          the end points (line.rs:111-116); here the primitive
                          is skipped and the draw reports this code             */
    SR_ENOTFOUND = 8,  /* unknown shader name                                   */
    SR_EBUSY = 9       /* resource in use                                       */
} sr_status;

/* ---------------------------------------------------------------- enums */
typedef enum sr_color_format {
    SR_COLOR_NONE = 0,
    SR_COLOR_RGBA32F = 1,   /* Vector4<f32>, 16 B per pixel */
    SR_COLOR_RGBA8 = 2      /* Vector4<u8>, 4 B per pixel, r in the low byte */
} sr_color_format;

typedef enum sr_prim { SR_PRIM_POINT = 1, SR_PRIM_LINE = 2, SR_PRIM_TRIANGLE = 3 } sr_prim;

typedef enum sr_gs_mode {
    SR_GS_NONE = 0,    /* VertexShader::run_to_fragment (vertex.rs:123-160)      */
    SR_GS_CLIP = 1,    /* .run(vs).clip_primitives().finish(vp) (geometry.rs:261) */
    SR_GS_NAMED = 2    /* .run(vs).run(named geometry shader).finish(vp)        */
} sr_gs_mode;

/* Option<FaceWinding> (src/geometry/winding.rs:11-44) */
typedef enum sr_cull { SR_CULL_NONE = 0, SR_CULL_CLOCKWISE = 1, SR_CULL_COUNTER_CLOCKWISE = 2 } sr_cull;

/* StencilTest (src/stencil.rs:94-129); `mask` is the mesh's stencil reference,
 * `value` the framebuffer's stencil. */
typedef enum sr_stencil_test {
    SR_STENCIL_ALWAYS = 0,
    SR_STENCIL_NEVER = 1,
    SR_STENCIL_LESS_THAN = 2,         /* mask <  value */
    SR_STENCIL_GREATER_THAN = 3,      /* mask >  value */
    SR_STENCIL_LESS_THAN_EQ = 4,      /* mask <= value */
    SR_STENCIL_GREATER_THAN_EQ = 5,   /* mask >= value */
    SR_STENCIL_EQUAL = 6,             /* mask == value */
    SR_STENCIL_NOT_EQUAL = 7          /* mask != value */
} sr_stencil_test;

/* StencilOp (src/stencil.rs:133-164); wrap selects Increment/Decrement{wrap}. */
typedef enum sr_stencil_op {
    SR_STENCIL_KEEP = 0,
    SR_STENCIL_INVERT = 1,
    SR_STENCIL_ZERO = 2,
    SR_STENCIL_REPLACE = 3,
    SR_STENCIL_INCREMENT = 4,
    SR_STENCIL_DECREMENT = 5
} sr_stencil_op;

typedef enum sr_stage {
    SR_STAGE_VERTEX = 0,
    SR_STAGE_GEOMETRY = 1,
    SR_STAGE_FRAGMENT = 2,
    SR_STAGE_BLEND = 3
} sr_stage;

/* Sampling for the textured shaders (src/texture.rs:14-18,89-113). */
typedef enum sr_filter { SR_SAMPLE_NEAREST = 0, SR_SAMPLE_BILINEAR = 1 } sr_filter;
/* Clamp: coordinates clamped to [0, 1]; wrap: fractional part; border:
 * outside [0, 1] reads transparent black (the reference's TextureRead::sample
 * is unimplemented, src/texture.rs:14-53). */
typedef enum sr_edge { SR_SAMPLE_CLAMP = 0, SR_SAMPLE_WRAP = 1, SR_SAMPLE_BORDER = 2 } sr_edge;

/* --------------------------------------------------------------- structs */

/* Framebuffer attachments (RenderBuffer<ColorDepthStencilAttachments<C,D,S>>,
 * src/framebuffer/renderbuffer/mod.rs:16-30).  Planes are stored SoA on the
 * device: colour plane, f32 depth plane, u8 stencil plane. */
typedef struct sr_fb_desc {
    uint32_t width;
    uint32_t height;
    uint32_t color_format;   /* sr_color_format */
    uint32_t depth;          /* 1: f32 depth attachment, 0: () */
    uint32_t stencil;        /* 1: u8 stencil attachment, 0: () */
} sr_fb_desc;

/* Viewport<f32> (src/geometry/clipvertex.rs:28-57) */
typedef struct sr_viewport {
    float x, y, width, height, near, far;
} sr_viewport;

typedef struct sr_pipeline sr_pipeline;
typedef struct sr_mesh sr_mesh;
typedef struct sr_texture sr_texture;

/* Re-rendering the outputs of earlier stages, as the reference's duplicate()
 * does (src/pipeline/stages/geometry.rs:40-54, fragment.rs:118-135: the
 * duplicate holds copies of the processed vertices and primitives, so a later
 * change of the uniforms does not reach them).
 *   SR_REUSE_VERTICES  the vertex-stage outputs of the pipeline's previous
 *                      draw feed this draw's geometry stage; both draws use a
 *                      geometry stage (SR_GS_CLIP or SR_GS_NAMED), the same
 *                      mesh, vertex shader and viewport
 *                      (GeometryShader::duplicate, then replace/finish)
 *   SR_REUSE_GEOMETRY  the previous draw's geometry-stage output is rasterised
 *                      again; primitive type, geometry mode and shader must
 *                      also match, so only culling, blend, tiles, stencil
 *                      reference, fragment shader, texture and line
 *                      anti-aliasing can differ (FragmentShader::duplicate)
 * A mismatch, no previous draw, or a mesh updated since is SR_EINVAL.  The
 * stages are skipped while their outputs are still resident and recomputed
 * from the saved inputs (the earlier uniforms) otherwise: the results are the
 * same either way. */
typedef enum sr_reuse { SR_REUSE_NONE = 0, SR_REUSE_VERTICES = 1, SR_REUSE_GEOMETRY = 2 } sr_reuse;

/* One pass of the typestate chain, flattened.  Defaults (sr_draw_init):
 * triangles, no GS, no culling, blend 0 (the `()` blend: replace), 128x128
 * semantic tiles (DEFAULT_TILE_SIZE, fragment.rs:29), stencil ref 0. */
typedef struct sr_draw {
    const sr_mesh* mesh;
    uint32_t prim;            /* sr_prim: T of render_mesh(T, ...)                 */
    int32_t vs;               /* vertex shader id                                  */
    uint32_t gs_mode;         /* sr_gs_mode                                        */
    int32_t gs;               /* geometry shader id for SR_GS_NAMED                */
    sr_viewport viewport;     /* run_to_fragment / finish viewport                 */
    uint32_t cull;            /* sr_cull: FragmentShader::cull_faces               */
    int32_t fs;               /* fragment shader id                                */
    int32_t blend;            /* blend id; 0 = `()` (source replaces destination) */
    uint32_t aa_lines;        /* FragmentShader::antialiased_lines                 */
    uint32_t tile_w, tile_h;  /* FragmentShader::tile_size (semantic tile)         */
    uint32_t stencil_ref;     /* render_mesh(.., Some(stencil)), default 0         */
    const sr_texture* texture;/* texture read by textured fragment shaders         */
    uint32_t tex_filter;      /* sr_filter */
    uint32_t tex_edge;        /* sr_edge */
    uint32_t reuse;           /* sr_reuse: duplicate() of an earlier stage         */
} sr_draw;

/* Per-draw counters gathered on the device. */
typedef struct sr_stats {
    uint64_t triangles_in;        /* input primitives (indices / 3)                */
    uint64_t triangles_generated; /* primitives after the geometry stage           */
    uint64_t triangles_raster;    /* primitives that can produce fragments         */
    uint64_t unsafe_triangles;    /* primitives rasterised against every tile      */
    uint64_t bin_entries;         /* (bin, primitive) pairs written by binning     */
    uint64_t fragments;           /* covered pixel centres reaching the depth test,
                                     counted once per pixel and primitive          */
    uint32_t nan_bbox;            /* primitives skipped for an all-NaN bbox        */
    uint32_t overflow;            /* nonzero if a fixed-capacity buffer overflowed */
    uint32_t kernel_launches;     /* kernels the draw launched                     */
    uint32_t profiled;            /* 1 if stage_ms holds timings                   */
    float stage_ms[6];            /* with sr_pipeline_set_profiling: device time of
                                     vertex, geometry, setup+binning, raster,
                                     stencil, total                               */
} sr_stats;

/* -------------------------------------------------------------- pipeline */

/* Pipeline::from_framebuffer (src/pipeline/mod.rs:110-140): width and height
 * must be non-zero (asserted there); the stencil config starts as Always/Keep.
 * `uniforms` points to an sr_uniforms (include/sr_shaders.h) and may be NULL. */
SR_API int sr_pipeline_create(const sr_fb_desc* fb, const void* uniforms, size_t uniforms_size,
                              sr_pipeline** out);
/* PipelineObject::uniforms_mut (src/pipeline/mod.rs:43-45) */
SR_API int sr_pipeline_set_uniforms(sr_pipeline* p, const void* uniforms, size_t uniforms_size);
/* PipelineObject::stencil_config_mut with GenericStencilConfig
 * (src/pipeline/mod.rs:86-88, src/stencil.rs:182-199) */
SR_API int sr_pipeline_set_stencil(sr_pipeline* p, int test, int op, int wrap);
/* PipelineObject::threadpool_mut (src/pipeline/mod.rs:78): the CUDA stream
 * (cudaStream_t as void*) that render calls are ordered on; NULL = legacy default.
 * Draws still pending on the previous stream are settled first, as sr_sync
 * does; their status is returned by the next sr_sync. */
SR_API int sr_pipeline_set_stream(sr_pipeline* p, void* stream);
SR_API int sr_pipeline_destroy(sr_pipeline* p);
/* Records CUDA events between the stages of every draw (no counterpart in the
 * reference, which has no profiling hooks); sr_get_stats then reports
 * stage_ms for the most recent draw. */
SR_API int sr_pipeline_set_profiling(sr_pipeline* p, int enable);

/* Framebuffer::clear (src/framebuffer/mod.rs:36, renderbuffer/mod.rs:125-133):
 * colour <- *color (float[4] for RGBA32F, uint8[4] for RGBA8), depth <- f32::MIN,
 * stencil <- 0, ordered on the stream after the draws enqueued so far (and
 * repeated in sequence if sr_sync has to replay them). */
SR_API int sr_framebuffer_clear(sr_pipeline* p, const void* color);
/* PixelRead / UnsafeFramebuffer getters (src/pixels/mod.rs:46-77): copy planes
 * to host memory (any pointer may be NULL); synchronises the pipeline stream. */
SR_API int sr_framebuffer_read(sr_pipeline* p, void* color, float* depth, uint8_t* stencil);
/* Enqueues the same copies on the pipeline's stream after the draws enqueued
 * so far and returns at once (no counterpart in the reference, whose reads are
 * synchronous).  Once the next sr_sync returns, the host buffers (pinned for a
 * truly asynchronous copy) hold the planes as they were at this point of the
 * sequence: a replay of the draws repeats the copy in its place. */
SR_API int sr_framebuffer_read_async(sr_pipeline* p, void* color, float* depth, uint8_t* stencil);
/* PixelWrite / UnsafeFramebuffer setters: host planes -> device (NULL skips).
 * Draws still pending are settled first, as sr_sync does; their status is
 * returned by the next sr_sync. */
SR_API int sr_framebuffer_write(sr_pipeline* p, const void* color, const float* depth,
                                const uint8_t* stencil);
/* Device addresses of the planes (for device-resident consumers). */
SR_API int sr_framebuffer_device_ptrs(sr_pipeline* p, void** color, float** depth, uint8_t** stencil);

/* ------------------------------------------------------------ resources */

/* Mesh<V> (src/mesh.rs:38-64) uploaded as SoA f32 attribute planes (each
 * n_verts floats; the vertex shader fixes their meaning) plus u32 indices.
 * Host buffers are copied before return; the mesh is immutable afterwards.
 * At most 2^31 vertices (SR_EINVAL beyond): vertex references are u32 and
 * the geometry stage adds up to 2^30 generated vertices after the mesh's. */
SR_API int sr_mesh_upload(const float* const* planes, uint32_t n_planes, uint32_t n_verts,
                          const uint32_t* indices, uint64_t n_indices, sr_mesh** out);
/* Replaces the contents of an uploaded mesh with new host data of the same
 * shape (plane count, vertex count, index count), without reallocating;
 * copies are ordered on `stream` (cudaStream_t as void*, NULL: synchronous).
 * Host buffers should be pinned for asynchronous copies.  Indices are not
 * scanned on the host here: primitives with an index >= n_verts are skipped
 * on the device and the next sr_sync returns SR_EINVAL. */
SR_API int sr_mesh_update(sr_mesh* m, const float* const* planes, uint32_t n_planes, uint32_t n_verts,
                          const uint32_t* indices, uint64_t n_indices, void* stream);
/* Releases the caller's handle.  Meshes are shared like the reference's
 * Arc<Mesh> (src/pipeline/mod.rs:146): a draw still pending on a pipeline
 * (until its sr_sync, which may replay it) and a server request not yet read
 * or released keep the mesh alive, and the last of them frees it. */
SR_API int sr_mesh_free(sr_mesh* m);
/* Device bytes held by a mesh (for HBM budgeting). */
SR_API uint64_t sr_mesh_bytes(const sr_mesh* m);

/* An RGBA8 texture (r in the low byte) read by the textured shaders. */
SR_API int sr_texture_upload(const uint32_t* rgba8, uint32_t width, uint32_t height, sr_texture** out);
/* Replaces the texels of an uploaded texture of the same size, ordered on
 * `stream` (NULL: synchronous). */
SR_API int sr_texture_update(sr_texture* t, const uint32_t* rgba8, uint32_t width, uint32_t height, void* stream);
/* Releases the caller's handle; pending draws and queued server requests
 * keep the texture alive as sr_mesh_free describes. */
SR_API int sr_texture_free(sr_texture* t);
/* An RGBA f32 texture (four floats per texel, r first), sampled by the
 * textured shaders like the RGBA8 ones but without the /255 conversion. */
SR_API int sr_texture_upload_rgba32f(const float* rgba, uint32_t width, uint32_t height, sr_texture** out);
/* Render to texture: copies a framebuffer's colour plane (RGBA8 or RGBA f32)
 * into a texture of the same size and texel type, ordered on the pipeline's
 * stream after its draws and repeated in its place if sr_sync replays them
 * (sr_sync the pipeline before draws on other pipelines sample it). */
SR_API int sr_texture_from_framebuffer(sr_pipeline* p, sr_texture* t);
/* Texture-buffer colour attachment (src/framebuffer/texturebuffer.rs:13-48,
 * 111-117, TextureBufferRef: the framebuffer's colour, stored apart from depth
 * and stencil, read as a texture without a copy): a texture that reads the
 * pipeline's colour plane in place, RGBA8 or RGBA f32.  It sees the
 * pipeline's draws once they are complete (sr_sync the pipeline, or draw on
 * the same stream).  The view holds a reference on the colour plane, as draws
 * hold references on meshes: destroying the pipeline leaves the plane (with
 * its last contents) to the views and the pending draws that sample them, and
 * the last sr_texture_free of a view frees it.  A draw may
 * not sample the plane it writes, a batch or a server request may not sample
 * a view at all, and sr_texture_update of a view is refused (SR_EINVAL). */
SR_API int sr_texture_view_framebuffer(sr_pipeline* p, sr_texture** out);

/* Shader registry: device functions compiled into the library, looked up by
 * name.  Stage is sr_stage.  Names: vertex "mvp_pos_nrm", "mvp_pos_nrm_uv",
 * "clip_color"; fragment "blinn_phong_dir", "textured_blinn_phong",
 * "vertex_color", "aces_lights", "constant_color"; blend "replace", "over";
 * geometry "clip", "vertex_normals", "face_normals". */
SR_API int sr_shader_lookup(const char* name, int stage, int* id);

/* --------------------------------------------------------------- render */

SR_API void sr_draw_init(sr_draw* d);
/* One pass of the chain Pipeline::render_mesh (src/pipeline/mod.rs:146-155)
 * -> VertexShader::run / run_to_fragment (stages/vertex.rs:87-160) ->
 * GeometryShader::clip_primitives + finish (stages/geometry.rs:60-129,
 * 261-336) -> FragmentShader::run (stages/fragment.rs:169-318), enqueued on
 * the pipeline's stream (see sr_draw). */
SR_API int sr_render(sr_pipeline* p, const sr_draw* d);
/* Waits for the pipeline's stream; returns the first device-recorded error of
 * the draws since the previous sync (SR_ENAN, SR_EOVERFLOW) or SR_ECUDA.
 * Scratch buffers that a draw outgrew are enlarged and the draws from the
 * first affected one replayed (up to 8 rounds); SR_EOVERFLOW means the frame
 * is incomplete: a draw needed more than 2^30 primitives or vertices out of
 * the geometry stage, or more than 2^32 - 1 (bin, primitive) pairs. */
SR_API int sr_sync(sr_pipeline* p);
/* Counters of the most recent sr_render (valid after sr_sync). */
SR_API int sr_get_stats(sr_pipeline* p, sr_stats* out);

/* ------------------------------------------------------------ batched draws
 * Many independent draws of uneven sizes rendered together: one launch per
 * stage (clear, vertex, setup, raster, resolve) pulls (draw, item) work items
 * from the whole batch, and the launch sequence is replayed as a CUDA graph.
 * Equivalent to sr_render(items[i].target, &items[i].draw) for every i (each
 * target's framebuffer ends up bit-identical).  The reference renders one
 * mesh per Pipeline::render_mesh call (src/pipeline/mod.rs:146-155); batching
 * has no counterpart there (src/lib.rs:43-44 notes that many small meshes are
 * slow).
 *
 * Eligible draws: triangles, gs_mode SR_GS_NONE (run_to_fragment), blend
 * "replace", no stencil writes (no stencil attachment, or test Always with op
 * Keep); every target distinct and synced (no draws pending since its last
 * sr_sync).  Others return SR_EINVAL / SR_EBUSY without rendering anything.
 * Uniforms come from each target (sr_pipeline_set_uniforms). */
typedef struct sr_batch sr_batch;
typedef struct sr_batch_item {
    sr_pipeline* target;        /* framebuffer and uniforms of this draw             */
    sr_draw draw;               /* as for sr_render                                  */
    uint32_t clear;             /* nonzero: clear the target first (depth f32::MIN)  */
    uint8_t clear_color[16];    /* clear colour in the target's format (RGBA32F: 4
                                   floats; RGBA8: 4 bytes, r first)                  */
} sr_batch_item;
SR_API int sr_batch_create(sr_batch** out);
SR_API int sr_batch_destroy(sr_batch* b);
/* Stream the batch runs on (NULL: the batch's own stream). */
SR_API int sr_batch_set_stream(sr_batch* b, void* stream);
/* use_graphs: replay the launch sequence as a CUDA graph (default 1);
 * autotune: measure the launch configurations once per batch size class and
 * keep the fastest (default 1). */
SR_API int sr_batch_set_options(sr_batch* b, int use_graphs, int autotune);
/* Forces a launch configuration: the 32x32 bins a primitive may span and
 * still be reduced in its bins' shared-memory keys (1..32, power of two),
 * the bbox pixels above which a primitive takes the large-primitive pass
 * instead, and the bin raster's CTAs per SM (1..8, capped at what fits); all
 * zero returns to the tuned / default choice.  Results do not depend on it. */
SR_API int sr_batch_set_config(sr_batch* b, uint32_t bins_per_primitive, uint32_t big_threshold, uint32_t ctas_per_sm);
SR_API int sr_batch_get_config(sr_batch* b, uint32_t* bins_per_primitive, uint32_t* big_threshold, uint32_t* ctas_per_sm);
/* Enqueues the batch (returns after enqueue; waits first for this batch
 * object's previous batch, whose host table it reuses). */
SR_API int sr_batch_render(sr_batch* b, const sr_batch_item* items, uint32_t n);
/* Waits for the last batch; SR_ENAN / SR_EINVAL (an index >= the vertex
 * count dropped its triangle) as sr_sync reports them. */
SR_API int sr_batch_sync(sr_batch* b);
/* Summed counters of the last batch (valid after sr_batch_sync). */
SR_API int sr_batch_get_stats(sr_batch* b, sr_stats* out);

/* ------------------------------------------------------------ serving
 * A request loop in front of the batched renderer.  Requests (a resident
 * mesh, a camera, a resolution) are admitted against an HBM budget, folded
 * into the next batch as soon as a batch slot and memory free up (several
 * batches run on the GPU at once, each on its own stream), rendered into
 * pooled device framebuffers that stay resident until the result is read,
 * and timed from submission to completion.  With `plain` set the same loop
 * serves each request alone through sr_render + sr_sync (the per-request
 * pipeline), for comparison.  Every request's result equals rendering it
 * alone with sr_render.  No counterpart in the reference (whose
 * Pipeline::render_mesh renders one mesh per call, src/pipeline/mod.rs:146). */
typedef struct sr_server sr_server;
typedef struct sr_server_config {
    uint64_t hbm_budget;        /* bytes the server may hold for framebuffers and
                                   scratch (0: 64 GiB)                            */
    uint32_t max_inflight;      /* batches on the GPU at once (0: 3)              */
    uint32_t max_batch;         /* requests per batch (0: 256)                    */
    uint32_t plain;             /* nonzero: one request at a time via sr_render   */
} sr_server_config;
typedef struct sr_request {
    sr_draw draw;               /* as for sr_render; eligible as for sr_batch_render */
    const void* uniforms;       /* the draw's sr_uniforms (copied at submission)  */
    size_t uniforms_size;
    uint32_t width, height;     /* framebuffer of the result (colour + f32 depth) */
    uint32_t color_format;      /* SR_COLOR_RGBA8 or SR_COLOR_RGBA32F             */
    uint8_t clear_color[16];    /* in the colour format                           */
} sr_request;
typedef struct sr_server_stats {
    uint64_t submitted, completed, batches;
    double mean_batch;          /* requests per batch                             */
    double p50_ms, p99_ms, mean_ms, max_ms;   /* submission -> completion         */
    double throughput_rps;      /* completed requests per second of serving time  */
    uint64_t peak_bytes;        /* largest admitted footprint                     */
} sr_server_stats;
SR_API int sr_server_create(const sr_server_config* cfg, sr_server** out);
/* Queues a request; returns at once with its ticket.  SR_EBUDGET if the
 * request alone exceeds the budget, SR_EINVAL if it is not eligible. */
SR_API int sr_server_submit(sr_server* s, const sr_request* r, uint64_t* ticket);
/* Waits for a request (SR_ETIMEOUT after timeout_ms). */
SR_API int sr_server_wait(sr_server* s, uint64_t ticket, uint32_t timeout_ms);
/* Copies a finished request's colour / depth to host memory (either may be
 * NULL) and releases its framebuffer. */
SR_API int sr_server_read(sr_server* s, uint64_t ticket, void* color, float* depth);
/* Releases a finished request's framebuffer without reading it. */
SR_API int sr_server_release(sr_server* s, uint64_t ticket);
/* Waits until every submitted request has finished (SR_ETIMEOUT). */
SR_API int sr_server_drain(sr_server* s, uint32_t timeout_ms);
SR_API int sr_server_get_stats(sr_server* s, sr_server_stats* out);
SR_API int sr_server_reset_stats(sr_server* s);
SR_API int sr_server_destroy(sr_server* s);

/* ---------------------------------------------------- allocation-free draw
 * sr_render_static has no counterpart in the reference.  It is for callers
 * that cannot let a library allocate device memory: an application whose own
 * allocator owns the GPU's memory, a real-time loop that cannot afford
 * cudaMalloc/cudaFree (and the device synchronisation they imply) inside a
 * frame, or a plugin given nothing but device pointers.  It draws one opaque
 * (blend "replace"), indexed triangle mesh with no geometry shader
 * (gs_mode SR_GS_NONE, as the sr_render chain run_to_fragment) and no stencil
 * attachment, producing the framebuffer sr_render produces for the same draw,
 * and it calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * Inputs and outputs are caller-owned DEVICE pointers:
 *   planes   n_planes attribute planes, plane j at planes + j * plane_stride
 *            (plane_stride a multiple of 4, >= n_verts; planes 16-byte aligned)
 *   indices  3 * n_triangles vertex indices; a triangle with an index >=
 *            n_verts draws nothing (this call does not wait for the GPU, so,
 *            unlike sr_sync, it cannot report that)
 *   texture  tex_w * tex_h RGBA8 texels (textured_blinn_phong only, else NULL)
 *   color    width * height pixels of fb->color_format (16-byte aligned for
 *            RGBA32F); depth: width * height f32 when fb->depth.  They are
 *            drawn into as they are: clearing them is the caller's job.
 * d->mesh and d->texture must be NULL; uniforms are an sr_uniforms.  Work is
 * enqueued on `stream` (NULL: the legacy default stream); the call returns
 * without waiting.
 *
 * Limits: width * height <= SR_STATIC_MAX_PIXELS, n_triangles <=
 * SR_STATIC_MAX_TRIANGLES, n_verts <= SR_STATIC_MAX_VERTICES; larger draws
 * return SR_EOVERFLOW without doing anything (use sr_render for them).  The
 * scratch is one fixed array of about 17.5 MiB in the library's device image,
 * held by every GPU that loads the library until the process exits.  Each
 * call clears the parts of it that must start at zero.
 *
 * All calls on a device share that one array: two calls whose work overlaps
 * on the GPU (different streams, or different host threads, without an
 * ordering between them) race and corrupt each other's output.  Order them
 * on one stream or with events.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress, with that device current);
 * make that first call before any stream capture begins.  Under CUDA's lazy
 * module loading (the default since CUDA 12.2) the driver loads this
 * library's device code, and with it reserves the array, only when it is
 * first needed on a device, which can be inside that first call: that
 * reservation is the driver's, not this call's, but it takes the time of a
 * device allocation, so make the first call on each device before a
 * latency-critical loop (a draw of an empty mesh is enough). */
#define SR_STATIC_MAX_PIXELS    (1u << 20)
#define SR_STATIC_MAX_TRIANGLES (1u << 16)
#define SR_STATIC_MAX_VERTICES  (1u << 16)
SR_API int sr_render_static(const sr_draw* d, const void* uniforms, size_t uniforms_size,
                            const float* planes, uint32_t n_planes, uint32_t plane_stride, uint32_t n_verts,
                            const uint32_t* indices, uint32_t n_triangles,
                            const uint32_t* texture, uint32_t tex_w, uint32_t tex_h,
                            const sr_fb_desc* fb, void* color, float* depth, void* stream);

/* Human-readable name of a status code. */
SR_API const char* sr_status_string(int status);
/* Library version, e.g. "softrender-gb300 0.1.0 sm_103a". */
SR_API const char* sr_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SR_H */
