/*
 * sr_oracle.h — CPU restatement of softrender's rendering path, used as the
 * parity oracle and the timed CPU baseline.  TEST INFRASTRUCTURE ONLY: the
 * product library never links, loads or calls this code.
 *
 * Parity status: the reference (Rust) cannot be built in this environment and
 * its own tests hold no raster golden vectors (the only value-pinning test is
 * coordinate_index, src/geometry/coordinate.rs:66-87, which the test suite
 * restates).  The restatement is pinned by line-cited equivalence and by the
 * hand-derived known-answer tests under tests/; "parity unpinned" against the
 * Rust binary itself.
 */
#ifndef SR_ORACLE_H
#define SR_ORACLE_H

#include <stdint.h>
#include <stddef.h>
#include "../include/sr_shaders.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_draw {
    const float* const* planes;   /* SoA vertex attribute planes             */
    uint32_t n_planes;
    uint32_t n_verts;
    const uint32_t* indices;
    uint64_t n_indices;
    uint32_t prim;                /* 1 point, 2 line, 3 triangle             */
    const char* vs;               /* vertex shader name                      */
    uint32_t gs_mode;             /* 0 none (run_to_fragment), 1 clip, 2 named */
    const char* gs;               /* named geometry shader                   */
    float viewport[6];            /* x, y, width, height, near, far          */
    uint32_t cull;                /* 0 none, 1 clockwise, 2 counter-clockwise */
    const char* fs;               /* fragment shader name                    */
    const char* blend;            /* "replace" or "over"                     */
    uint32_t aa_lines;
    uint32_t tile_w, tile_h;
    uint32_t stencil_ref;
    uint32_t stencil_test, stencil_op, stencil_wrap;
    const void* texture;          /* RGBA8 or RGBA f32 texels, may be NULL   */
    uint32_t tex_w, tex_h, tex_filter, tex_edge;
    uint32_t tex_f32;             /* 1: RGBA f32 texels                      */
    const sr_uniforms* uniforms;  /* derived fields must be filled           */
} or_draw;

typedef struct or_fb {
    uint32_t width, height;
    uint32_t color_format;        /* 0 none, 1 RGBA32F, 2 RGBA8              */
    void* color;
    float* depth;                 /* NULL: no depth attachment               */
    uint8_t* stencil;             /* NULL: no stencil attachment             */
} or_fb;

typedef struct or_stats {
    uint64_t triangles_generated; /* primitives leaving the geometry stage   */
    uint64_t fragments;           /* covered, z<0 pixel centres, owner pass  */
    uint64_t tiles;               /* semantic tiles in the frame             */
    uint32_t nan_bbox;            /* primitives with an all-NaN bbox         */
    uint32_t status;              /* 0 ok, else an sr_status code            */
    double vertex_s;              /* wall time of the vertex stage           */
    double geometry_s;            /* geometry stage + finish (clip GS only)  */
    double raster_s;              /* fragment stage over the tiles rendered  */
} or_stats;

/* Renders one draw into fb.  n_threads == 1 is the normative (deterministic)
 * order; n_threads > 1 mirrors Pool::new(num_cpus) with its atomic-counter
 * work split (outputs then race on seam pixels exactly as the reference's do
 * and are not compared); n_threads < 0 runs -n_threads workers in an order
 * whose result equals the 1-thread order (geometry outputs concatenated in
 * input order, tiles in phases that never run two tiles sharing a pixel at
 * once).  Only tiles [tile_begin, tile_end) of the row-major
 * tile list are rasterised (tile_end = UINT32_MAX for all). */
int or_render(const or_draw* d, or_fb* fb, int n_threads, uint32_t tile_begin, uint32_t tile_end,
              or_stats* stats);
/* As or_render, rasterising only the n tiles tile_first, tile_first +
 * tile_step, ... (those inside the tile list): a timing sample spread over
 * the whole frame.  tile_step = 0 returns 1. */
int or_render_strided(const or_draw* d, or_fb* fb, int n_threads, uint32_t tile_first, uint32_t tile_step,
                      uint32_t n, or_stats* stats);

/* Screen-space positions (x, y, z, 1/w per vertex, 12 floats per triangle)
 * of the triangles the fragment stage rasterises, after the vertex and
 * geometry stages; *n receives the count (out may hold fewer). */
int or_raster_tris(const or_draw* d, uint32_t width, uint32_t height, float* out, uint64_t cap, uint64_t* n);

/* Framebuffer::clear: colour <- color, depth <- f32::MIN, stencil <- 0 */
void or_clear(or_fb* fb, const void* color);

/* Helpers exposed for known-answer tests. */
void or_tiles(uint32_t width, uint32_t height, uint32_t tw, uint32_t th, uint32_t* out_rects,
              uint32_t cap, uint32_t* n_out);
void or_normalize(const float clip[4], const float viewport[6], float out[4]);
uint32_t or_clip_triangle(const float* a, const float* b, const float* c, uint32_t nk,
                          float* out, uint32_t cap);
float or_powf(float x, float y);
float or_u8_unit(uint32_t c);
uint64_t or_coordinate_into_index(uint32_t x, uint32_t y, uint32_t width);
void or_coordinate_from_index(uint64_t index, uint32_t width, uint32_t* x, uint32_t* y);
void or_derive_uniforms(sr_uniforms* u);

#ifdef __cplusplus
}
#endif

#endif
