// sr_internal.cuh — types shared by the kernels and the C-ABI host runtime.
//
// Device data layout (all in HBM, owned by the pipeline / mesh objects):
//   mesh planes      SoA f32, each plane padded to a multiple of 4 vertices
//                    (16-byte aligned planes)
//   mesh indices     u32, 3 per triangle
//   vertex store     clip4[v]  AoS float4 clip-space position (clip GS only)
//                    scr4[v]   AoS float4 screen position (x, y, z, 1/w)
//                    vary[v]   AoS varyings, stride VSTRIDE floats
//                    slots [0, n_verts) are mesh vertices, slots from
//                    gen_base on are vertices created by the clipper
//   raster triangles refs (3 u32 vertex-store slots per triangle) for
//                    generated primitives, or the mesh indices directly
//   setup records    4 float4 per raster triangle (edge terms, z, bbox)
//   bins             per-bin entry lists of raster-triangle indices
//   framebuffer      SoA planes: colour (RGBA f32 or RGBA8), f32 depth, u8 stencil
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <atomic>
#include <stdint.h>

#include "sr.h"
#include "sr_shaders.h"

// `#pragma unroll` in functions the host compiles too (the device pass only)
#ifdef __CUDA_ARCH__
#define SR_UNROLL _Pragma("unroll")
#else
#define SR_UNROLL
#endif

namespace sr {

constexpr int VSTRIDE = 12;        // varying floats per vertex (10 used at most)
constexpr int MAX_PLANES = 8;      // attribute planes read by a vertex shader
constexpr float F32_LOWEST = -3.40282347e+38f;   // f32::MIN, the depth clear value (attachments/depth.rs:31)

enum VsId { VS_MVP_POS_NRM = 0, VS_MVP_POS_NRM_UV = 1, VS_CLIP_COLOR = 2, VS_CLIP_RGBA8 = 3, VS_COUNT };
enum FsId { FS_BLINN_PHONG_DIR = 0, FS_TEXTURED_BLINN_PHONG = 1, FS_VERTEX_COLOR = 2,
            FS_ACES_LIGHTS = 3, FS_CONSTANT_COLOR = 4, FS_COUNT };
enum BlendId { BLEND_REPLACE = 0, BLEND_OVER = 1, BLEND_COUNT };
enum GsId { GS_CLIP = 0, GS_VERTEX_NORMALS = 1, GS_FACE_NORMALS = 2, GS_COUNT };

__host__ __device__ inline int vs_planes(int vs) { return vs == VS_MVP_POS_NRM ? 6 : vs == VS_CLIP_RGBA8 ? 4 : 8; }
__host__ __device__ constexpr int vs_nk(int vs) { return vs == VS_MVP_POS_NRM ? 8 : vs == VS_MVP_POS_NRM_UV ? 10 : 4; }

// Device error / counter block (one per pipeline).  The first part persists
// until sr_sync; the statistics part is zeroed at the start of every draw.
struct DeviceFlags {
    unsigned int poison;          // a stage overflowed: later framebuffer stages skip
    unsigned int overflow_bits;   // OVF_* bits
    unsigned int poison_draw;     // id of the first draw that overflowed (atomicMin)
    unsigned int nan_total;       // primitives met with an all-NaN bbox since the last sync
    unsigned int bad_index;       // a mesh index >= vertex count was met (primitive skipped)
    unsigned int copy_timeout;    // a tile copy's bounded wait gave up (the tile was skipped)
    unsigned long long need_gen_tris;
    unsigned long long need_gen_verts;
    unsigned long long need_entries;
    // ---- per-draw statistics (sr_stats) and device-side sizes
    unsigned long long triangles_generated;
    unsigned long long triangles_raster;
    unsigned long long unsafe;
    unsigned long long entries;
    unsigned long long fragments;
    unsigned long long n_gen_tris;     // raster triangles produced by the geometry stage
    unsigned long long n_gen_verts;
    unsigned long long n_unsafe_list;  // primitives on the unsafe list (extension pass)
    unsigned long long n_big;          // primitives on the large-bbox list (opaque path)
    unsigned int nan_bbox;
    unsigned int pad;
    unsigned long long work_raster;    // next primitive to hand out (dynamic raster work queue)
    unsigned long long work_resolve;   // next block to hand out (batched resolve)
};
constexpr size_t FLAGS_STATS_OFFSET = 48;
static_assert(offsetof(DeviceFlags, triangles_generated) == FLAGS_STATS_OFFSET, "DeviceFlags layout");

enum { OVF_GEN_TRIS = 1, OVF_GEN_VERTS = 2, OVF_ENTRIES = 4, OVF_SORT = 8 };

// Per-draw parameters passed by value to the kernels (constant bank).
struct DrawParams {
    uint32_t W, H;
    uint32_t tile_w, tile_h;
    uint32_t ncols, nrows;        // semantic tile grid
    uint32_t bin_w_log2, bin_h_log2;
    uint32_t bins_x, bins_y;
    uint32_t n_verts, gen_base;   // vertex-store slot of the first generated vertex
    uint32_t n_in;                // input primitives
    uint32_t n_raster_host;       // raster primitives when known on the host (0: read flags->n_gen_tris)
    uint32_t cull;
    uint32_t stencil_test, stencil_op, stencil_wrap, sref;
    uint32_t has_depth, has_stencil, color_format;
    uint32_t keep_degenerate;     // keep exactly-degenerate clip outputs (stencil events)
    uint32_t gen_tri_cap, gen_vert_cap;
    uint64_t entry_cap;
    float vp[6];
    int vs, fs, blend;
    uint32_t tex_w, tex_h, tex_filter, tex_edge;
    uint32_t tex_f32;             // the texture holds RGBA f32 texels
    uint32_t mode_b;              // exhaustive raster (stencil events gate fragments)
    uint32_t stencil_active;      // stencil plane changes during this draw
    uint32_t draw_id;             // sequence number of the draw since the last sync
    uint32_t force_unsafe;        // test hook: treat every primitive as unsafe
    uint32_t aa_lines;            // Xiaolin Wu lines (FragmentShader::antialiased_lines)
    uint32_t magic_w, magic_h;    // div_magic(tile_w), div_magic(tile_h): set with the tile size on the host
};

// Setup record of a raster triangle (64 bytes):
//   r0 = {A = y2-y3, B = x3-x2, C = y3-y1, D = x1-x3}
//   r1 = {x3, y3, det, z1}
//   r2 = {z2, z3, flags (bits), unused}
//   r3 = {ix0, iy0, ix1, iy1} integer bbox (floor), as int bits
enum { REC_UNSAFE = 1u, REC_RASTER = 2u };

struct Workspace;  // host side, defined in sr_api.cu

// Stencil event counters (see sr_stencil.cu)
struct StencilCountArgs {
    int* diff2d;                 // (W+1) x (H+1) 2D difference array
    int* lines;                  // CX, CXa, CXb (W+1 each), CY, CYl, CYr (H+1 each)
    unsigned long long* globals; // N, L, R, A, B, LA, LB, RA, RB
    int* colseg;                 // column scan scratch: stencil_colseg_rows(H) x (W+1)
};
// rows of the column-scan scratch: one per STENCIL_SEG rows of the (H+1)-row array
constexpr uint32_t STENCIL_SEG = 32;
inline uint32_t stencil_colseg_rows(uint32_t H) { return (H + 1 + STENCIL_SEG - 1) / STENCIL_SEG; }

// m = ceil(2^32 / t), so that floor(p / t) == umulhi32(p, m) for p < 2^15 and
// 2 <= t < 2^16 (m = (2^32 + e) / t with e < t: the excess p e / (t 2^32)
// stays below 1 / t).  For t == 1 it wraps to 0, which seam_count reads as
// "every coordinate is a multiple of t".  Computed once per draw on the host
// (DrawParams::magic_w, magic_h): the 64-bit division is slow on the device.
__host__ __device__ __forceinline__ uint32_t div_magic(uint32_t t) {
    return (uint32_t)((0x100000000ull + t - 1) / t);
}

// ------------------------------------------------------------ device helpers
__device__ __forceinline__ uint32_t zkey(float z) {
    uint32_t u = __float_as_uint(z);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float zkey_inv(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}
// floor(v) saturated to [lo, hi] as int; v must not be NaN
__device__ __forceinline__ int floor_sat(float v, int lo, int hi) {
    if (!(v >= (float)lo)) return lo;      // also -inf
    if (v >= (float)hi) return hi;
    return (int)floorf(v);
}

// StencilTest::test(value, mask) and StencilOp::op (src/stencil.rs:114-164)
__host__ __device__ __forceinline__ bool stencil_test(uint32_t test, uint32_t value, uint32_t mask) {
    switch (test) {
    case 0: return true;
    case 1: return false;
    case 2: return mask < value;
    case 3: return mask > value;
    case 4: return mask <= value;
    case 5: return mask >= value;
    case 6: return mask == value;
    default: return mask != value;
    }
}
__host__ __device__ __forceinline__ uint32_t stencil_op(uint32_t op, uint32_t wrap, uint32_t value, uint32_t mask) {
    switch (op) {
    case 0: return value;
    case 1: return (~value) & 0xffu;
    case 2: return 0;
    case 3: return mask;
    case 4: return wrap ? ((value + 1) & 0xffu) : (value == 255 ? 255 : value + 1);
    default: return wrap ? ((value - 1) & 0xffu) : (value == 0 ? 0 : value - 1);
    }
}

// Semantic tile geometry (fragment.rs:188-216): tile column C spans
// [C*tw, min((C+1)*tw, W-1)] inclusive; adjacent tiles share a column.
struct TileSpan {
    int first;   // first tile index containing the pixel
    int count;   // 1 or 2
};
__host__ __device__ __forceinline__ TileSpan tiles_of(uint32_t p, uint32_t t, uint32_t n, uint32_t last) {
    TileSpan s;
    if (p > 0 && p < last && (p % t) == 0) { s.first = (int)(p / t) - 1; s.count = 2; }
    else { uint32_t c = p / t; if (c > n - 1) c = n - 1; s.first = (int)c; s.count = 1; }
    return s;
}
// Schedule of the line / point raster: tile (c, r) runs in phase c + K r, the
// phases one after another and the tiles of a phase concurrently.  Tiles that
// can write a common pixel (seams; Xiaolin Wu lines also plot one pixel beyond
// their tile) are at most D tile columns apart, D = 1 + floor(2 / tile_w) for
// Wu lines and 1 otherwise; K = D + 1 keeps any two of them in distinct
// phases, in the row-major order the reference visits them.
__host__ __device__ __forceinline__ uint32_t lp_phase_step(bool wu_lines, uint32_t tile_w) {
    return (wu_lines && tile_w < 3) ? (tile_w == 2 ? 3u : 4u) : 2u;
}
// first tile row of phase `phase` (its column phase - K r is below ncols)
__host__ __device__ __forceinline__ uint32_t lp_phase_first_row(uint32_t phase, uint32_t ncols, uint32_t kstep) {
    return phase + 1 > ncols ? (phase - ncols + kstep) / kstep : 0u;
}

// Is coordinate p inside the projection of [i0, i1] clamped to tile index c?
// (clamp_as_int of triangle.rs:66-78, with floor-rounded bbox ends)
__device__ __forceinline__ bool clamp_axis(int i0, int i1, uint32_t p, uint32_t c, uint32_t t, uint32_t last) {
    uint32_t lo = c * t;
    uint32_t hi = min((c + 1) * t, last);
    int pi = (int)p;
    if (p == lo) return i0 <= pi;
    if (p == hi) return i1 >= pi;
    return i0 <= pi && pi <= i1;
}

// Sound segment test of the extension pass (see sr_setup.cu): true when one of
// the reference's u, v, w is certainly negative on the whole clamped segment
// [x0, x1] x [y0, y1] (one of the two ranges is a single coordinate).
__host__ __device__ __forceinline__ bool segment_cleared(float4 r0, float4 r1, uint32_t x0, uint32_t y0, uint32_t x1,
                                                         uint32_t y1) {
    const float g = 5.0e-7f;
    const float eps = 6.0e-8f;
    const float det = r1.z;
    const float s = det > 0.0f ? 1.0f : -1.0f;
    float nu[2], nv[2], Su[2], Sv[2];
    uint32_t xs[2] = {x0, x1}, ys[2] = {y0, y1};
SR_UNROLL
    for (int e = 0; e < 2; ++e) {
        float dx = ((float)xs[e] + 0.5f) - r1.x;
        float dy = ((float)ys[e] + 0.5f) - r1.y;
        nu[e] = r0.x * dx + r0.y * dy;
        nv[e] = r0.z * dx + r0.w * dy;
        Su[e] = fabsf(r0.x) * fabsf(dx) + fabsf(r0.y) * fabsf(dy);
        Sv[e] = fabsf(r0.z) * fabsf(dx) + fabsf(r0.w) * fabsf(dy);
    }
    float sum = fmaxf(Su[0], Su[1]), svm = fmaxf(Sv[0], Sv[1]);
    float tiny = fabsf(det) * 1.0e-30f;
    bool cu = (s * nu[0] + g * sum + tiny < 0.0f) && (s * nu[1] + g * sum + tiny < 0.0f);
    if (cu) return true;
    bool cv = (s * nv[0] + g * svm + tiny < 0.0f) && (s * nv[1] + g * svm + tiny < 0.0f);
    if (cv) return true;
    float mag = fabsf(det) + fmaxf(fabsf(nu[0]), fabsf(nu[1])) + fmaxf(fabsf(nv[0]), fabsf(nv[1]));
    float mw = 2.0f * g * (sum + svm) + 16.0f * eps * mag;
    bool cw = (s * (det - nu[0] - nv[0]) + mw < 0.0f) && (s * (det - nu[1] - nv[1]) + mw < 0.0f);
    return cw;
}

// The same sign test over the pixel rectangle [x0, x1] x [y0, y1]: the
// numerators and det - N_u - N_v are affine and their error bounds S convex,
// so the four corners decide (each bound taken at its largest corner).
__host__ __device__ __forceinline__ bool rect_cleared(float4 r0, float4 r1, int x0, int y0, int x1, int y1) {
    const float g = 5.0e-7f;
    const float eps = 6.0e-8f;
    const float det = r1.z;
    const float s = det > 0.0f ? 1.0f : -1.0f;
    float nu[4], nv[4], su = 0.0f, sv = 0.0f, mu = 0.0f, mv = 0.0f;
SR_UNROLL
    for (int e = 0; e < 4; ++e) {
        const float dx = ((float)((e & 1) ? x1 : x0) + 0.5f) - r1.x;
        const float dy = ((float)((e & 2) ? y1 : y0) + 0.5f) - r1.y;
        nu[e] = r0.x * dx + r0.y * dy;
        nv[e] = r0.z * dx + r0.w * dy;
        su = fmaxf(su, fabsf(r0.x) * fabsf(dx) + fabsf(r0.y) * fabsf(dy));
        sv = fmaxf(sv, fabsf(r0.z) * fabsf(dx) + fabsf(r0.w) * fabsf(dy));
        mu = fmaxf(mu, fabsf(nu[e]));
        mv = fmaxf(mv, fabsf(nv[e]));
    }
    const float tiny = fabsf(det) * 1.0e-30f;
    bool cu = true, cv = true, cw = true;
    const float mw = 2.0f * g * (su + sv) + 16.0f * eps * (fabsf(det) + mu + mv);
SR_UNROLL
    for (int e = 0; e < 4; ++e) {
        cu = cu && (s * nu[e] + g * su + tiny < 0.0f);
        cv = cv && (s * nv[e] + g * sv + tiny < 0.0f);
        cw = cw && (s * (det - nu[e] - nv[e]) + mw < 0.0f);
    }
    return cu || cv || cw;
}

}  // namespace sr

// Opaque handles of the C ABI
// Meshes and textures are shared like the reference's Arc<Mesh>
// (src/pipeline/mod.rs:146): the caller's handle holds one reference, and so
// does every draw that may still read the object (a pending draw until sync,
// a queued server request until read); the last release frees it.
struct sr_mesh {
    float* planes = nullptr;        // n_planes planes of n_pad floats
    uint32_t n_planes = 0;
    uint32_t n_verts = 0;
    uint32_t n_pad = 0;
    uint32_t* indices = nullptr;
    uint64_t n_indices = 0;
    uint64_t bytes = 0;
    uint64_t version = 0;           // bumped by every sr_mesh_update
    std::atomic<uint32_t> refs{1};
};

// A pipeline's colour plane, shared with the texture views of it: the
// pipeline and every view hold a reference, the last release frees it.
struct sr_color_plane {
    void* data = nullptr;
    std::atomic<uint32_t> refs{1};
};

struct sr_texture {
    uint32_t* data = nullptr;       // RGBA8 texels, or RGBA f32 texels (4 floats each) when f32
    uint32_t w = 0, h = 0;
    uint32_t f32 = 0;               // 1: RGBA f32 texels
    // RGBA8 textures that the library writes (uploads, updates, framebuffer
    // copies; not views): every texel also as its four c / 255 values, kept
    // in step with `data` on the same streams, which is what draws sample
    float4* unit = nullptr;
    bool view = false;              // reads a pipeline's colour plane in place (`plane`, referenced)
    sr_color_plane* plane = nullptr;
    std::atomic<uint32_t> refs{1};
};

// The texels a draw samples and whether they are RGBA f32 (sr_sample): an
// RGBA8 texture's unit expansion when it has one -- the same values the
// sampler would derive from its bytes -- else its own texels.
inline const uint32_t* sampled_texels(const sr_texture* t, uint32_t* f32) {
    if (!t) { *f32 = 0; return nullptr; }
    if (!t->f32 && t->unit) { *f32 = 1; return reinterpret_cast<const uint32_t*>(t->unit); }
    *f32 = t->f32;
    return t->data;
}

// ------------------------------------------------------- grid sizing (host)
// Streaming-multiprocessor count of the current device (cached per device).
inline int sm_count() {
    static int n[64] = {0};
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= 64) d = 0;
    if (!n[d] && (cudaDeviceGetAttribute(&n[d], cudaDevAttrMultiProcessorCount, d) != cudaSuccess || n[d] <= 0))
        n[d] = 152;
    return n[d];
}
// Grid of a persistent (grid-stride) kernel: as many CTAs as can be resident
// at once (at most max_per_sm per SM), so no CTA waits for another to exit.
template <typename K>
inline unsigned resident_grid(K kernel, int threads, int max_per_sm) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0) != cudaSuccess || nb <= 0) nb = 1;
    if (nb > max_per_sm) nb = max_per_sm;
    return (unsigned)nb * (unsigned)sm_count();
}

// ---------------------------------------------------------------- launches
// Kernel launchers implemented in the .cu files (host-callable).
namespace sr {

struct VertexStore {
    float4* clip4;
    float4* scr4;
    float* vary;
    uint32_t cap;
};

void launch_vertex(const DrawParams& P, const sr_uniforms& U, const sr_mesh* m, VertexStore vs,
                   bool write_clip, cudaStream_t st);
void launch_clip(const DrawParams& P, const sr_mesh* m, VertexStore vs, unsigned long long* counts,
                 unsigned long long* offsets, unsigned long long* scan_tmp, uint32_t* refs,
                 DeviceFlags* flags, cudaStream_t st);
void launch_setup_bin(const DrawParams& P, const uint32_t* vidx, VertexStore vs, float4* setup,
                      uint32_t* binrect, uint32_t* bin_counts, uint32_t* bin_off, uint32_t* bin_cursor,
                      uint32_t* entries, uint32_t* scan_tmp, uint32_t* unsafe_list, float4* unsafe_rect,
                      unsigned long long* area, const StencilCountArgs& S, DeviceFlags* flags, cudaStream_t st);

void launch_stencil_apply(const DrawParams& P, const StencilCountArgs& S, uint8_t* stencil,
                          DeviceFlags* flags, cudaStream_t st);

struct OpaqueArgs {
    const float4* setup;
    unsigned long long* area;        // per raster primitive: bbox pixels in the frame (setup output)
    uint32_t* big_list;              // primitives with more than RG_BIG bbox pixels
    unsigned long long* gkeys;       // W x H winner keys, zero between draws
    uint32_t* bitmap;                // touched 32x32 blocks, zero between draws
    const uint32_t* unsafe_list;
    const float4* unsafe_rect;       // per unsafe-list entry: its coverage region (NaN: unbounded), or null
    const uint32_t* vidx;
    const float* vary;
    const uint32_t* tex;
    void* color;
    float* depth;
    const uint8_t* stencil;
    uint32_t gate;
    DeviceFlags* flags;
};
// Opaque draws (sr_opaque.cu); returns the number of kernels launched.
int launch_opaque(const DrawParams& P, const sr_uniforms& U, const OpaqueArgs& A, cudaStream_t st);
// Opaque draws over 32x32 screen bins (sr_tiled.cu), after setup has counted
// each bin's primitives; returns the number of kernels launched.
// Primitives of one bin a raster work item reduces (the bin raster's CTA
// size); a bin of e listed primitives has ceil(e / BIN_CHUNK) work items.
constexpr uint32_t BIN_CHUNK = 256;
// Capacity of a work-item -> bin table (the batched bin raster's) for
// `entries` list entries over `bins` bins: ceil(e_b / BIN_CHUNK) items per
// bin, one for a bin with only keys from elsewhere.
inline uint64_t bin_item_cap(uint64_t entries, uint64_t bins) { return entries / BIN_CHUNK + 2 * bins + 1; }

struct TiledArgs {
    const float4* setup;
    const uint2* binrect;            // per raster primitive: its bbox's bin rectangle (setup output)
    const uint32_t* bin_counts;      // primitives per bin (setup output)
    uint32_t* cursor;                // n_bins slot counters, zero
    uint32_t* bin_off;               // n_bins + 1 list offsets
    uint32_t* chunk_off;             // n_bins + 1 offsets of the bins' raster work items
    uint32_t* entries;               // the bins' primitive lists
    uint64_t entry_cap;
    unsigned long long* gkeys;       // W x H extension keys, zero between draws
    uint32_t* bitmap;                // bins holding extension keys, zero between draws
    uint32_t* gids;                  // 1024 winner slots per bin (bin-major)
    const uint32_t* unsafe_list;
    const float4* unsafe_rect;       // per unsafe-list entry: its coverage region (NaN: unbounded)
    const uint32_t* vidx;
    const float* vary;
    const uint32_t* tex;
    void* color;
    float* depth;
    const uint8_t* stencil;
    uint32_t gate;
    DeviceFlags* flags;
};
int launch_tiled(const DrawParams& P, const sr_uniforms& U, const TiledArgs& A, cudaStream_t st);
// Bin lists of the ordered path (sr_bins.cu): pairs counted per primitive,
// written in primitive order and stably radix-sorted by bin.
struct BinBuffers {
    uint32_t* pcount;       // n + 1 pair counts
    uint32_t* poff;         // n + 1 exclusive offsets (poff[n] = pairs)
    uint32_t* scan_tmp;     // scratch of the scans
    uint32_t* keys[2];      // bin ids (ping-pong), capacity cap
    uint32_t* vals[2];      // primitive ids (ping-pong), capacity cap
    uint32_t* hist;         // 256 x radix_blocks(cap)
    uint32_t* hist_off;     // its exclusive scan
    uint32_t* ranges;       // [begin, end) per bin
    uint64_t cap;           // pair capacity
};
uint32_t radix_blocks(uint64_t cap);
// Returns the sorted primitive list (one of vals[]).
uint32_t* launch_bins(const DrawParams& P, const uint2* binrect, const float4* setup, const uint32_t* unsafe_list,
                      const BinBuffers& B, DeviceFlags* flags, cudaStream_t st);

// Lines and points (sr_lp.cu).  An LP vertex is 64 bytes: screen position
// and 12 varyings.
struct LPV;
void launch_lp_geometry(const DrawParams& P, const sr_uniforms& U, const sr_mesh* m, VertexStore vs, uint32_t prim_n,
                        uint32_t gs_mode, uint32_t gs, LPV* out, uint8_t* valid, DeviceFlags* flags,
                        cudaStream_t st);
uint32_t launch_lp_raster(const DrawParams& P, const sr_uniforms& U, const LPV* v, const uint8_t* valid,
                          uint32_t n_prims, uint32_t prim_n, const uint32_t* tex, void* color, float* depth,
                          uint8_t* stencil, DeviceFlags* flags, cudaStream_t st);
// Blending / stencil-gated draws over sorted bins (sr_raster.cu).
void launch_ordered(const DrawParams& P, const sr_uniforms& U, const float4* setup, const uint32_t* bin_off,
                    const uint32_t* entries, const uint32_t* vidx, const float* vary, const uint32_t* tex, void* color,
                    float* depth, uint8_t* stencil, uint32_t gate, DeviceFlags* flags, cudaStream_t st);

}  // namespace sr
