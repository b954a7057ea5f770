// sr_lp.cu — lines and points: their geometry stage (indexed, the clipping
// arms of clip_primitives, the normal-visualisation geometry shaders) and
// their rasterisation (rasterization/line.rs, rasterization/point.rs).
//
// Geometry: every input primitive yields a fixed number of output slots
// (0 or 1 line / point for clipping, 3 or 1 lines for the normal shaders), so
// outputs keep input order without compaction; a per-slot flag marks the
// ones clipping removed.  Output vertices are screen vertices (normalised,
// finish()) with their 12 varyings.
//
// Raster: the reference visits every primitive in every semantic tile, in
// submission order, and tiles overlap by one row/column.  Tile (r, c) runs in
// phase c + 2r: two tiles sharing a pixel are always in different phases, in
// row-major order ((r, c) < (r, c+1) < (r+1, c) < (r+1, c+1)), so launching
// the phases in order reproduces the reference's order on seam pixels while
// the tiles of a phase run concurrently.  In a tile one warp tests 32
// primitives at a time against the tile (Liang-Barsky for lines, the
// half-open test for points); the hits are plotted one after another in
// submission order by the lane that owns them.
#include "sr_internal.cuh"
#include "sr_shade.cuh"
#include "sr_vertex.cuh"

namespace sr {

struct LPV {
    float4 p;            // screen position (x, y, z, 1/w)
    float4 k0, k1, k2;   // varyings
};

// All three varying quads of a vertex slot; those beyond the vertex shader's
// varyings are not written by the vertex stage and are carried along unused.
__device__ __forceinline__ void load_k(const float* __restrict__ vary, uint32_t slot, float4& a, float4& b, float4& c) {
    const float4* q = reinterpret_cast<const float4*>(vary + (size_t)slot * VSTRIDE);
    a = __ldg(q);
    b = __ldg(q + 1);
    c = __ldg(q + 2);
}

// ------------------------------------------------------------- geometry
// Indexed primitives (run_to_fragment): copy the normalised vertices.
__global__ void lp_indexed_kernel(uint32_t n_prims, uint32_t prim_n, uint32_t n_verts,
                                  const uint32_t* __restrict__ idx, const float4* __restrict__ scr4,
                                  const float* __restrict__ vary, LPV* __restrict__ out,
                                  uint8_t* __restrict__ valid, DeviceFlags* flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_prims) return;
    bool ok = true;
    for (uint32_t j = 0; j < prim_n; ++j) {
        const uint32_t v = __ldg(idx + (size_t)i * prim_n + j);
        if (v >= n_verts) { ok = false; atomicOr(&flags->bad_index, 1u); break; }
        LPV o;
        o.p = __ldg(scr4 + v);
        load_k(vary, v, o.k0, o.k1, o.k2);
        out[(size_t)i * prim_n + j] = o;
    }
    valid[i] = ok ? 1 : 0;
}

struct CVx {   // clip-space vertex with varyings (ClipVertex, geometry/clipvertex.rs:6-14)
    float p[4];
    float k[12];
};

__device__ __forceinline__ CVx load_cv(const float4* __restrict__ clip4, const float* __restrict__ vary, uint32_t v) {
    CVx c;
    const float4 p = __ldg(clip4 + v);
    c.p[0] = p.x; c.p[1] = p.y; c.p[2] = p.z; c.p[3] = p.w;
    float4 a, b, d;
    load_k(vary, v, a, b, d);
    c.k[0] = a.x; c.k[1] = a.y; c.k[2] = a.z; c.k[3] = a.w;
    c.k[4] = b.x; c.k[5] = b.y; c.k[6] = b.z; c.k[7] = b.w;
    c.k[8] = d.x; c.k[9] = d.y; c.k[10] = d.z; c.k[11] = d.w;
    return c;
}

// ClippingPlane::has_inside (geometry/clip.rs:33-44), planes L, R, T, B, Near, Far
__device__ __forceinline__ bool has_inside(int plane, const CVx& v) {
    const float x = v.p[0], y = v.p[1], z = v.p[2], w = v.p[3];
    switch (plane) {
    case 0: return x >= -w;
    case 1: return x <= w;
    case 2: return y >= -w;
    case 3: return y <= w;
    case 4: return z >= 0.0f;
    default: return z <= w;
    }
}

// ClippingPlane::intersect (geometry/clip.rs:46-63); lerp of interpolate.rs:56-57
__device__ __forceinline__ CVx intersect(int plane, const CVx& v1, const CVx& v2) {
    float a, b;
    switch (plane) {
    case 0: a = v1.p[3] + v1.p[0]; b = v2.p[3] + v2.p[0]; break;
    case 1: a = v1.p[3] - v1.p[0]; b = v2.p[3] - v2.p[0]; break;
    case 2: a = v1.p[3] + v1.p[1]; b = v2.p[3] + v2.p[1]; break;
    case 3: a = v1.p[3] - v1.p[1]; b = v2.p[3] - v2.p[1]; break;
    case 4: a = v1.p[2]; b = v2.p[2]; break;
    default: a = v1.p[3] - v1.p[2]; b = v2.p[3] - v2.p[2]; break;
    }
    const float t = a / (a - b);
    CVx o;
#pragma unroll
    for (int i = 0; i < 4; ++i) o.p[i] = (1.0f - t) * v1.p[i] + t * v2.p[i];
#pragma unroll
    for (int i = 0; i < 12; ++i) o.k[i] = (1.0f - t) * v1.k[i] + t * v2.k[i];
    return o;
}

__device__ __forceinline__ LPV finish_v(const CVx& c, const VpMatrix& vpm) {
    LPV o;
    const sr_v4 s = normalize_pos(sr_make_v4(c.p[0], c.p[1], c.p[2], c.p[3]), vpm.m);
    o.p = make_float4(s.x, s.y, s.z, s.w);
    o.k0 = make_float4(c.k[0], c.k[1], c.k[2], c.k[3]);
    o.k1 = make_float4(c.k[4], c.k[5], c.k[6], c.k[7]);
    o.k2 = make_float4(c.k[8], c.k[9], c.k[10], c.k[11]);
    return o;
}

// clip_primitives, line arm (geometry.rs:300-328) and point arm (:329-333).
__global__ void lp_clip_kernel(uint32_t n_prims, uint32_t prim_n, uint32_t n_verts, VpMatrix vpm,
                               const uint32_t* __restrict__ idx, const float4* __restrict__ clip4,
                               const float* __restrict__ vary, LPV* __restrict__ out, uint8_t* __restrict__ valid,
                               DeviceFlags* flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_prims) return;
    uint32_t v0 = __ldg(idx + (size_t)i * prim_n), v1 = prim_n == 2 ? __ldg(idx + (size_t)i * prim_n + 1) : v0;
    if (v0 >= n_verts || v1 >= n_verts) { atomicOr(&flags->bad_index, 1u); valid[i] = 0; return; }
    if (prim_n == 1) {
        const CVx p = load_cv(clip4, vary, v0);
        bool in = true;
        for (int plane = 0; plane < 6; ++plane) in = in && has_inside(plane, p);
        valid[i] = in ? 1 : 0;
        if (in) out[i] = finish_v(p, vpm);
        return;
    }
    CVx start = load_cv(clip4, vary, v0), end = load_cv(clip4, vary, v1);
    int intersections = 0;
    for (int plane = 0; plane < 6; ++plane) {
        const bool s_in = has_inside(plane, start), p_in = has_inside(plane, end);
        if (s_in != p_in) {
            const CVx inter = intersect(plane, start, end);
            if (s_in) end = inter;
            else start = inter;
            intersections += 1;
        } else if (!s_in) {
            valid[i] = 0;
            return;
        }
        if (intersections > 2) break;
    }
    out[2 * (size_t)i] = finish_v(start, vpm);
    out[2 * (size_t)i + 1] = finish_v(end, vpm);
    valid[i] = 1;
}

// The normal-visualisation geometry shaders (full_example/src/shaders.rs:35-89):
// a triangle emits its three vertex normals (`vertex_normals`) or its face
// normal (`face_normals`) as lines of length 0.05 from the world position in
// varyings 0..3 along the normal in varyings 4..7, projected by
// projection * view; lines and points are re-emitted unchanged.
__global__ void lp_normals_kernel(uint32_t n_prims, uint32_t prim_n, uint32_t n_verts, uint32_t face, sr_uniforms U,
                                  VpMatrix vpm, const uint32_t* __restrict__ idx, const float4* __restrict__ clip4,
                                  const float* __restrict__ vary, LPV* __restrict__ out, uint8_t* __restrict__ valid,
                                  DeviceFlags* flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_prims) return;
    uint32_t v[3];
    bool ok = true;
    for (uint32_t j = 0; j < prim_n; ++j) {
        v[j] = __ldg(idx + (size_t)i * prim_n + j);
        ok = ok && v[j] < n_verts;
    }
    // valid flags are per output primitive: 3 lines per triangle for vertex
    // normals, 1 for face normals, the primitive itself otherwise
    const uint32_t per = (prim_n == 3 && !face) ? 3u : 1u;
    if (!ok) {
        atomicOr(&flags->bad_index, 1u);
        for (uint32_t j = 0; j < per; ++j) valid[(size_t)i * per + j] = 0;
        return;
    }
    const float NORMAL_LENGTH = 0.05f;
    if (prim_n != 3) {
        for (uint32_t j = 0; j < prim_n; ++j) out[(size_t)i * prim_n + j] = finish_v(load_cv(clip4, vary, v[j]), vpm);
        valid[i] = 1;
        return;
    }
    if (!face) {
        for (int j = 0; j < 3; ++j) {
            CVx a = load_cv(clip4, vary, v[j]);
            const sr_v4 pos = sr_make_v4(a.k[0], a.k[1], a.k[2], a.k[3]);
            const sr_v4 nrm = sr_make_v4(a.k[4], a.k[5], a.k[6], a.k[7]);
            const sr_v4 st = sr_m4_mul_v4(U.pv, pos);
            const sr_v4 en = sr_m4_mul_v4(U.pv, sr_add4(pos, sr_scale4(nrm, NORMAL_LENGTH)));
            CVx b = a;
            a.p[0] = st.x; a.p[1] = st.y; a.p[2] = st.z; a.p[3] = st.w;
            b.p[0] = en.x; b.p[1] = en.y; b.p[2] = en.z; b.p[3] = en.w;
            out[6 * (size_t)i + 2 * j] = finish_v(a, vpm);
            out[6 * (size_t)i + 2 * j + 1] = finish_v(b, vpm);
            valid[3 * (size_t)i + j] = 1;
        }
        return;
    } else {
        const float ONE_THIRD = 1.0f / 3.0f;
        const CVx a = load_cv(clip4, vary, v[0]), b = load_cv(clip4, vary, v[1]), c = load_cv(clip4, vary, v[2]);
        CVx m;
        for (int q = 0; q < 4; ++q) m.p[q] = 0.0f;
        for (int q = 0; q < 12; ++q) m.k[q] = (a.k[q] * ONE_THIRD + b.k[q] * ONE_THIRD) + c.k[q] * ONE_THIRD;
        const sr_v4 pos = sr_make_v4(m.k[0], m.k[1], m.k[2], m.k[3]);
        const sr_v4 nrm = sr_make_v4(m.k[4], m.k[5], m.k[6], m.k[7]);
        const sr_v4 st = sr_m4_mul_v4(U.pv, pos);
        const sr_v4 en = sr_m4_mul_v4(U.pv, sr_add4(pos, sr_scale4(sr_normalize4(nrm), NORMAL_LENGTH)));
        CVx s = m, e = m;
        s.p[0] = st.x; s.p[1] = st.y; s.p[2] = st.z; s.p[3] = st.w;
        e.p[0] = en.x; e.p[1] = en.y; e.p[2] = en.z; e.p[3] = en.w;
        out[2 * (size_t)i] = finish_v(s, vpm);
        out[2 * (size_t)i + 1] = finish_v(e, vpm);
    }
    valid[i] = 1;
}

// ---------------------------------------------------------------- raster
struct LPTile {
    uint32_t x0, y0, x1, y1;   // inclusive corners (fragment.rs:188-216)
};

// Depth test, fragment shader, alpha multiply, blend and writes shared by
// both rasterisers (line.rs:79-106, point.rs:60-84); alpha < 0: no multiply.
template <int FS, int FMT, int BLEND>
__device__ __forceinline__ void lp_shade(const DrawParams& P, const sr_uniforms& U, const uint32_t* tex, void* color,
                                         float* depth, size_t idx, const float* pz, const float* k, double alpha) {
    const float z = pz[2];
    if (!(z < 0.0f)) return;
    if (P.has_depth) {
        const float dt = depth[idx];
        if (!(z >= dt)) return;
    }
    sr_v4 col = shade_fs<FS>(U, k, tex, P);
    if (FMT == SR_COLOR_RGBA32F) {
        float4* px = reinterpret_cast<float4*>(color) + idx;
        if (alpha >= 0.0) col.w = col.w * (float)alpha;           // AlphaMultiply for f32
        const float4 d = *px;
        const sr_v4 o = BLEND == BLEND_OVER ? sr_blend_over_f32(col, sr_make_v4(d.x, d.y, d.z, d.w)) : col;
        *px = make_float4(o.x, o.y, o.z, o.w);
    } else if (FMT == SR_COLOR_RGBA8) {
        uint32_t* px = reinterpret_cast<uint32_t*>(color) + idx;
        uint32_t src = sr_to_rgba8(col);
        if (alpha >= 0.0) {
            // AlphaMultiply for u8 (color/helper.rs:31-40) with the alpha
            // scalar converted by NumCast f64 -> u8 (truncation; 0 outside [0, 256))
            const uint8_t a8 = alpha >= 0.0 && alpha < 256.0 ? (uint8_t)alpha : 0;
            const uint8_t ch = (uint8_t)(src >> 24);
            const uint8_t na = sr_f32_to_u8((float)ch * ((float)a8 / 255.0f));
            src = (src & 0x00ffffffu) | ((uint32_t)na << 24);
        }
        *px = BLEND == BLEND_OVER ? sr_blend_over_rgba8(src, *px) : src;
    }
    if (P.has_depth) depth[idx] = z;
}

// f32::hypot as (float)sqrt((double)x*x + (double)y*y)
__device__ __forceinline__ float hypot_df(float x, float y) {
    const double dx = x, dy = y;
    return (float)__dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

// liang_barsky_iterative (geometry/line.rs:6-54)
__device__ __forceinline__ bool liang_barsky(float x1, float y1, float x2, float y2, float xmin, float ymin,
                                             float xmax, float ymax, float* o) {
    float t0 = 0.0f, t1 = 1.0f;
    const float dx = x2 - x1, dy = y2 - y1;
    for (int edge = 0; edge < 4; ++edge) {
        float p, q;
        switch (edge) {
        case 0: p = -dx; q = x1 - xmin; break;
        case 1: p = dx; q = xmax - x1; break;
        case 2: p = -dy; q = y1 - ymin; break;
        default: p = dy; q = ymax - y1; break;
        }
        if (p == 0.0f && q < 0.0f) return false;
        const float r = q / p;
        if (p < 0.0f) {
            if (r > t1) return false;
            else if (r > t0) t0 = r;
        } else if (p > 0.0f) {
            if (r < t0) return false;
            else if (r < t1) t1 = r;
        }
    }
    o[0] = x1 + t0 * dx; o[1] = y1 + t0 * dy;
    o[2] = x1 + t1 * dx; o[3] = y1 + t1 * dy;
    return true;
}

__device__ __forceinline__ bool lp_owner(const DrawParams& P, const LPTile& t, uint32_t px, uint32_t py) {
    return (px < t.x1 || t.x1 == P.W - 1) && (py < t.y1 || t.y1 == P.H - 1);
}

// The per-pixel closure of rasterize_line (rasterization/line.rs:54-109).
// Pixels outside the framebuffer are skipped (the reference indexes them
// unchecked).
template <int FS, int FMT, int BLEND>
__device__ __forceinline__ void line_fragment(const DrawParams& P, const sr_uniforms& U, const uint32_t* tex,
                                              void* color, float* depth, uint8_t* stencil, const LPTile& tile,
                                              const LPV& st, const LPV& en, float cx1, float cy1, float dlen,
                                              long long x, long long y, double alpha, unsigned long long& frags) {
    if (!(x >= 0 && y >= 0) || (unsigned long long)x >= P.W || (unsigned long long)y >= P.H) return;
    const size_t idx = (size_t)x + (size_t)y * P.W;
    const uint8_t s = P.has_stencil ? stencil[idx] : 0;
    if (!stencil_test(P.stencil_test, s, P.sref)) return;
    if (P.has_stencil) stencil[idx] = stencil_op(P.stencil_op, P.stencil_wrap, s, P.sref);
    const float xf = (float)x + 0.5f, yf = (float)y + 0.5f;
    const float t = hypot_df(cx1 - xf, cy1 - yf) / dlen;
    const float a[4] = {st.p.x, st.p.y, st.p.z, st.p.w}, b[4] = {en.p.x, en.p.y, en.p.z, en.p.w};
    float pz[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) pz[i] = (1.0f - t) * a[i] + t * b[i];
    if (pz[2] < 0.0f && lp_owner(P, tile, (uint32_t)x, (uint32_t)y)) ++frags;
    const float ka[12] = {st.k0.x, st.k0.y, st.k0.z, st.k0.w, st.k1.x, st.k1.y, st.k1.z, st.k1.w,
                          st.k2.x, st.k2.y, st.k2.z, st.k2.w};
    const float kb[12] = {en.k0.x, en.k0.y, en.k0.z, en.k0.w, en.k1.x, en.k1.y, en.k1.z, en.k1.w,
                          en.k2.x, en.k2.y, en.k2.z, en.k2.w};
    float k[12];
#pragma unroll
    for (int i = 0; i < 12; ++i) k[i] = (1.0f - t) * ka[i] + t * kb[i];
    lp_shade<FS, FMT, BLEND>(P, U, tex, color, depth, idx, pz, k, alpha);
}

__device__ __forceinline__ double fract_d(double v) { return v - trunc(v); }
__device__ __forceinline__ long long d2ll(double v) { return isnan(v) ? 0 : (long long)v; }

// rasterize_line (rasterization/line.rs:22-119): Liang-Barsky against the
// tile, then Bresenham (:125-151) or Xiaolin Wu (:159-239, f64).
template <int FS, int FMT, int BLEND>
__device__ void rasterize_line(const DrawParams& P, const sr_uniforms& U, const uint32_t* tex, void* color,
                               float* depth, uint8_t* stencil, const LPTile& tile, const LPV& st, const LPV& en,
                               const float* o, unsigned long long& frags) {
    const float x1 = o[0], y1 = o[1], x2 = o[2], y2 = o[3];
    const float dlen = hypot_df(x1 - x2, y1 - y2);
#define SR_PLOT(X, Y, A) line_fragment<FS, FMT, BLEND>(P, U, tex, color, depth, stencil, tile, st, en, x1, y1, dlen, \
                                                       (X), (Y), (A), frags)
    if (P.aa_lines) {
        double X0 = x1, Y0 = y1, X1 = x2, Y1 = y2;
        const bool steep = fabs(Y1 - Y0) > fabs(X1 - X0);
        if (steep) { double q = X0; X0 = Y0; Y0 = q; q = X1; X1 = Y1; Y1 = q; }
        if (X0 > X1) { double q = X0; X0 = X1; X1 = q; q = Y0; Y0 = Y1; Y1 = q; }
        const double dx = X1 - X0, dy = Y1 - Y0;
        const double gradient = dx < 0.0001 ? 1.0 : dy / dx;
        double xend = round(X0);
        double yend = Y0 + gradient * (xend - X0);
        double xgap = 1.0 - fract_d(X0 + 0.5);
        const double xpxl1 = xend, ypxl1 = trunc(yend);
        if (steep) {
            SR_PLOT(d2ll(ypxl1), d2ll(xpxl1), (1.0 - fract_d(yend)) * xgap);
            SR_PLOT(d2ll(ypxl1 + 1.0), d2ll(xpxl1), fract_d(yend) * xgap);
        } else {
            SR_PLOT(d2ll(xpxl1), d2ll(ypxl1), (1.0 - fract_d(yend)) * xgap);
            SR_PLOT(d2ll(xpxl1), d2ll(ypxl1 + 1.0), fract_d(yend) * xgap);
        }
        double intery = yend + gradient;
        xend = round(X1);
        yend = Y1 + gradient * (xend - X1);
        xgap = fract_d(X1 + 0.5);
        const double xpxl2 = xend, ypxl2 = trunc(yend);
        if (steep) {
            SR_PLOT(d2ll(ypxl2), d2ll(xpxl2), (1.0 - fract_d(yend)) * xgap);
            SR_PLOT(d2ll(ypxl2 + 1.0), d2ll(xpxl2), fract_d(yend) * xgap);
        } else {
            SR_PLOT(d2ll(xpxl2), d2ll(ypxl2), (1.0 - fract_d(yend)) * xgap);
            SR_PLOT(d2ll(xpxl2), d2ll(ypxl2 + 1.0), fract_d(yend) * xgap);
        }
        // the span between the end points (bounded by the tile's width)
        for (double x = xpxl1 + 1.0; x <= xpxl2 - 1.0; x += 1.0) {
            const double y = trunc(intery);
            if (steep) {
                SR_PLOT(d2ll(y), d2ll(x), 1.0 - fract_d(intery));
                SR_PLOT(d2ll(y + 1.0), d2ll(x), fract_d(intery));
            } else {
                SR_PLOT(d2ll(x), d2ll(y), 1.0 - fract_d(intery));
                SR_PLOT(d2ll(x), d2ll(y + 1.0), fract_d(intery));
            }
            intery += gradient;
        }
    } else {
        long long X0 = (long long)x1, Y0 = (long long)y1;
        const long long X1 = (long long)x2, Y1 = (long long)y2;
        const long long dx = X1 > X0 ? X1 - X0 : X0 - X1;
        const long long dy = -(Y1 > Y0 ? Y1 - Y0 : Y0 - Y1);
        const long long sx = X0 < X1 ? 1 : -1, sy = Y0 < Y1 ? 1 : -1;
        long long err = dx + dy;
        // at most dx - dy + 1 steps (the clipped segment lies in the tile)
        for (long long guard = 0; guard <= dx - dy; ++guard) {
            SR_PLOT(X0, Y0, 1.0);
            if (X0 == X1 && Y0 == Y1) break;
            const long long e2 = 2 * err;
            if (e2 >= dy) { err += dy; X0 += sx; }
            if (e2 <= dx) { err += dx; Y0 += sy; }
        }
    }
#undef SR_PLOT
}

// One warp per semantic tile of phase `phase` (tile (r, c) with
// c + kstep * r == phase); primitives in submission order.
template <int FS, int FMT, int BLEND>
__global__ void __launch_bounds__(32) raster_lp_kernel(DrawParams P, sr_uniforms U, uint32_t phase, uint32_t kstep,
                                                       const LPV* __restrict__ v, const uint8_t* __restrict__ valid,
                                                       uint32_t n_prims, uint32_t prim_n, const uint32_t* tex,
                                                       void* color, float* depth, uint8_t* stencil,
                                                       DeviceFlags* flags) {
    const int r_lo = (int)lp_phase_first_row(phase, P.ncols, kstep);
    const int r = r_lo + (int)blockIdx.x;
    const int c = (int)phase - (int)kstep * r;
    if (r >= (int)P.nrows || c < 0 || c >= (int)P.ncols) return;
    LPTile tile;
    tile.x0 = (uint32_t)c * P.tile_w;
    tile.x1 = min(((uint32_t)c + 1) * P.tile_w, P.W - 1);
    tile.y0 = (uint32_t)r * P.tile_h;
    tile.y1 = min(((uint32_t)r + 1) * P.tile_h, P.H - 1);
    const uint32_t lane = threadIdx.x;
    unsigned long long frags = 0;
    for (uint32_t base = 0; base < n_prims; base += 32) {
        const uint32_t i = base + lane;
        bool hit = false;
        float o[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (i < n_prims && valid[i]) {
            if (prim_n == 2) {
                const float4 a = v[2 * (size_t)i].p, b = v[2 * (size_t)i + 1].p;
                hit = liang_barsky(a.x, a.y, b.x, b.y, (float)tile.x0, (float)tile.y0, (float)tile.x1,
                                   (float)tile.y1, o);
                // a NaN clipped end point (a NaN or infinite vertex): the
                // reference's cast to i64 panics for Bresenham (line.rs:111-116)
                // and is undefined for Xiaolin Wu (`as i64` of NaN, line.rs:163,
                // before Rust 1.45); the line is skipped and the draw reports
                // SR_ENAN (plotting it at 0 from every tile would also race
                // between tiles of one phase)
                if (hit && (isnan(o[0]) || isnan(o[1]) || isnan(o[2]) || isnan(o[3]))) {
                    hit = false;
                    atomicAdd(&flags->nan_total, 1u);
                    atomicAdd(&flags->nan_bbox, 1u);
                }
            } else {
                const float4 a = v[i].p;
                hit = (float)tile.x0 <= a.x && a.x < (float)tile.x1 && (float)tile.y0 <= a.y && a.y < (float)tile.y1;
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, hit);
        while (m) {
            const int j = __ffs(m) - 1;
            m &= m - 1;
            if ((int)lane == j) {
                if (prim_n == 2) {
                    rasterize_line<FS, FMT, BLEND>(P, U, tex, color, depth, stencil, tile, v[2 * (size_t)i],
                                                   v[2 * (size_t)i + 1], o, frags);
                } else {
                    // rasterize_point (rasterization/point.rs:21-87)
                    const LPV& q = v[i];
                    const uint32_t px = (uint32_t)q.p.x, py = (uint32_t)q.p.y;
                    const size_t idx = (size_t)px + (size_t)py * P.W;
                    const uint8_t s = P.has_stencil ? stencil[idx] : 0;
                    if (stencil_test(P.stencil_test, s, P.sref)) {
                        if (P.has_stencil) stencil[idx] = stencil_op(P.stencil_op, P.stencil_wrap, s, P.sref);
                        const float pz[4] = {q.p.x, q.p.y, q.p.z, q.p.w};
                        if (q.p.z < 0.0f && lp_owner(P, tile, px, py)) ++frags;
                        const float k[12] = {q.k0.x, q.k0.y, q.k0.z, q.k0.w, q.k1.x, q.k1.y, q.k1.z, q.k1.w,
                                             q.k2.x, q.k2.y, q.k2.z, q.k2.w};
                        lp_shade<FS, FMT, BLEND>(P, U, tex, color, depth, idx, pz, k, -1.0);
                    }
                }
            }
            __syncwarp();
        }
    }
    for (int o2 = 16; o2 > 0; o2 >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o2);
    if (lane == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// ------------------------------------------------------------- launchers
void launch_lp_geometry(const DrawParams& P, const sr_uniforms& U, const sr_mesh* m, VertexStore vs, uint32_t prim_n,
                        uint32_t gs_mode, uint32_t gs, LPV* out, uint8_t* valid, DeviceFlags* flags,
                        cudaStream_t st) {
    const uint32_t n = (uint32_t)(m->n_indices / prim_n);
    if (n == 0) return;
    const dim3 block(128), grid((n + 127) / 128);
    const VpMatrix vpm = viewport_matrix(P.vp);
    if (gs_mode == SR_GS_NONE)
        lp_indexed_kernel<<<grid, block, 0, st>>>(n, prim_n, P.n_verts, m->indices, vs.scr4, vs.vary, out, valid, flags);
    else if (gs_mode == SR_GS_CLIP || gs == GS_CLIP)
        lp_clip_kernel<<<grid, block, 0, st>>>(n, prim_n, P.n_verts, vpm, m->indices, vs.clip4, vs.vary, out, valid,
                                               flags);
    else
        lp_normals_kernel<<<grid, block, 0, st>>>(n, prim_n, P.n_verts, gs == GS_FACE_NORMALS ? 1u : 0u, U, vpm,
                                                  m->indices, vs.clip4, vs.vary, out, valid, flags);
}

template <int FS, int FMT, int BLEND>
static void launch_lp_phases(const DrawParams& P, const sr_uniforms& U, const LPV* v, const uint8_t* valid,
                             uint32_t n_prims, uint32_t prim_n, const uint32_t* tex, void* color, float* depth,
                             uint8_t* stencil, DeviceFlags* flags, cudaStream_t st) {
    const uint32_t kstep = lp_phase_step(P.aa_lines && prim_n == 2, P.tile_w);
    const uint32_t phases = (P.ncols - 1) + kstep * (P.nrows - 1) + 1;
    for (uint32_t ph = 0; ph < phases; ++ph)
        raster_lp_kernel<FS, FMT, BLEND><<<P.nrows, 32, 0, st>>>(P, U, ph, kstep, v, valid, n_prims, prim_n, tex,
                                                                 color, depth, stencil, flags);
}

uint32_t launch_lp_raster(const DrawParams& P, const sr_uniforms& U, const LPV* v, const uint8_t* valid,
                          uint32_t n_prims, uint32_t prim_n, const uint32_t* tex, void* color, float* depth,
                          uint8_t* stencil, DeviceFlags* flags, cudaStream_t st) {
    if (P.ncols == 0 || P.nrows == 0 || n_prims == 0) return 0;
#define SR_LPB(FS, FMT) \
    if (P.blend == BLEND_OVER) launch_lp_phases<FS, FMT, BLEND_OVER>(P, U, v, valid, n_prims, prim_n, tex, color, depth, stencil, flags, st); \
    else launch_lp_phases<FS, FMT, BLEND_REPLACE>(P, U, v, valid, n_prims, prim_n, tex, color, depth, stencil, flags, st);
#define SR_LPF(FS) \
    if (P.color_format == SR_COLOR_RGBA8) { SR_LPB(FS, SR_COLOR_RGBA8) } \
    else if (P.color_format == SR_COLOR_RGBA32F) { SR_LPB(FS, SR_COLOR_RGBA32F) } \
    else { SR_LPB(FS, SR_COLOR_NONE) }
    switch (P.fs) {
    case FS_BLINN_PHONG_DIR: SR_LPF(FS_BLINN_PHONG_DIR) break;
    case FS_TEXTURED_BLINN_PHONG: SR_LPF(FS_TEXTURED_BLINN_PHONG) break;
    case FS_VERTEX_COLOR: SR_LPF(FS_VERTEX_COLOR) break;
    case FS_ACES_LIGHTS: SR_LPF(FS_ACES_LIGHTS) break;
    default: SR_LPF(FS_CONSTANT_COLOR) break;
    }
#undef SR_LPF
#undef SR_LPB
    return (P.ncols - 1) + 2 * (P.nrows - 1) + 1;
}

}  // namespace sr
