// sr_setup.cuh — per-primitive setup helpers shared by the per-draw and the
// batched setup kernels (stages/rasterization/triangle.rs:48-78).
#pragma once
#include "sr_internal.cuh"

namespace sr {

constexpr uint32_t RECT_EMPTY = 0xffffffffu;   // binrect of a primitive with no regular bins

// Setup record, 4 x float4 per raster primitive:
//   r0 = (y2-y3, x3-x2, y3-y1, x1-x3)   edge coefficients of the numerators
//   r1 = (x3, y3, det, z1)
//   r2 = (z2, z3, flags, s)             s = det_sign(det)
//   r3 = clamped-to-frame bbox as ints (x0, y0, x1, y1)
// s is +1 or -1 for 0 < |det| < 1e18 and 0 otherwise: s * n < -1e-18 then
// proves that the quotient n / det rounds to a negative non-zero value
// (|n / det| > 1e-36 cannot underflow), so such a pixel is outside that edge.
__device__ __forceinline__ float det_sign(float det) {
    return (det > 0.0f && det < 1.0e18f) ? 1.0f : ((det < 0.0f && det > -1.0e18f) ? -1.0f : 0.0f);
}

// ------------------------------------------------------- extension pass
// An unsafe primitive can produce fragments outside its bbox, but only at
// the pixels where the reference evaluates it there: the projection of its
// bbox onto each semantic tile it does not overlap (a column segment, a row
// segment or a corner pixel on that tile's edge).  For each such segment a
// sound sign test clears the whole segment when one of u, v, w is certainly
// negative on it; remaining pixels are evaluated exactly (the reference's
// expressions), and the primitive is added to the bin of every pixel that
// yields a fragment, unless that bin already lists it.
//
// Sign test: the reference's numerator n_u(P) differs from the exact edge
// function N_u(P) by at most gamma_4 * S_u(P), S_u = |y2-y3||x-x3| + |x3-x2||y-y3|
// (convex on the segment, so its maximum is at an end point).  N_u is affine,
// so s*n_u(end) + 2 gamma_4 max S_u < 0 at both ends (s = sign of the computed
// det) makes u < 0 on the whole segment; v likewise.  For w = (1-u)-v the
// quantity det - N_u - N_v is affine and w < 0 follows when it is negative
// beyond the numerator errors plus 8 eps |det| (the roundings of the two
// quotients and two subtractions while u, v lie in [0, 2]; outside that range
// u < 0, v < 0 or w < 0 holds anyway).
__device__ __forceinline__ uint32_t clampu(int v, uint32_t lo, uint32_t hi) {
    return v < (int)lo ? lo : (v > (int)hi ? hi : (uint32_t)v);
}

// The extension bins of unsafe primitive t (one warp; lane strides over the
// semantic tiles): for every tile its bbox misses, the clamped tile-edge
// segment (triangle.rs:66-78) is skipped when the sound sign test clears it,
// otherwise its pixels are evaluated exactly and every bin holding a
// fragment outside the regular bin rectangle is reported through emit(bin)
// (consecutive repeats of a bin within a segment collapse).
template <class Emit>
__device__ __forceinline__ void ext_bins(const DrawParams& P, const float4* __restrict__ setup, uint2 br, uint32_t t,
                                         uint32_t lane, Emit emit) {
    const uint32_t ntiles = P.ncols * P.nrows;
    const float4* r = setup + 4 * (size_t)t;
    const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
    const int ix0 = __float_as_int(r3.x), iy0 = __float_as_int(r3.y);
    const int ix1 = __float_as_int(r3.z), iy1 = __float_as_int(r3.w);
    const bool has_rect = br.x != RECT_EMPTY;
    const uint32_t bx0 = br.x & 0xffffu, by0 = br.x >> 16, bx1 = br.y & 0xffffu, by1 = br.y >> 16;
    for (uint32_t ti = lane; ti < ntiles; ti += 32) {
        const uint32_t C = ti % P.ncols, R = ti / P.ncols;
        const uint32_t lx = C * P.tile_w, hx = min((C + 1) * P.tile_w, P.W - 1);
        const uint32_t ly = R * P.tile_h, hy = min((R + 1) * P.tile_h, P.H - 1);
        const bool ox = ix1 >= (int)lx && ix0 <= (int)hx;
        const bool oy = iy1 >= (int)ly && iy0 <= (int)hy;
        if (ox && oy) continue;   // bbox meets the tile: those pixels lie in the bbox bins
        const uint32_t cx0 = clampu(ix0, lx, hx), cx1 = clampu(ix1, lx, hx);
        const uint32_t cy0 = clampu(iy0, ly, hy), cy1 = clampu(iy1, ly, hy);
        if (segment_cleared(r0, r1, cx0, cy0, cx1, cy1)) continue;
        uint32_t last_b = 0xffffffffu;
        for (uint32_t py = cy0; py <= cy1; ++py) {
            for (uint32_t px = cx0; px <= cx1; ++px) {
                const float x = (float)px + 0.5f, y = (float)py + 0.5f;
                const float dx = x - r1.x, dy = y - r1.y;
                const float u = (r0.x * dx + r0.y * dy) / r1.z;
                const float v = (r0.z * dx + r0.w * dy) / r1.z;
                const float w = 1.0f - u - v;
                if (u < 0.0f || v < 0.0f || w < 0.0f) continue;
                const float z = (r1.w * u + r2.x * v) + r2.y * w;
                if (!(z < 0.0f)) continue;
                const uint32_t bxx = px >> P.bin_w_log2, byy = py >> P.bin_h_log2;
                if (has_rect && bxx >= bx0 && bxx <= bx1 && byy >= by0 && byy <= by1) continue;
                const uint32_t b = byy * P.bins_x + bxx;
                if (b == last_b) continue;
                last_b = b;
                emit(b);
            }
        }
    }
}

__device__ __forceinline__ void tri_slots(uint32_t t, const uint32_t* __restrict__ vidx, uint32_t& a, uint32_t& b,
                                          uint32_t& c) {
    a = __ldg(vidx + 3 * (size_t)t);
    b = __ldg(vidx + 3 * (size_t)t + 1);
    c = __ldg(vidx + 3 * (size_t)t + 2);
}

// Conservative bound of the pixel centres whose computed coverage
// !(u<0 || v<0 || w<0) can hold (the inflated triangle of sr_setup.cu): true when no pixel centre
// outside the integer bbox [ix0, ix1] x [iy0, iy1] can be covered.  `region`, when given,
// receives the inflated triangle's rectangle (x0, y0, x1, y1): every pixel centre of the
// frame whose computed coverage holds lies inside it; all NaN when no bound is computed.
__host__ __device__ __forceinline__ bool inflated_region(float x1, float y1, float x2, float y2, float x3, float y3,
                                                         float det, uint32_t W, uint32_t H, int ix0, int iy0, int ix1,
                                                         int iy1, float4* region = nullptr) {
    if (region) *region = make_float4(NAN, NAN, NAN, NAN);
    const float BIG = 1.0e6f;
    if (!(fabsf(x1) < BIG && fabsf(x2) < BIG && fabsf(x3) < BIG && fabsf(y1) < BIG && fabsf(y2) < BIG &&
          fabsf(y3) < BIG))
        return false;
    float a = y2 - y3, b = x3 - x2, c = y3 - y1, d = x1 - x3;
    float Rx = fmaxf(fabsf(0.5f - x3), fabsf((float)W - x3));
    float Ry = fmaxf(fabsf(0.5f - y3), fabsf((float)H - y3));
    // g >= 2 * gamma_4 (gamma_4 = 4u/(1-4u), u = 2^-24): absolute rounding of
    // the two-product numerators and the determinant, with slack for the
    // float evaluation of these bounds themselves
    const float g = 5.0e-7f;
    const float eps = 6.0e-8f;
    float Su = fabsf(a) * Rx + fabsf(b) * Ry;
    float Sv = fabsf(c) * Rx + fabsf(d) * Ry;
    float SD = fabsf(a * d) + fabsf(b * c);
    float absD = fabsf(det);
    float Dlo = absD - g * SD * 2.0f;
    if (!(Dlo > 1.0e-20f) || !(absD > 4.0f * g * SD)) return false;
    float tu = (g * Su + 1.0e-30f) / Dlo;
    float tv = (g * Sv + 1.0e-30f) / Dlo;
    float tw = 2.0f * (g * SD / Dlo + (g * (Su + Sv)) / Dlo + 16.0f * eps);
    if (!(tu < 1.0f && tv < 1.0f && tw < 1.0f)) return false;
    // vertices of {l_u >= -tu, l_v >= -tv, l_w >= -tw}
    float v1x = x1 + tv * (x1 - x2) + tw * (x1 - x3), v1y = y1 + tv * (y1 - y2) + tw * (y1 - y3);
    float v2x = x2 + tu * (x2 - x1) + tw * (x2 - x3), v2y = y2 + tu * (y2 - y1) + tw * (y2 - y3);
    float v3x = x3 + tu * (x3 - x1) + tv * (x3 - x2), v3y = y3 + tu * (y3 - y1) + tv * (y3 - y2);
    float slack = 1.0e-3f + 4.0e-6f * (fabsf(x1) + fabsf(x2) + fabsf(x3) + fabsf(y1) + fabsf(y2) + fabsf(y3));
    float fx0 = fminf(fminf(v1x, v2x), v3x) - slack, fx1 = fmaxf(fmaxf(v1x, v2x), v3x) + slack;
    float fy0 = fminf(fminf(v1y, v2y), v3y) - slack, fy1 = fmaxf(fmaxf(v1y, v2y), v3y) + slack;
    if (region) *region = make_float4(fx0, fy0, fx1, fy1);
    // a side only constrains where the frame has pixel centres beyond it
    // (ix0 etc. are clamped to [-1, W] / [-1, H])
    bool ok_l = ix0 <= 0 || fx0 > (float)ix0 - 0.5f;
    bool ok_r = ix1 >= (int)W - 1 || fx1 < (float)ix1 + 1.5f;
    bool ok_t = iy0 <= 0 || fy0 > (float)iy0 - 0.5f;
    bool ok_b = iy1 >= (int)H - 1 || fy1 < (float)iy1 + 1.5f;
    return ok_l && ok_r && ok_t && ok_b;
}

}  // namespace sr
