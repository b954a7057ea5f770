// sr_opaque.cuh — device code of the opaque raster path shared by the
// per-draw kernels (sr_opaque.cu) and the batched kernels (sr_batch.cu).
#pragma once
#include "sr_internal.cuh"
#include "sr_shade.cuh"

namespace sr {

constexpr int RG_THREADS = 256;
constexpr uint32_t TOUCH_LOG2 = 5;               // touched-block bitmap granularity: 32 x 32


__device__ __forceinline__ void mark_touched(uint32_t* bitmap, uint32_t blocks_x, uint32_t px, uint32_t py) {
    uint32_t b = (py >> TOUCH_LOG2) * blocks_x + (px >> TOUCH_LOG2);
    const uint32_t bit = 1u << (b & 31);
    // test first: blocks are shared by many primitives, and an atomic per
    // primitive on the same word would serialise in L2
    if (!(bitmap[b >> 5] & bit)) atomicOr(bitmap + (b >> 5), bit);
}

// high 32 bits of a 32 x 32-bit product
__host__ __device__ __forceinline__ uint32_t umulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}
// number of semantic tiles along one axis containing coordinate p (1 or 2)
__host__ __device__ __forceinline__ int seam_count(uint32_t p, uint32_t t, uint32_t m, uint32_t last) {
    return (p > 0 && p < last && (m == 0 || umulhi32(p, m) * t == p)) ? 2 : 1;
}
// mark the 32x32 blocks of a clamped bbox as touched
__device__ __forceinline__ void mark_rect(uint32_t* bitmap, uint32_t blocks_x, uint32_t x0, uint32_t y0, uint32_t x1,
                                          uint32_t y1) {
    for (uint32_t by = y0 >> TOUCH_LOG2; by <= (y1 >> TOUCH_LOG2); ++by)
        for (uint32_t bx = x0 >> TOUCH_LOG2; bx <= (x1 >> TOUCH_LOG2); ++bx) {
            const uint32_t b = by * blocks_x + bx, bit = 1u << (b & 31);
            if (!(bitmap[b >> 5] & bit)) atomicOr(bitmap + (b >> 5), bit);   // test first (see mark_touched)
        }
}

// The exact per-pixel sequence of rasterize_triangle (triangle.rs:104-126) for
// one (primitive, pixel) item: barycentrics in the reference's op order,
// inclusive coverage, z < 0, optional stencil gate.  Returns the item's 64-bit
// winner key, or 0 when the pixel yields no fragment (counted in `frags`).
// The target is given by its scalars (frame size, semantic tile size with
// its division magics, depth attachment, stencil gate).
//
// seams: bit 0 set when the primitive's bbox may contain a seam column, bit 1
// a seam row (seam_bits); otherwise that axis has one semantic tile.
__device__ __forceinline__ unsigned long long frag_key(uint32_t W, uint32_t H, uint32_t tile_w, uint32_t tile_h,
                                                       uint32_t mx, uint32_t my, uint32_t seams, bool has_depth,
                                                       float4 r0, float4 r1, float4 r2, uint32_t t, uint32_t px,
                                                       uint32_t py, uint32_t N, const uint8_t* __restrict__ stencil,
                                                       uint32_t gate_with_stencil, uint32_t stencil_test_id,
                                                       uint32_t sref, unsigned long long& frags) {
    const float x = (float)px + 0.5f, y = (float)py + 0.5f;
    const float dx = x - r1.x, dy = y - r1.y;
    // r2.w = det_sign(det): a certainly negative u or v rejects the pixel
    // without the divisions
    const float nu = r0.x * dx + r0.y * dy;
    if (r2.w * nu < -1.0e-18f) return 0ull;
    const float nv = r0.z * dx + r0.w * dy;
    if (r2.w * nv < -1.0e-18f) return 0ull;
    // w = (1-u)-v is certainly negative when s (det - nu - nv), evaluated in
    // f32, lies below -2^-21 (|det| + |nu| + |nv|): with U = nu/det, V = nv/det,
    // the two quotients and 1-u round by at most 2^-24 relative (plus 2^-150
    // absolute), so |det| ((1-u) - v) <= s (det - nu - nv) + 2^-24 (|det| +
    // 2|nu| + |nv|) + tiny, and the f32 evaluation of det - nu - nv errs by at
    // most 2^-24 (2|det| + 2|nu| + |nv|): the margin covers both with room to
    // spare, so (1-u) < v and w, the rounded difference, is negative.  An
    // infinite or NaN term makes the test false (no rejection).
    if (r2.w * ((r1.z - nu) - nv) < -0x1p-21f * (fabsf(r1.z) + fabsf(nu) + fabsf(nv))) return 0ull;
    const float u = nu / r1.z, v = nv / r1.z;
    const float w = 1.0f - u - v;
    if (u < 0.0f || v < 0.0f || w < 0.0f) return 0ull;
    const float z = (r1.w * u + r2.x * v) + r2.y * w;
    if (!(z < 0.0f)) return 0ull;
    if (gate_with_stencil && !stencil_test(stencil_test_id, __ldg(stencil + (size_t)py * W + px), sref)) return 0ull;
    const int kp = ((seams & 1u) ? seam_count(px, tile_w, mx, W - 1) : 1) *
                   ((seams & 2u) ? seam_count(py, tile_h, my, H - 1) : 1);
    ++frags;
    const uint32_t zk = has_depth ? zkey(z) : 0u;
    return ((unsigned long long)zk << 32) | (unsigned long long)((uint32_t)(kp - 1) * N + t + 1u);
}

// frag_key reduced into a per-pixel key buffer with a 64-bit atomicMax.
__device__ __forceinline__ void frag_emit(uint32_t W, uint32_t H, uint32_t tile_w, uint32_t tile_h, uint32_t mx,
                                          uint32_t my, uint32_t seams, bool has_depth, float4 r0, float4 r1, float4 r2,
                                          uint32_t t,
                                          uint32_t px, uint32_t py, uint32_t N, unsigned long long* __restrict__ gkeys,
                                          const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil,
                                          uint32_t stencil_test_id, uint32_t sref, unsigned long long& frags) {
    const unsigned long long k = frag_key(W, H, tile_w, tile_h, mx, my, seams, has_depth, r0, r1, r2, t, px, py, N,
                                          stencil, gate_with_stencil, stencil_test_id, sref, frags);
    if (k) atomicMax(gkeys + (size_t)py * W + px, k);
}

__device__ __forceinline__ void rg_fragment(const DrawParams& P, float4 r0, float4 r1, float4 r2, uint32_t t,
                                            uint32_t px, uint32_t py, uint32_t N,
                                            unsigned long long* __restrict__ gkeys, uint32_t* __restrict__ bitmap,
                                            const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil,
                                            uint32_t mx, uint32_t my, uint32_t seams, unsigned long long& frags) {
    frag_emit(P.W, P.H, P.tile_w, P.tile_h, mx, my, seams, P.has_depth != 0, r0, r1, r2, t, px, py, N, gkeys,
              stencil, gate_with_stencil, P.stencil_test, P.sref, frags);
}

// Whether the clamped bbox [x0, x1] x [y0, y1] contains a seam column (bit 0:
// 0 < p < W-1 with p a multiple of the tile width) or a seam row (bit 1): the
// largest multiple of t up to hi, floor(hi / t) t (hi < 2^15, by the tile
// size's division magic), is at least lo.
__device__ __forceinline__ uint32_t seam_bits(uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                                              const DrawParams& P) {
    uint32_t s = 0;
    {
        const uint32_t lo = max(x0, 1u), hi = min(x1, P.W - 2);
        if (lo <= hi && (P.magic_w == 0 || umulhi32(hi, P.magic_w) * P.tile_w >= lo)) s |= 1u;
    }
    {
        const uint32_t lo = max(y0, 1u), hi = min(y1, P.H - 2);
        if (lo <= hi && (P.magic_h == 0 || umulhi32(hi, P.magic_h) * P.tile_h >= lo)) s |= 2u;
    }
    return s;
}

constexpr uint32_t RG_BIG = 2048;   // bbox pixels above which a primitive goes to the block-cooperative pass

// Extension fragments of one unsafe primitive t (see ext_direct_kernel): the
// warp's lanes stride over the semantic tiles, each finding its tile's
// clamped segment (triangle.rs:66-78) and testing it with the sound sign
// test; the segments the test does not clear are then evaluated one after
// another with the lanes spread over the segment's pixels (a segment is one
// pixel wide or high, up to a tile long).  `mark(px, py)` records the pixel's
// 32x32 block as touched.
template <class Mark>
__device__ __forceinline__ void ext_prim_m(const DrawParams& P, uint32_t t, uint32_t N,
                                           const float4* __restrict__ setup, unsigned long long* __restrict__ gkeys,
                                           const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil,
                                           uint32_t lane, unsigned long long& frags, Mark mark) {
    const uint32_t ntiles = P.ncols * P.nrows;
    const float4* r = setup + 4 * (size_t)t;
    const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
    const int ix0 = __float_as_int(r3.x), iy0 = __float_as_int(r3.y);
    const int ix1 = __float_as_int(r3.z), iy1 = __float_as_int(r3.w);
    for (uint32_t tb = 0; tb < ntiles; tb += 32) {
        const uint32_t ti = tb + lane;
        uint32_t cx0 = 0, cx1 = 0, cy0 = 0, cy1 = 0;
        bool open = false;
        if (ti < ntiles) {
            const uint32_t C = ti % P.ncols, R = ti / P.ncols;
            const uint32_t lx = C * P.tile_w, hx = min((C + 1) * P.tile_w, P.W - 1);
            const uint32_t ly = R * P.tile_h, hy = min((R + 1) * P.tile_h, P.H - 1);
            if (!(ix1 >= (int)lx && ix0 <= (int)hx && iy1 >= (int)ly && iy0 <= (int)hy)) {
                cx0 = ix0 < (int)lx ? lx : (ix0 > (int)hx ? hx : (uint32_t)ix0);
                cx1 = ix1 < (int)lx ? lx : (ix1 > (int)hx ? hx : (uint32_t)ix1);
                cy0 = iy0 < (int)ly ? ly : (iy0 > (int)hy ? hy : (uint32_t)iy0);
                cy1 = iy1 < (int)ly ? ly : (iy1 > (int)hy ? hy : (uint32_t)iy1);
                open = !segment_cleared(r0, r1, cx0, cy0, cx1, cy1);
            }
        }
        uint32_t todo = __ballot_sync(0xffffffffu, open);
        while (todo) {
            const uint32_t src = __ffs(todo) - 1;
            todo &= todo - 1;
            const uint32_t sx0 = __shfl_sync(0xffffffffu, cx0, src), sx1 = __shfl_sync(0xffffffffu, cx1, src);
            const uint32_t sy0 = __shfl_sync(0xffffffffu, cy0, src), sy1 = __shfl_sync(0xffffffffu, cy1, src);
            const uint32_t sti = tb + src, C = sti % P.ncols, R = sti / P.ncols;
            const uint32_t sw = sx1 - sx0 + 1, npx = sw * (sy1 - sy0 + 1);
            for (uint32_t i = lane; i < npx; i += 32) {
                const uint32_t px = sx0 + i % sw, py = sy0 + i / sw;
                const float x = (float)px + 0.5f, y = (float)py + 0.5f;
                const float dx = x - r1.x, dy = y - r1.y;
                const float u = (r0.x * dx + r0.y * dy) / r1.z;
                const float v = (r0.z * dx + r0.w * dy) / r1.z;
                const float w = 1.0f - u - v;
                if (u < 0.0f || v < 0.0f || w < 0.0f) continue;
                const float z = (r1.w * u + r2.x * v) + r2.y * w;
                if (!(z < 0.0f)) continue;
                const size_t gi = (size_t)py * P.W + px;
                if (gate_with_stencil && !stencil_test(P.stencil_test, __ldg(stencil + gi), P.sref)) continue;
                // rank of tile (R, C) among the tiles containing the pixel
                TileSpan cs = tiles_of(px, P.tile_w, P.ncols, P.W - 1);
                TileSpan rs = tiles_of(py, P.tile_h, P.nrows, P.H - 1);
                const int rank = (int)(R - rs.first) * cs.count + (int)(C - cs.first);
                if (rank == cs.count * rs.count - 1) ++frags;
                const uint32_t zk = P.has_depth ? zkey(z) : 0u;
                atomicMax(gkeys + gi, ((unsigned long long)zk << 32) |
                                          (unsigned long long)((uint32_t)rank * N + t + 1u));
                mark(px, py);
            }
        }
    }
}

// Extension fragments of one unsafe primitive t whose computed coverage is
// bounded by `region` (the inflated triangle's rectangle, see inflated_region
// in sr_setup.cuh): only pixel centres inside it can be covered, so the
// candidates are its pixels outside the bbox (a ring at most a pixel or two
// wide), each evaluated for every semantic tile whose clamped bbox
// (triangle.rs:66-78) holds it.  The warp's lanes stride over the ring.
template <class Mark>
__device__ __forceinline__ void ext_prim_ring(const DrawParams& P, uint32_t t, uint32_t N, float4 region,
                                              const float4* __restrict__ setup, unsigned long long* __restrict__ gkeys,
                                              const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil,
                                              uint32_t lane, unsigned long long& frags, Mark mark) {
    const float4* r = setup + 4 * (size_t)t;
    const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
    const int ix0 = __float_as_int(r3.x), iy0 = __float_as_int(r3.y);
    const int ix1 = __float_as_int(r3.z), iy1 = __float_as_int(r3.w);
    // pixel centres p + 0.5 inside [region.x, region.z] x [region.y, region.w]
    // (the region is only computed for coordinates below 1e6 in magnitude)
    const int cx0 = max((int)ceilf(region.x - 0.5f), 0), cx1 = min((int)floorf(region.z - 0.5f), (int)P.W - 1);
    const int cy0 = max((int)ceilf(region.y - 0.5f), 0), cy1 = min((int)floorf(region.w - 0.5f), (int)P.H - 1);
    if (cx0 > cx1 || cy0 > cy1) return;
    // the ring: strips left and right of the bbox (all candidate rows), then
    // above and below it (the bbox's columns)
    const int mx0 = max(ix0, cx0), mx1 = min(ix1, cx1);
    int rx[4][2], ry[4][2];
    rx[0][0] = cx0; rx[0][1] = min(ix0 - 1, cx1); ry[0][0] = cy0; ry[0][1] = cy1;
    rx[1][0] = max(ix1 + 1, cx0); rx[1][1] = cx1; ry[1][0] = cy0; ry[1][1] = cy1;
    rx[2][0] = mx0; rx[2][1] = mx1; ry[2][0] = cy0; ry[2][1] = min(iy0 - 1, cy1);
    rx[3][0] = mx0; rx[3][1] = mx1; ry[3][0] = max(iy1 + 1, cy0); ry[3][1] = cy1;
    uint32_t cnt[4], total = 0;
SR_UNROLL
    for (int k = 0; k < 4; ++k) {
        cnt[k] = (rx[k][0] <= rx[k][1] && ry[k][0] <= ry[k][1])
                     ? (uint32_t)(rx[k][1] - rx[k][0] + 1) * (uint32_t)(ry[k][1] - ry[k][0] + 1)
                     : 0u;
        total += cnt[k];
    }
    for (uint32_t i = lane; i < total; i += 32) {
        uint32_t j = i;
        int k = 0;
        while (j >= cnt[k]) { j -= cnt[k]; ++k; }
        const uint32_t w = (uint32_t)(rx[k][1] - rx[k][0] + 1);
        const uint32_t px = (uint32_t)rx[k][0] + j % w, py = (uint32_t)ry[k][0] + j / w;
        const TileSpan cs = tiles_of(px, P.tile_w, P.ncols, P.W - 1);
        const TileSpan rs = tiles_of(py, P.tile_h, P.nrows, P.H - 1);
        bool evaluated = false;
        float z = 0.0f;
        for (int a = 0; a < rs.count; ++a) {
            for (int c = 0; c < cs.count; ++c) {
                const uint32_t R = (uint32_t)(rs.first + a), C = (uint32_t)(cs.first + c);
                if (!clamp_axis(ix0, ix1, px, C, P.tile_w, P.W - 1) || !clamp_axis(iy0, iy1, py, R, P.tile_h, P.H - 1))
                    continue;
                if (!evaluated) {   // the same f32 values in every tile pass
                    evaluated = true;
                    const float x = (float)px + 0.5f, y = (float)py + 0.5f;
                    const float dx = x - r1.x, dy = y - r1.y;
                    const float u = (r0.x * dx + r0.y * dy) / r1.z;
                    const float v = (r0.z * dx + r0.w * dy) / r1.z;
                    const float ww = 1.0f - u - v;
                    if (u < 0.0f || v < 0.0f || ww < 0.0f) { a = rs.count; break; }
                    z = (r1.w * u + r2.x * v) + r2.y * ww;
                    if (!(z < 0.0f)) { a = rs.count; break; }
                    if (gate_with_stencil && !stencil_test(P.stencil_test, __ldg(stencil + (size_t)py * P.W + px), P.sref)) {
                        a = rs.count;
                        break;
                    }
                }
                const int rank = a * cs.count + c;
                if (rank == cs.count * rs.count - 1) ++frags;
                const uint32_t zk = P.has_depth ? zkey(z) : 0u;
                atomicMax(gkeys + (size_t)py * P.W + px,
                          ((unsigned long long)zk << 32) | (unsigned long long)((uint32_t)rank * N + t + 1u));
                mark(px, py);
            }
        }
    }
}

__device__ __forceinline__ void ext_prim(const DrawParams& P, uint32_t t, uint32_t N, const float4* __restrict__ setup,
                                         unsigned long long* __restrict__ gkeys, uint32_t* __restrict__ bitmap,
                                         const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil,
                                         uint32_t lane, unsigned long long& frags) {
    const uint32_t blocks_x = (P.W + 31) >> 5;
    ext_prim_m(P, t, N, setup, gkeys, stencil, gate_with_stencil, lane, frags,
               [=](uint32_t px, uint32_t py) { mark_touched(bitmap, blocks_x, px, py); });
}

// Resolve of one pixel whose winning key k is non-zero: the key against the
// depth the draw started from (d0, read by the caller; ignored without a
// depth attachment), the winner's barycentrics recomputed, its varyings
// interpolated and shaded, colour and depth written.  Returns false when the
// key loses (the pixel keeps its values).
template <int FS, int FMT>
__device__ __forceinline__ bool resolve_pixel(const DrawParams& P, const sr_uniforms& U, uint32_t px, uint32_t py,
                                              unsigned long long k, float d0, uint32_t N,
                                              const float4* __restrict__ setup, const uint32_t* __restrict__ vidx,
                                              const float* __restrict__ vary, const uint32_t* __restrict__ tex,
                                              void* __restrict__ color, float* __restrict__ depth,
                                              const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil) {
    const size_t gi = (size_t)py * P.W + px;
    if (P.has_depth && (isnan(d0) || (uint32_t)(k >> 32) < zkey(d0))) return false;
    if (gate_with_stencil && !stencil_test(P.stencil_test, stencil[gi], P.sref)) return false;
    // the key's low word is pass * N + t + 1 with pass < 4 (a pixel lies in
    // at most four semantic tiles)
    uint32_t t = (uint32_t)(k & 0xffffffffull) - 1u;
#pragma unroll
    for (int pass = 0; pass < 3; ++pass) t = t >= N ? t - N : t;
    const float4* r = setup + 4 * (size_t)t;
    const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2);
    const float x = (float)px + 0.5f, y = (float)py + 0.5f;
    const float dx = x - r1.x, dy = y - r1.y;
    const float u = (r0.x * dx + r0.y * dy) / r1.z;
    const float v = (r0.z * dx + r0.w * dy) / r1.z;
    const float w = 1.0f - u - v;
    const float z = (r1.w * u + r2.x * v) + r2.y * w;
    constexpr int NK = FsTraits<FS>::NK;
    float kv[12];
    if (NK > 0) {
        const uint32_t a = __ldg(vidx + 3 * (size_t)t), bq = __ldg(vidx + 3 * (size_t)t + 1),
                       c = __ldg(vidx + 3 * (size_t)t + 2);
        interp_varyings<NK>(vary, a, bq, c, u, v, w, kv);
    }
    if (FMT == SR_COLOR_RGBA32F) {
        const sr_v4 col = shade_fs<FS>(U, kv, tex, P);
        reinterpret_cast<float4*>(color)[gi] = make_float4(col.x, col.y, col.z, col.w);
    } else if (FMT == SR_COLOR_RGBA8) {
        reinterpret_cast<uint32_t*>(color)[gi] = shade_fs_rgba8<FS>(U, kv, tex, P);
    }
    if (P.has_depth) depth[gi] = z;
    return true;
}

// Resolve of one pixel from its winner's low key word (pass * N + primitive
// + 1, non-zero): the winner's barycentrics and z recomputed -- the same
// values its fragment had -- then z against the depth the draw started from
// (d0; ignored without a depth attachment), the stencil gate, varyings,
// shading, colour and depth written.  Returns false when the winner loses.
template <int FS, int FMT>
__device__ __forceinline__ bool resolve_winner(const DrawParams& P, const sr_uniforms& U, uint32_t px, uint32_t py,
                                               uint32_t id, float d0, uint32_t N, const float4* __restrict__ setup,
                                               const uint32_t* __restrict__ vidx, const float* __restrict__ vary,
                                               const uint32_t* __restrict__ tex, void* __restrict__ color,
                                               float* __restrict__ depth, const uint8_t* __restrict__ stencil,
                                               uint32_t gate_with_stencil) {
    const size_t gi = (size_t)py * P.W + px;
    uint32_t t = id - 1u;
#pragma unroll
    for (int pass = 0; pass < 3; ++pass) t = t >= N ? t - N : t;
    const float4* r = setup + 4 * (size_t)t;
    const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2);
    const float x = (float)px + 0.5f, y = (float)py + 0.5f;
    const float dx = x - r1.x, dy = y - r1.y;
    const float u = (r0.x * dx + r0.y * dy) / r1.z;
    const float v = (r0.z * dx + r0.w * dy) / r1.z;
    const float w = 1.0f - u - v;
    const float z = (r1.w * u + r2.x * v) + r2.y * w;
    if (P.has_depth && (isnan(d0) || zkey(z) < zkey(d0))) return false;
    if (gate_with_stencil && !stencil_test(P.stencil_test, stencil[gi], P.sref)) return false;
    constexpr int NK = FsTraits<FS>::NK;
    float kv[12];
    if (NK > 0) {
        const uint32_t a = __ldg(vidx + 3 * (size_t)t), bq = __ldg(vidx + 3 * (size_t)t + 1),
                       c = __ldg(vidx + 3 * (size_t)t + 2);
        interp_varyings<NK>(vary, a, bq, c, u, v, w, kv);
    }
    if (FMT == SR_COLOR_RGBA32F) {
        const sr_v4 col = shade_fs<FS>(U, kv, tex, P);
        reinterpret_cast<float4*>(color)[gi] = make_float4(col.x, col.y, col.z, col.w);
    } else if (FMT == SR_COLOR_RGBA8) {
        reinterpret_cast<uint32_t*>(color)[gi] = shade_fs_rgba8<FS>(U, kv, tex, P);
    }
    if (P.has_depth) depth[gi] = z;
    return true;
}

// Resolve of one touched 32x32 block b: each pixel's winning key against the
// depth the draw started from, barycentrics of the winner recomputed, its
// varyings interpolated and shaded, colour and depth written once; the keys
// and the block's bitmap bit are reset for the next draw.  With `clear_first`
// the draw follows a clear of its target that has not been written (the
// batched path defers it): the start depth is the cleared f32::MIN and every
// pixel without a winner receives the clear colour and depth here.
template <int FS, int FMT>
__device__ __forceinline__ void resolve_block(const DrawParams& P, const sr_uniforms& U, uint32_t b, uint32_t N,
                                              const float4* __restrict__ setup, const uint32_t* __restrict__ vidx,
                                              const float* __restrict__ vary, const uint32_t* __restrict__ tex,
                                              void* __restrict__ color, float* __restrict__ depth,
                                              const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil,
                                              unsigned long long* __restrict__ gkeys, uint32_t* __restrict__ bitmap,
                                              bool clear_first = false, uint4 clear_color = uint4{}) {
    const uint32_t blocks_x = (P.W + 31) >> 5;
    const uint32_t X0 = (b % blocks_x) << 5, Y0 = (b / blocks_x) << 5;
    const uint32_t bw = min(32u, P.W - X0), bh = min(32u, P.H - Y0);
    for (uint32_t i = threadIdx.x; i < 1024; i += blockDim.x) {
        const uint32_t lx = i & 31, ly = i >> 5;
        if (lx >= bw || ly >= bh) continue;
        const uint32_t px = X0 + lx, py = Y0 + ly;
        const size_t gi = (size_t)py * P.W + px;
        const unsigned long long k = gkeys[gi];
        bool win = false;
        if (k != 0) {
            gkeys[gi] = 0;
            const float d0 = P.has_depth ? (clear_first ? F32_LOWEST : depth[gi]) : 0.0f;
            win = resolve_pixel<FS, FMT>(P, U, px, py, k, d0, N, setup, vidx, vary, tex, color, depth, stencil,
                                         gate_with_stencil);
        }
        if (!win && clear_first) {
            if (FMT == SR_COLOR_RGBA32F) reinterpret_cast<uint4*>(color)[gi] = clear_color;
            else if (FMT == SR_COLOR_RGBA8) reinterpret_cast<uint32_t*>(color)[gi] = clear_color.x;
            if (P.has_depth) depth[gi] = F32_LOWEST;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) atomicAnd(bitmap + (b >> 5), ~(1u << (b & 31)));
}

}  // namespace sr
