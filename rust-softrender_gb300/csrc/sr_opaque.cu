// sr_opaque.cu — the opaque draw path (blend `()`, shaders that never discard).
//
// For such draws the reference's per-pixel sequence (triangle.rs:80-155:
// coverage, z < 0, `z >= depth` then shade and overwrite) leaves each pixel
// with the shade of the LAST fragment in submission order among those whose z
// equals the largest z, its depth being that z (ties pass `>=`).  Seam pixels
// are processed once per semantic tile containing them, in row-major tile
// order; for a primitive covering the pixel inside its bbox every pass sees
// the same fragment, and outside the bbox only the clamped tile-edge events
// of the tile being processed occur.  So the winner is the maximum over all
// fragments of the 64-bit key
//       zkey(z) << 32  |  pass * N + primitive + 1
// where zkey orders floats, pass is the rank of the tile among those
// containing the pixel and N the number of raster primitives.  The maximum is
// order independent, so fragments are generated fully in parallel and reduced
// with fire-and-forget 64-bit atomicMax into a per-pixel key buffer; a resolve
// pass then shades each pixel's winner once (deferred shading) and compares
// with the depth the draw started from.
//
// Work distribution: each warp takes 32 consecutive primitives and spreads
// their bbox pixels over its lanes; primitives with large bboxes are handled
// by whole blocks in a second pass.
#include "sr_internal.cuh"
#include "sr_scan.cuh"
#include "sr_shade.cuh"

namespace sr {


constexpr int RG_THREADS = 256;
constexpr uint32_t TOUCH_LOG2 = 5;               // touched-block bitmap granularity: 32 x 32

__device__ __forceinline__ bool surely_negative(float n, float det) {
    return (n * det < 0.0f) && fabsf(n) > 1.0e-18f && fabsf(det) < 1.0e18f;
}

__device__ __forceinline__ void mark_touched(uint32_t* bitmap, uint32_t blocks_x, uint32_t px, uint32_t py) {
    uint32_t b = (py >> TOUCH_LOG2) * blocks_x + (px >> TOUCH_LOG2);
    uint32_t bit = 1u << (b & 31);
    if (!(bitmap[b >> 5] & bit)) atomicOr(bitmap + (b >> 5), bit);   // a stale read only costs an extra atomic
}

// ceil(2^32 / t): floor(p / t) == __umulhi(p, m) for p, t < 2^16
__device__ __forceinline__ uint32_t div_magic(uint32_t t) { return (uint32_t)((0x100000000ull + t - 1) / t); }
// number of semantic tiles along one axis containing coordinate p (1 or 2)
__device__ __forceinline__ int seam_count(uint32_t p, uint32_t t, uint32_t m, uint32_t last) {
    return (p > 0 && p < last && __umulhi(p, m) * t == p) ? 2 : 1;
}
// mark the 32x32 blocks of a clamped bbox as touched
__device__ __forceinline__ void mark_rect(uint32_t* bitmap, uint32_t blocks_x, uint32_t x0, uint32_t y0, uint32_t x1,
                                          uint32_t y1) {
    for (uint32_t by = y0 >> TOUCH_LOG2; by <= (y1 >> TOUCH_LOG2); ++by)
        for (uint32_t bx = x0 >> TOUCH_LOG2; bx <= (x1 >> TOUCH_LOG2); ++bx) {
            const uint32_t b = by * blocks_x + bx, bit = 1u << (b & 31);
            if (!(bitmap[b >> 5] & bit)) atomicOr(bitmap + (b >> 5), bit);
        }
}

// Exact test of one (primitive, pixel) item; emits the fragment key.
__device__ __forceinline__ void rg_fragment(const DrawParams& P, float4 r0, float4 r1, float4 r2, uint32_t t,
                                            uint32_t px, uint32_t py, uint32_t N,
                                            unsigned long long* __restrict__ gkeys, uint32_t* __restrict__ bitmap,
                                            const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil,
                                            uint32_t mx, uint32_t my, unsigned long long& frags) {
    const float x = (float)px + 0.5f, y = (float)py + 0.5f;
    const float dx = x - r1.x, dy = y - r1.y;
    const float nu = r0.x * dx + r0.y * dy;
    if (surely_negative(nu, r1.z)) return;
    const float nv = r0.z * dx + r0.w * dy;
    if (surely_negative(nv, r1.z)) return;
    const float u = nu / r1.z, v = nv / r1.z;
    const float w = 1.0f - u - v;
    if (u < 0.0f || v < 0.0f || w < 0.0f) return;
    const float z = (r1.w * u + r2.x * v) + r2.y * w;
    if (!(z < 0.0f)) return;
    const size_t gi = (size_t)py * P.W + px;
    if (gate_with_stencil && !stencil_test(P.stencil_test, __ldg(stencil + gi), P.sref)) return;
    const int kp = seam_count(px, P.tile_w, mx, P.W - 1) * seam_count(py, P.tile_h, my, P.H - 1);
    ++frags;
    const uint32_t zk = P.has_depth ? zkey(z) : 0u;
    atomicMax(gkeys + gi, ((unsigned long long)zk << 32) | (unsigned long long)((uint32_t)(kp - 1) * N + t + 1u));
}

constexpr uint32_t RG_BIG = 2048;   // bbox pixels above which a primitive goes to the block-cooperative pass

// Each warp takes G consecutive primitives (G a power of two <= 32, chosen by
// the host so that small meshes still spread over every SM); their bbox pixels
// are flattened into items spread over the lanes (warp prefix sum of the pixel
// counts and a log2(G)-step shuffle search for each lane's owner), so adjacent
// lanes test adjacent pixels.  Records are staged in shared memory per warp.
template <uint32_t G>
__global__ void __launch_bounds__(RG_THREADS) raster_small_kernel(
    DrawParams P, const float4* __restrict__ setup, const unsigned long long* __restrict__ area,
    unsigned long long* __restrict__ gkeys, uint32_t* __restrict__ bitmap, const uint8_t* __restrict__ stencil,
    uint32_t gate_with_stencil, uint32_t* __restrict__ big_list, DeviceFlags* flags) {
    __shared__ float4 srec[RG_THREADS / 32][32][3];
    __shared__ uint32_t sxy[RG_THREADS / 32][32];           // x0 | y0 << 16
    __shared__ uint32_t sw[RG_THREADS / 32][32];            // bbox width
    __shared__ unsigned long long smag[RG_THREADS / 32][32]; // ceil(2^32 / width)
    if (flags->poison) return;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long frags = 0;
    const uint32_t mx = div_magic(P.tile_w), my = div_magic(P.tile_h);
    const uint32_t blocks_x = (P.W + 31) >> 5;
    for (uint32_t t0 = warp * G; t0 < N; t0 += nwarps * G) {
        const uint32_t t = t0 + lane;
        uint32_t a = 0;
        if (lane < G && t < N) {
            const unsigned long long at = area[t];
            if (at > RG_BIG) {
                big_list[atomicAdd(&flags->n_big, 1ull)] = t;
            } else if (at) {
                a = (uint32_t)at;
                const float4* r = setup + 4 * (size_t)t;
                srec[wl][lane][0] = __ldg(r);
                srec[wl][lane][1] = __ldg(r + 1);
                srec[wl][lane][2] = __ldg(r + 2);
                const float4 r3 = __ldg(r + 3);
                const uint32_t x0 = (uint32_t)max(__float_as_int(r3.x), 0);
                const uint32_t y0 = (uint32_t)max(__float_as_int(r3.y), 0);
                const uint32_t x1 = (uint32_t)min(__float_as_int(r3.z), (int)P.W - 1);
                const uint32_t y1 = (uint32_t)min(__float_as_int(r3.w), (int)P.H - 1);
                const uint32_t w = x1 - x0 + 1;
                mark_rect(bitmap, blocks_x, x0, y0, x1, y1);
                sxy[wl][lane] = x0 | (y0 << 16);
                sw[wl][lane] = w;
                smag[wl][lane] = ((1ull << 32) + w - 1) / w;
            }
        }
        __syncwarp();
        const uint32_t inc = warp_inclusive_scan(a);
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        const uint32_t ex = inc - a;
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t q = base + lane;
            uint32_t lo = 0;
#pragma unroll
            for (uint32_t step = G >> 1; step >= 1; step >>= 1) {
                const uint32_t c = lo + step;
                const uint32_t v = __shfl_sync(0xffffffffu, ex, c & 31u);
                if (c < G && v <= q) lo = c;
            }
            const uint32_t exo = __shfl_sync(0xffffffffu, ex, lo);
            if (q < total) {
                const uint32_t local = q - exo;
                const uint32_t w = sw[wl][lo];
                const uint32_t row = (uint32_t)(((unsigned long long)local * smag[wl][lo]) >> 32);  // local / w
                const uint32_t xy = sxy[wl][lo];
                rg_fragment(P, srec[wl][lo][0], srec[wl][lo][1], srec[wl][lo][2], t0 + lo,
                            (xy & 0xffffu) + (local - row * w), (xy >> 16) + row, N, gkeys, bitmap, stencil,
                            gate_with_stencil, mx, my, frags);
            }
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if (lane == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// Primitives with large bboxes: each block strides over one primitive's pixels.
__global__ void __launch_bounds__(RG_THREADS) raster_big_kernel(
    DrawParams P, const float4* __restrict__ setup, const unsigned long long* __restrict__ area,
    unsigned long long* __restrict__ gkeys, uint32_t* __restrict__ bitmap, const uint8_t* __restrict__ stencil,
    uint32_t gate_with_stencil, const uint32_t* __restrict__ big_list, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t nb = (uint32_t)flags->n_big;
    unsigned long long frags = 0;
    const uint32_t mx = div_magic(P.tile_w), my = div_magic(P.tile_h);
    const uint32_t blocks_x = (P.W + 31) >> 5;
    for (uint32_t k = blockIdx.x; k < nb; k += gridDim.x) {
        const uint32_t t = big_list[k];
        const float4* r = setup + 4 * (size_t)t;
        const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
        const uint32_t x0 = (uint32_t)max(__float_as_int(r3.x), 0);
        const uint32_t y0 = (uint32_t)max(__float_as_int(r3.y), 0);
        const uint32_t x1 = (uint32_t)min(__float_as_int(r3.z), (int)P.W - 1);
        const uint32_t w = x1 - x0 + 1;
        const unsigned long long at = area[t];
        {
            const uint32_t y1 = (uint32_t)min(__float_as_int(r3.w), (int)P.H - 1);
            const uint32_t bx0 = x0 >> TOUCH_LOG2, by0 = y0 >> TOUCH_LOG2;
            const uint32_t nbx = (x1 >> TOUCH_LOG2) - bx0 + 1, nby = (y1 >> TOUCH_LOG2) - by0 + 1;
            for (uint32_t j = threadIdx.x; j < nbx * nby; j += RG_THREADS) {
                const uint32_t b = (by0 + j / nbx) * blocks_x + bx0 + j % nbx, bit = 1u << (b & 31);
                if (!(bitmap[b >> 5] & bit)) atomicOr(bitmap + (b >> 5), bit);
            }
        }
        for (unsigned long long j = threadIdx.x; j < at; j += RG_THREADS) {
            const uint32_t row = (uint32_t)(j / w), col = (uint32_t)(j - (unsigned long long)row * w);
            rg_fragment(P, r0, r1, r2, t, x0 + col, y0 + row, N, gkeys, bitmap, stencil, gate_with_stencil, mx, my, frags);
        }
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// Unsafe primitives: fragments at the clamped tile-edge targets outside the
// bbox (the projection of the bbox onto every semantic tile it does not
// overlap).  A segment is skipped when a sound sign test proves u, v or w
// negative on all of it; other pixels are evaluated exactly and emit their
// key with the rank of the tile being processed.

__global__ void __launch_bounds__(256) ext_direct_kernel(DrawParams P, const uint32_t* __restrict__ unsafe_list,
                                                         const float4* __restrict__ setup,
                                                         unsigned long long* __restrict__ gkeys,
                                                         uint32_t* __restrict__ bitmap, const uint8_t* __restrict__ stencil,
                                                         uint32_t gate_with_stencil, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t nu = (uint32_t)flags->n_unsafe_list;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t ntiles = P.ncols * P.nrows;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t blocks_x = (P.W + 31) >> 5;
    unsigned long long frags = 0;
    for (uint32_t k = warp; k < nu; k += nwarps) {
        const uint32_t t = unsafe_list[k];
        const float4* r = setup + 4 * (size_t)t;
        const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
        const int ix0 = __float_as_int(r3.x), iy0 = __float_as_int(r3.y);
        const int ix1 = __float_as_int(r3.z), iy1 = __float_as_int(r3.w);
        for (uint32_t ti = lane; ti < ntiles; ti += 32) {
            const uint32_t C = ti % P.ncols, R = ti / P.ncols;
            const uint32_t lx = C * P.tile_w, hx = min((C + 1) * P.tile_w, P.W - 1);
            const uint32_t ly = R * P.tile_h, hy = min((R + 1) * P.tile_h, P.H - 1);
            if (ix1 >= (int)lx && ix0 <= (int)hx && iy1 >= (int)ly && iy0 <= (int)hy) continue;
            const uint32_t cx0 = ix0 < (int)lx ? lx : (ix0 > (int)hx ? hx : (uint32_t)ix0);
            const uint32_t cx1 = ix1 < (int)lx ? lx : (ix1 > (int)hx ? hx : (uint32_t)ix1);
            const uint32_t cy0 = iy0 < (int)ly ? ly : (iy0 > (int)hy ? hy : (uint32_t)iy0);
            const uint32_t cy1 = iy1 < (int)ly ? ly : (iy1 > (int)hy ? hy : (uint32_t)iy1);
            if (segment_cleared(r0, r1, cx0, cy0, cx1, cy1)) continue;
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
                    mark_touched(bitmap, blocks_x, px, py);
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// Per touched 32x32 block: winner of each pixel vs the depth the draw started
// from, shading, colour and depth writes; keys and the bitmap bit are reset.
template <int FS, int FMT>
__global__ void __launch_bounds__(256) resolve_kernel(DrawParams P, sr_uniforms U, const float4* __restrict__ setup,
                                                      const uint32_t* __restrict__ vidx, const float* __restrict__ vary,
                                                      const uint32_t* __restrict__ tex, void* __restrict__ color,
                                                      float* __restrict__ depth, const uint8_t* __restrict__ stencil,
                                                      uint32_t gate_with_stencil, unsigned long long* __restrict__ gkeys,
                                                      uint32_t* __restrict__ bitmap, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t blocks_x = (P.W + 31) >> 5;
    const uint32_t b = blockIdx.x;
    if (!(bitmap[b >> 5] & (1u << (b & 31)))) return;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t X0 = (b % blocks_x) << 5, Y0 = (b / blocks_x) << 5;
    const uint32_t bw = min(32u, P.W - X0), bh = min(32u, P.H - Y0);
    for (uint32_t i = threadIdx.x; i < 1024; i += blockDim.x) {
        const uint32_t lx = i & 31, ly = i >> 5;
        if (lx >= bw || ly >= bh) continue;
        const uint32_t px = X0 + lx, py = Y0 + ly;
        const size_t gi = (size_t)py * P.W + px;
        const unsigned long long k = gkeys[gi];
        if (k == 0) continue;
        gkeys[gi] = 0;
        if (P.has_depth) {
            const float d0 = depth[gi];
            if (isnan(d0) || (uint32_t)(k >> 32) < zkey(d0)) continue;
        }
        if (gate_with_stencil && !stencil_test(P.stencil_test, stencil[gi], P.sref)) continue;
        const uint32_t t = ((uint32_t)(k & 0xffffffffull) - 1u) % N;
        const float4* r = setup + 4 * (size_t)t;
        const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2);
        const float x = (float)px + 0.5f, y = (float)py + 0.5f;
        const float dx = x - r1.x, dy = y - r1.y;
        const float u = (r0.x * dx + r0.y * dy) / r1.z;
        const float v = (r0.z * dx + r0.w * dy) / r1.z;
        const float w = 1.0f - u - v;
        const float z = (r1.w * u + r2.x * v) + r2.y * w;
        constexpr int NK = FS == FS_TEXTURED_BLINN_PHONG ? 10 : FS == FS_VERTEX_COLOR ? 4 : FS == FS_CONSTANT_COLOR ? 0 : 8;
        float kv[12];
        if (NK > 0) {
            const uint32_t a = __ldg(vidx + 3 * (size_t)t), bq = __ldg(vidx + 3 * (size_t)t + 1),
                           c = __ldg(vidx + 3 * (size_t)t + 2);
            const float4* ka = reinterpret_cast<const float4*>(vary + (size_t)a * VSTRIDE);
            const float4* kb = reinterpret_cast<const float4*>(vary + (size_t)bq * VSTRIDE);
            const float4* kc = reinterpret_cast<const float4*>(vary + (size_t)c * VSTRIDE);
#pragma unroll
            for (int q = 0; q < (NK + 3) / 4; ++q) {
                const float4 xa = __ldg(ka + q), xb = __ldg(kb + q), xc = __ldg(kc + q);
                kv[4 * q + 0] = (xa.x * u + xb.x * v) + xc.x * w;
                kv[4 * q + 1] = (xa.y * u + xb.y * v) + xc.y * w;
                kv[4 * q + 2] = (xa.z * u + xb.z * v) + xc.z * w;
                kv[4 * q + 3] = (xa.w * u + xb.w * v) + xc.w * w;
            }
        }
        const sr_v4 col = shade_fs<FS>(U, kv, tex, P);
        if (FMT == SR_COLOR_RGBA32F) reinterpret_cast<float4*>(color)[gi] = make_float4(col.x, col.y, col.z, col.w);
        else if (FMT == SR_COLOR_RGBA8) reinterpret_cast<uint32_t*>(color)[gi] = sr_to_rgba8(col);
        if (P.has_depth) depth[gi] = z;
    }
    __syncthreads();
    if (threadIdx.x == 0) atomicAnd(bitmap + (b >> 5), ~(1u << (b & 31)));
}

template <int FS>
static void launch_resolve_fs(const DrawParams& P, const sr_uniforms& U, const OpaqueArgs& A, cudaStream_t st) {
    const uint32_t nblk = ((P.W + 31) >> 5) * ((P.H + 31) >> 5);
#define SR_RES(FMT) resolve_kernel<FS, FMT><<<nblk, 256, 0, st>>>(P, U, A.setup, A.vidx, A.vary, A.tex, A.color, \
        A.depth, A.stencil, A.gate, A.gkeys, A.bitmap, A.flags)
    if (P.color_format == SR_COLOR_RGBA32F) SR_RES(SR_COLOR_RGBA32F);
    else if (P.color_format == SR_COLOR_RGBA8) SR_RES(SR_COLOR_RGBA8);
    else SR_RES(SR_COLOR_NONE);
#undef SR_RES
}

// launches: raster_small, raster_big, ext_direct, resolve
int launch_opaque(const DrawParams& P, const sr_uniforms& U, const OpaqueArgs& A, cudaStream_t st) {
    // primitives per warp: 32, halved while that would leave fewer warps than
    // the GPU holds (152 SMs x 48 resident warps); clipped draws estimate the
    // primitive count by the input count
    const uint32_t n_est = P.n_raster_host ? P.n_raster_host : P.n_in;
    uint32_t G = 32;
    while (G > 1 && n_est / G < 152u * 48u) G >>= 1;
#define SR_RS(g) raster_small_kernel<g><<<152 * 8, RG_THREADS, 0, st>>>(P, A.setup, A.area, A.gkeys, A.bitmap, \
                                                                      A.stencil, A.gate, A.big_list, A.flags)
    switch (G) {
    case 1: SR_RS(1); break;
    case 2: SR_RS(2); break;
    case 4: SR_RS(4); break;
    case 8: SR_RS(8); break;
    case 16: SR_RS(16); break;
    default: SR_RS(32); break;
    }
#undef SR_RS
    raster_big_kernel<<<152 * 2, RG_THREADS, 0, st>>>(P, A.setup, A.area, A.gkeys, A.bitmap, A.stencil, A.gate,
                                                       A.big_list, A.flags);
    ext_direct_kernel<<<152 * 4, 256, 0, st>>>(P, A.unsafe_list, A.setup, A.gkeys, A.bitmap, A.stencil, A.gate, A.flags);
    switch (P.fs) {
    case FS_BLINN_PHONG_DIR: launch_resolve_fs<FS_BLINN_PHONG_DIR>(P, U, A, st); break;
    case FS_TEXTURED_BLINN_PHONG: launch_resolve_fs<FS_TEXTURED_BLINN_PHONG>(P, U, A, st); break;
    case FS_VERTEX_COLOR: launch_resolve_fs<FS_VERTEX_COLOR>(P, U, A, st); break;
    case FS_ACES_LIGHTS: launch_resolve_fs<FS_ACES_LIGHTS>(P, U, A, st); break;
    default: launch_resolve_fs<FS_CONSTANT_COLOR>(P, U, A, st); break;
    }
    return 4;
}

}  // namespace sr
