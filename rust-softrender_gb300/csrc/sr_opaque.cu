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
#include "sr_opaque.cuh"

namespace sr {


// Each warp takes G consecutive primitives (G a power of two <= 32, chosen by
// the host so that small meshes still spread over every SM); their bbox pixels
// are flattened into items spread over the lanes (warp prefix sum of the pixel
// counts), so adjacent lanes test adjacent pixels.  The non-empty primitives'
// records are staged, compacted, in shared memory per warp; for each window of
// 32 items the lanes OR-reduce a mask of the primitive starts inside it, and
// an item's owner is the number of starts at or before it, less one.
template <uint32_t G>
__global__ void __launch_bounds__(RG_THREADS) raster_small_kernel(
    DrawParams P, const float4* __restrict__ setup, const unsigned long long* __restrict__ area,
    unsigned long long* __restrict__ gkeys, uint32_t* __restrict__ bitmap, const uint8_t* __restrict__ stencil,
    uint32_t gate_with_stencil, uint32_t* __restrict__ big_list, DeviceFlags* flags) {
    __shared__ float4 srec[RG_THREADS / 32][32][3];
    __shared__ uint32_t sxy[RG_THREADS / 32][32];           // x0 | y0 << 16
    __shared__ uint32_t sw[RG_THREADS / 32][32];            // pairs per row | bbox width << 16
    __shared__ uint32_t sst[RG_THREADS / 32][32];           // first item
    __shared__ uint32_t st[RG_THREADS / 32][32];            // primitive index
    __shared__ unsigned long long smag[RG_THREADS / 32][32]; // ceil(2^32 / pairs per row)
    if (flags->poison) return;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    unsigned long long frags = 0;
    const uint32_t mx = P.magic_w, my = P.magic_h;
    const uint32_t blocks_x = (P.W + 31) >> 5;
    for (;;) {
        // dynamic work queue: a warp takes the next G primitives
        uint32_t t0 = 0;
        if (lane == 0) t0 = (uint32_t)min(atomicAdd(&flags->work_raster, (unsigned long long)G), 0xffffffffull);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= N) break;
        const uint32_t t = t0 + lane;
        // items: horizontal pairs of bbox pixels, ceil(w / 2) per bbox row
        uint32_t a = 0, x0 = 0, y0 = 0, x1 = 0, y1 = 0;
        if (lane < G && t < N) {
            const unsigned long long at = area[t];
            if (at > RG_BIG) {
                big_list[atomicAdd(&flags->n_big, 1ull)] = t;
            } else if (at) {
                const float4 r3 = __ldg(setup + 4 * (size_t)t + 3);
                x0 = (uint32_t)max(__float_as_int(r3.x), 0);
                y0 = (uint32_t)max(__float_as_int(r3.y), 0);
                x1 = (uint32_t)min(__float_as_int(r3.z), (int)P.W - 1);
                y1 = (uint32_t)min(__float_as_int(r3.w), (int)P.H - 1);
                a = (y1 - y0 + 1) * ((x1 - x0 + 2) >> 1);
            }
        }
        const uint32_t inc = warp_inclusive_scan(a);
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        const uint32_t ex = inc - a;
        const uint32_t nonempty = __ballot_sync(0xffffffffu, a != 0);
        if (a) {
            // compacted slot: the rank of this primitive among the non-empty ones
            const uint32_t c = __popc(nonempty & ((1u << lane) - 1u));
            const float4* r = setup + 4 * (size_t)t;
            srec[wl][c][0] = __ldg(r);
            srec[wl][c][1] = __ldg(r + 1);
            srec[wl][c][2] = __ldg(r + 2);
            const uint32_t w = x1 - x0 + 1, wp = (w + 1) >> 1;
            mark_rect(bitmap, blocks_x, x0, y0, x1, y1);
            const uint32_t sb = seam_bits(x0, y0, x1, y1, P);
            sxy[wl][c] = x0 | (y0 << 16) | ((sb & 1u) << 15) | ((sb & 2u) << 30);
            sw[wl][c] = wp | (w << 16);
            sst[wl][c] = ex;
            st[wl][c] = t;
            smag[wl][c] = ((1ull << 32) + wp - 1) / wp;
        }
        __syncwarp();
        const uint32_t le = (2u << lane) - 1u;   // lanes 0..lane
        uint32_t before = 0;                     // primitive starts before the window
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t q = base + lane;
            const uint32_t rel = ex - base;
            const uint32_t starts = __reduce_or_sync(0xffffffffu, (a && rel < 32u) ? (1u << rel) : 0u);
            const uint32_t o = before + __popc(starts & le) - 1u;
            before += __popc(starts);
            if (q < total) {
                const uint32_t local = q - sst[wl][o];
                const uint32_t wpw = sw[wl][o], wp = wpw & 0xffffu;
                const uint32_t row = (uint32_t)(((unsigned long long)local * smag[wl][o]) >> 32);  // local / wp
                const uint32_t col = 2 * (local - row * wp);
                const uint32_t xy = sxy[wl][o];
                const float4 r0 = srec[wl][o][0], r1 = srec[wl][o][1], r2 = srec[wl][o][2];
                const uint32_t px = (xy & 0x7fffu) + col, py = ((xy >> 16) & 0x7fffu) + row, tt = st[wl][o];
                const uint32_t seams = ((xy >> 15) & 1u) | ((xy >> 30) & 2u);
                rg_fragment(P, r0, r1, r2, tt, px, py, N, gkeys, bitmap, stencil, gate_with_stencil, mx, my, seams,
                            frags);
                if (col + 1 < (wpw >> 16))
                    rg_fragment(P, r0, r1, r2, tt, px + 1, py, N, gkeys, bitmap, stencil, gate_with_stencil, mx, my,
                                seams, frags);
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
    const uint32_t mx = P.magic_w, my = P.magic_h;
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
        const uint32_t sb = seam_bits(x0, y0, x1, (uint32_t)min(__float_as_int(r3.w), (int)P.H - 1), P);
        {
            const uint32_t y1 = (uint32_t)min(__float_as_int(r3.w), (int)P.H - 1);
            const uint32_t bx0 = x0 >> TOUCH_LOG2, by0 = y0 >> TOUCH_LOG2;
            const uint32_t nbx = (x1 >> TOUCH_LOG2) - bx0 + 1, nby = (y1 >> TOUCH_LOG2) - by0 + 1;
            for (uint32_t j = threadIdx.x; j < nbx * nby; j += RG_THREADS) {
                const uint32_t b = (by0 + j / nbx) * blocks_x + bx0 + j % nbx, bit = 1u << (b & 31);
                if (!(bitmap[b >> 5] & bit)) atomicOr(bitmap + (b >> 5), bit);
            }
        }
        // each thread steps its (row, column) by RG_THREADS bbox pixels
        // instead of dividing per pixel
        uint32_t row = threadIdx.x / w, col = threadIdx.x - row * w;
        const uint32_t drow = RG_THREADS / w, dcol = RG_THREADS - drow * w;
        for (uint32_t j = threadIdx.x; j < (uint32_t)at; j += RG_THREADS) {
            rg_fragment(P, r0, r1, r2, t, x0 + col, y0 + row, N, gkeys, bitmap, stencil, gate_with_stencil, mx, my,
                        sb, frags);
            row += drow;
            col += dcol;
            if (col >= w) { col -= w; ++row; }
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
                                                         const float4* __restrict__ unsafe_rect,
                                                         const float4* __restrict__ setup,
                                                         unsigned long long* __restrict__ gkeys,
                                                         uint32_t* __restrict__ bitmap, const uint8_t* __restrict__ stencil,
                                                         uint32_t gate_with_stencil, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t nu = (uint32_t)flags->n_unsafe_list;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t blocks_x = (P.W + 31) >> 5;
    unsigned long long frags = 0;
    for (uint32_t k = warp; k < nu; k += nwarps) {
        // a primitive with a bounded coverage region takes the ring of pixels
        // around its bbox; the rest every semantic tile's clamped segment
        const float4 rg = unsafe_rect ? unsafe_rect[k] : make_float4(NAN, NAN, NAN, NAN);
        if (!isnan(rg.x))
            ext_prim_ring(P, unsafe_list[k], N, rg, setup, gkeys, stencil, gate_with_stencil, lane, frags,
                          [=](uint32_t px, uint32_t py) { mark_touched(bitmap, blocks_x, px, py); });
        else
            ext_prim(P, unsafe_list[k], N, setup, gkeys, bitmap, stencil, gate_with_stencil, lane, frags);
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
    const uint32_t b = blockIdx.x;
    if (!(bitmap[b >> 5] & (1u << (b & 31)))) return;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    resolve_block<FS, FMT>(P, U, b, N, setup, vidx, vary, tex, color, depth, stencil, gate_with_stencil, gkeys,
                           bitmap);
}

void ext_direct_launch(const DrawParams& P, const uint32_t* unsafe_list, const float4* unsafe_rect,
                       const float4* setup, unsigned long long* gkeys, uint32_t* bitmap, const uint8_t* stencil,
                       uint32_t gate, DeviceFlags* flags, cudaStream_t st) {
    ext_direct_kernel<<<resident_grid(ext_direct_kernel, 256, 4), 256, 0, st>>>(P, unsafe_list, unsafe_rect, setup,
                                                                               gkeys, bitmap, stencil, gate, flags);
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
    // the GPU holds (48 resident warps per SM); clipped draws estimate the
    // primitive count by the input count
    const uint32_t n_est = P.n_raster_host ? P.n_raster_host : P.n_in;
    uint32_t G = 32;
    while (G > 1 && n_est / G < (uint32_t)sm_count() * 48u) G >>= 1;
#define SR_RS(g) raster_small_kernel<g><<<resident_grid(raster_small_kernel<g>, RG_THREADS, 8), RG_THREADS, 0, st>>>( \
        P, A.setup, A.area, A.gkeys, A.bitmap, \
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
    raster_big_kernel<<<resident_grid(raster_big_kernel, RG_THREADS, 2), RG_THREADS, 0, st>>>(P, A.setup, A.area, A.gkeys, A.bitmap, A.stencil, A.gate,
                                                       A.big_list, A.flags);
    ext_direct_launch(P, A.unsafe_list, A.unsafe_rect, A.setup, A.gkeys, A.bitmap, A.stencil, A.gate, A.flags, st);
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
