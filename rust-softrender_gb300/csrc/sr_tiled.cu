// sr_tiled.cu — the opaque draw path over 32x32 screen bins.
//
// Opaque draws (blend `()`, shaders that never discard) leave each pixel with
// the shade of its winning fragment: the maximum over all fragments of the
// 64-bit key  zkey(z) << 32 | pass * N + primitive + 1  (sr_opaque.cu states
// why).  The maximum does not depend on the order fragments arrive in, so
// here every 32x32 bin of the frame is one CTA that owns its pixels' keys in
// shared memory:
//   1. setup counts, per bin, the primitives whose clamped bbox meets it;
//   2. one CTA scans the counts into list offsets;
//   3. every primitive writes its index into the list of each of those bins
//      (order within a list is free: the key maximum decides);
//   4. unsafe primitives' fragments outside their bbox (the clamped
//      tile-edge events of triangle.rs:66-78) go, rarely, through the global
//      key buffer and the touched-bin bitmap (ext_direct_kernel);
//   5. the bin kernel seeds its 1024 keys (from the global buffer where the
//      bitmap says so), walks its primitive list with the bbox pixels of a
//      warp's primitives flattened over the lanes (shared-memory atomicMax
//      of the key), and then resolves its pixels in place: start depth,
//      winner's barycentrics, varyings, shading, one colour and depth write.
// Nothing per pixel goes through global memory except the framebuffer itself
// (and the rare extension keys), and no global atomics are taken per
// fragment.
#include "sr_internal.cuh"
#include "sr_scan.cuh"
#include "sr_shade.cuh"
#include "sr_opaque.cuh"
#include "sr_setup.cuh"

namespace sr {

constexpr uint32_t TL_THREADS = 256;
constexpr uint32_t TL_WARPS = TL_THREADS / 32;
constexpr uint32_t TL_BIN_LOG2 = 5;   // bins of 32 x 32 pixels (the touched-block bitmap's granularity)
static_assert(TL_BIN_LOG2 == TOUCH_LOG2, "the extension keys' bitmap marks bins");

// Exclusive scan of n <= 2^24 bin counts in one CTA: each thread sums a
// contiguous run, the CTA scans the run sums, each thread writes its run's
// offsets.  out[n] = total.
__global__ void __launch_bounds__(1024) bin_scan_kernel(const uint32_t* __restrict__ in, uint32_t n,
                                                        uint32_t* __restrict__ out, const DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t per = (n + 1023) / 1024;
    const uint32_t j0 = threadIdx.x * per, j1 = min(j0 + per, n);
    uint32_t s = 0;
    for (uint32_t j = j0; j < j1; ++j) s += in[j];
    uint32_t tot;
    uint32_t ex = block_exclusive_scan<uint32_t, 1024>(s, &tot);
    for (uint32_t j = j0; j < j1; ++j) {
        const uint32_t v = in[j];
        out[j] = ex;
        ex += v;
    }
    if (threadIdx.x == 0) out[n] = tot;
}

// Writes every primitive into the list of each bin its clamped bbox meets.
// A draw whose lists outgrow the entry buffer poisons the pipeline (sr_sync
// grows the buffer and replays).  `cursor` (n_bins, zero) counts the slots
// taken per bin.  One-bin primitives of a warp that share a bin take their
// slots with one atomic.
__global__ void __launch_bounds__(256) bin_scatter_kernel(uint32_t n_host, uint32_t n_launch, uint32_t bins_x,
                                                          const uint2* __restrict__ binrect,
                                                          const uint32_t* __restrict__ bin_off, uint32_t n_bins,
                                                          uint32_t* __restrict__ cursor, uint32_t* __restrict__ entries,
                                                          uint64_t cap, uint32_t draw_id, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t total = bin_off[n_bins];
    if (total > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (total > flags->need_entries) flags->need_entries = total;
            atomicOr(&flags->overflow_bits, (unsigned)OVF_ENTRIES);
            atomicOr(&flags->poison, 1u);
            atomicMin(&flags->poison_draw, draw_id);
        }
        return;
    }
    const uint32_t n = n_host ? n_host : (uint32_t)flags->n_gen_tris;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    uint2 br = make_uint2(RECT_EMPTY, RECT_EMPTY);
    if (t < n && t < n_launch) br = binrect[t];
    uint32_t bx0 = 1, by0 = 1, bx1 = 0, by1 = 0;
    uint32_t single = 0xffffffffu;   // the bin of a one-bin primitive
    if (br.x != RECT_EMPTY) {
        bx0 = br.x & 0xffffu; by0 = br.x >> 16; bx1 = br.y & 0xffffu; by1 = br.y >> 16;
        if (bx0 == bx1 && by0 == by1) single = by0 * bins_x + bx0;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, single);
    const uint32_t leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (single != 0xffffffffu && lane == leader) base = atomicAdd(cursor + single, (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (single != 0xffffffffu) {
        entries[bin_off[single] + base + __popc(peers & ((1u << lane) - 1u))] = t;
    } else if (br.x != RECT_EMPTY) {
        for (uint32_t by = by0; by <= by1; ++by)
            for (uint32_t bx = bx0; bx <= bx1; ++bx) {
                const uint32_t b = by * bins_x + bx;
                entries[bin_off[b] + atomicAdd(cursor + b, 1u)] = t;
            }
    }
}

// One CTA per 32x32 bin.  G = primitives a warp takes from the bin's list at a
// time; their bbox pixels (clipped to the bin) are flattened over the lanes in
// items of two horizontally adjacent pixels, as in raster_small_kernel.
template <int FS, int FMT, uint32_t G>
__global__ void __launch_bounds__(TL_THREADS) bin_raster_kernel(
    DrawParams P, sr_uniforms U, const float4* __restrict__ setup, const uint32_t* __restrict__ bin_off,
    const uint32_t* __restrict__ entries, const uint32_t* __restrict__ vidx, const float* __restrict__ vary,
    const uint32_t* __restrict__ tex, void* __restrict__ color, float* __restrict__ depth,
    const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil, unsigned long long* __restrict__ gkeys,
    uint32_t* __restrict__ bitmap, DeviceFlags* flags) {
    __shared__ unsigned long long keys[1u << (2 * TL_BIN_LOG2)];
    __shared__ float4 srec[TL_WARPS][G][3];
    __shared__ uint32_t sxy[TL_WARPS][G];             // x0 | y0 << 16 (bin-relative) | seam bits 15, 31
    __shared__ uint32_t sw[TL_WARPS][G];              // pairs per row | clipped width << 16
    __shared__ uint32_t sst[TL_WARPS][G];             // first item
    __shared__ uint32_t st[TL_WARPS][G];              // primitive index
    __shared__ unsigned long long smag[TL_WARPS][G];  // ceil(2^32 / pairs per row)
    __shared__ uint32_t s_next;
    if (flags->poison) return;
    const uint32_t b = blockIdx.x;
    const uint32_t e0 = bin_off[b], cnt = bin_off[b + 1] - e0;
    const bool ext = (bitmap[b >> 5] >> (b & 31)) & 1u;
    if (cnt == 0 && !ext) return;   // no fragment can land here: the pixels keep their values
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t X0 = (b % P.bins_x) << TL_BIN_LOG2, Y0 = (b / P.bins_x) << TL_BIN_LOG2;
    const uint32_t X1 = min(X0 + (1u << TL_BIN_LOG2) - 1, P.W - 1), Y1 = min(Y0 + (1u << TL_BIN_LOG2) - 1, P.H - 1);
    for (uint32_t i = threadIdx.x; i < (1u << (2 * TL_BIN_LOG2)); i += TL_THREADS) {
        unsigned long long k = 0;
        if (ext) {
            const uint32_t px = X0 + (i & 31), py = Y0 + (i >> TL_BIN_LOG2);
            if (px <= X1 && py <= Y1) {
                const size_t gi = (size_t)py * P.W + px;
                k = gkeys[gi];
                if (k) gkeys[gi] = 0;
            }
        }
        keys[i] = k;
    }
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();

    const uint32_t lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    unsigned long long frags = 0;
    const uint32_t mx = div_magic(P.tile_w), my = div_magic(P.tile_h);
    for (;;) {
        uint32_t k0 = 0;
        if (lane == 0) k0 = atomicAdd(&s_next, G);
        k0 = __shfl_sync(0xffffffffu, k0, 0);
        if (k0 >= cnt) break;
        uint32_t a = 0, x0 = 0, y0 = 0, x1 = 0, y1 = 0, t = 0;
        if (lane < G && k0 + lane < cnt) {
            t = __ldg(entries + e0 + k0 + lane);
            const float4 r3 = __ldg(setup + 4 * (size_t)t + 3);
            x0 = (uint32_t)max(__float_as_int(r3.x), (int)X0);
            y0 = (uint32_t)max(__float_as_int(r3.y), (int)Y0);
            x1 = (uint32_t)min(__float_as_int(r3.z), (int)X1);
            y1 = (uint32_t)min(__float_as_int(r3.w), (int)Y1);
            if (x0 <= x1 && y0 <= y1) a = (y1 - y0 + 1) * ((x1 - x0 + 2) >> 1);
        }
        const uint32_t inc = warp_inclusive_scan(a);
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        const uint32_t ex = inc - a;
        const uint32_t nonempty = __ballot_sync(0xffffffffu, a != 0);
        if (a) {
            const uint32_t c = __popc(nonempty & ((1u << lane) - 1u));
            const float4* r = setup + 4 * (size_t)t;
            srec[wl][c][0] = __ldg(r);
            srec[wl][c][1] = __ldg(r + 1);
            srec[wl][c][2] = __ldg(r + 2);
            const uint32_t w = x1 - x0 + 1, wp = (w + 1) >> 1;
            const uint32_t sb = seam_bits(x0, y0, x1, y1, P.W, P.H, P.tile_w, P.tile_h);
            sxy[wl][c] = (x0 - X0) | ((y0 - Y0) << 16) | ((sb & 1u) << 15) | ((sb & 2u) << 30);
            sw[wl][c] = wp | (w << 16);
            sst[wl][c] = ex;
            st[wl][c] = t;
            smag[wl][c] = ((1ull << 32) + wp - 1) / wp;
        }
        __syncwarp();
        const uint32_t le = (2u << lane) - 1u;
        uint32_t before = 0;
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t q = base + lane;
            const uint32_t rel = ex - base;
            const uint32_t starts = __reduce_or_sync(0xffffffffu, (a && rel < 32u) ? (1u << rel) : 0u);
            const uint32_t o = before + __popc(starts & le) - 1u;
            before += __popc(starts);
            if (q < total) {
                const uint32_t local = q - sst[wl][o];
                const uint32_t wpw = sw[wl][o], wp = wpw & 0xffffu;
                const uint32_t row = (uint32_t)(((unsigned long long)local * smag[wl][o]) >> 32);
                const uint32_t col = 2 * (local - row * wp);
                const uint32_t xy = sxy[wl][o];
                const float4 r0 = srec[wl][o][0], r1 = srec[wl][o][1], r2 = srec[wl][o][2];
                const uint32_t lx = (xy & 0x7fffu) + col, ly = ((xy >> 16) & 0x7fffu) + row, tt = st[wl][o];
                const uint32_t seams = ((xy >> 15) & 1u) | ((xy >> 30) & 2u);
                const uint32_t slot = (ly << TL_BIN_LOG2) + lx;
                unsigned long long k = frag_key(P.W, P.H, P.tile_w, P.tile_h, mx, my, seams, P.has_depth != 0, r0, r1,
                                                r2, tt, X0 + lx, Y0 + ly, N, stencil, gate_with_stencil,
                                                P.stencil_test, P.sref, frags);
                if (k) atomicMax(keys + slot, k);
                if (col + 1 < (wpw >> 16)) {
                    k = frag_key(P.W, P.H, P.tile_w, P.tile_h, mx, my, seams, P.has_depth != 0, r0, r1, r2, tt,
                                 X0 + lx + 1, Y0 + ly, N, stencil, gate_with_stencil, P.stencil_test, P.sref, frags);
                    if (k) atomicMax(keys + slot + 1, k);
                }
            }
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if (lane == 0 && frags) atomicAdd(&flags->fragments, frags);
    __syncthreads();
    if (ext && threadIdx.x == 0) atomicAnd(bitmap + (b >> 5), ~(1u << (b & 31)));

    // resolve: the bin's pixels with a winner
    for (uint32_t i = threadIdx.x; i < (1u << (2 * TL_BIN_LOG2)); i += TL_THREADS) {
        const unsigned long long k = keys[i];
        if (!k) continue;
        const uint32_t px = X0 + (i & 31), py = Y0 + (i >> TL_BIN_LOG2);
        if (px > X1 || py > Y1) continue;
        const float d0 = P.has_depth ? depth[(size_t)py * P.W + px] : 0.0f;
        resolve_pixel<FS, FMT>(P, U, px, py, k, d0, N, setup, vidx, vary, tex, color, depth, stencil,
                               gate_with_stencil);
    }
}

template <int FS>
static void launch_bin_raster_fs(const DrawParams& P, const sr_uniforms& U, const TiledArgs& A, uint32_t n_bins,
                                 cudaStream_t st) {
#define SR_BR(FMT) bin_raster_kernel<FS, FMT, 16><<<n_bins, TL_THREADS, 0, st>>>(P, U, A.setup, A.bin_off, A.entries, \
        A.vidx, A.vary, A.tex, A.color, A.depth, A.stencil, A.gate, A.gkeys, A.bitmap, A.flags)
    if (P.color_format == SR_COLOR_RGBA32F) SR_BR(SR_COLOR_RGBA32F);
    else if (P.color_format == SR_COLOR_RGBA8) SR_BR(SR_COLOR_RGBA8);
    else SR_BR(SR_COLOR_NONE);
#undef SR_BR
}

void ext_direct_launch(const DrawParams& P, const uint32_t* unsafe_list, const float4* unsafe_rect,
                       const float4* setup, unsigned long long* gkeys, uint32_t* bitmap, const uint8_t* stencil,
                       uint32_t gate, DeviceFlags* flags, cudaStream_t st);

// launches: bin scan, scatter, extension keys, bin raster (setup, with the
// bin counts, is launched by the caller)
int launch_tiled(const DrawParams& P, const sr_uniforms& U, const TiledArgs& A, cudaStream_t st) {
    const uint32_t n_bins = P.bins_x * P.bins_y;
    bin_scan_kernel<<<1, 1024, 0, st>>>(A.bin_counts, n_bins, A.bin_off, A.flags);
    const uint32_t n_launch = P.n_raster_host ? P.n_raster_host : P.gen_tri_cap;
    bin_scatter_kernel<<<(n_launch + 255) / 256 ? (n_launch + 255) / 256 : 1, 256, 0, st>>>(
        P.n_raster_host, n_launch, P.bins_x, A.binrect, A.bin_off, n_bins, A.cursor, A.entries, A.entry_cap,
        P.draw_id, A.flags);
    ext_direct_launch(P, A.unsafe_list, A.unsafe_rect, A.setup, A.gkeys, A.bitmap, A.stencil, A.gate, A.flags, st);
    switch (P.fs) {
    case FS_BLINN_PHONG_DIR: launch_bin_raster_fs<FS_BLINN_PHONG_DIR>(P, U, A, n_bins, st); break;
    case FS_TEXTURED_BLINN_PHONG: launch_bin_raster_fs<FS_TEXTURED_BLINN_PHONG>(P, U, A, n_bins, st); break;
    case FS_VERTEX_COLOR: launch_bin_raster_fs<FS_VERTEX_COLOR>(P, U, A, n_bins, st); break;
    case FS_ACES_LIGHTS: launch_bin_raster_fs<FS_ACES_LIGHTS>(P, U, A, n_bins, st); break;
    default: launch_bin_raster_fs<FS_CONSTANT_COLOR>(P, U, A, n_bins, st); break;
    }
    return 4;
}

}  // namespace sr
