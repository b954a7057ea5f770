// sr_bins.cu — bin lists of the ordered raster path, in submission order.
//
// The ordered kernel (sr_raster.cu) replays each bin's primitives in
// submission order, so every bin needs its primitives sorted.  The lists are
// built without per-bin sorting or atomic cursors:
//   1. every raster primitive counts its (bin, primitive) pairs: the bins of
//      its bbox rectangle plus, for unsafe primitives, the bins of its
//      clamped tile-edge fragments outside that rectangle;
//   2. an exclusive scan over primitives gives each primitive its slice, and
//      the pairs are written in primitive order;
//   3. a stable LSD radix sort by bin (8-bit digits) keeps that order within
//      each bin;
//   4. each bin's [begin, end) range is read off the sorted keys.
#include "sr_internal.cuh"
#include "sr_scan.cuh"
#include "sr_setup.cuh"

namespace sr {

constexpr uint32_t RADIX_THREADS = 256;
constexpr uint32_t RADIX_ITEMS = 8;                            // per thread
constexpr uint32_t RADIX_TILE = RADIX_THREADS * RADIX_ITEMS;   // items per block

__device__ __forceinline__ uint32_t rect_count(uint2 br) {
    if (br.x == RECT_EMPTY) return 0;
    const uint32_t bx0 = br.x & 0xffffu, by0 = br.x >> 16, bx1 = br.y & 0xffffu, by1 = br.y >> 16;
    return (bx1 - bx0 + 1) * (by1 - by0 + 1);
}

// pairs per primitive: the bbox rectangle's bins (extension bins are added
// by ext_count_kernel)
__global__ void prim_count_kernel(uint32_t n_host, uint32_t n_launch, const uint2* __restrict__ binrect,
                                  uint32_t* __restrict__ pcount, DeviceFlags* flags) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = n_host ? n_host : (uint32_t)flags->n_gen_tris;   // primitives of this draw
    if (flags->poison || t >= n || t >= n_launch) return;
    pcount[t] = rect_count(binrect[t]);
}

__global__ void __launch_bounds__(256) ext_count_kernel(DrawParams P, const uint32_t* __restrict__ unsafe_list,
                                                        const float4* __restrict__ setup,
                                                        const uint2* __restrict__ binrect,
                                                        uint32_t* __restrict__ pcount, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t nu = (uint32_t)flags->n_unsafe_list;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long emitted = 0;
    for (uint32_t k = warp; k < nu; k += nwarps) {
        const uint32_t t = unsafe_list[k];
        uint32_t c = 0;
        ext_bins(P, setup, binrect[t], t, lane, [&](uint32_t) { ++c; });
        for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
        if (lane == 0) {
            pcount[t] += c;
            emitted += c;
        }
    }
    if (lane == 0 && emitted) atomicAdd(&flags->entries, emitted);
}

// total pairs against the capacity of the pair buffers
__global__ void check_pairs_kernel(uint32_t n, const uint32_t* __restrict__ poff, uint64_t cap, uint32_t draw_id,
                                   DeviceFlags* flags) {
    if (flags->poison) return;
    const unsigned long long tot = poff[n];
    if (tot > flags->need_entries) flags->need_entries = tot;
    if (tot > cap) {
        atomicOr(&flags->overflow_bits, (unsigned)OVF_ENTRIES);
        atomicOr(&flags->poison, 1u);
        atomicMin(&flags->poison_draw, draw_id);
    }
}

// the bbox rectangle's pairs of primitive t at its slice (row-major bins)
// (order within a primitive's slice is free: each bin occurs once in it).
// Rectangles of more than 16 bins are written by the whole warp, one bin per
// lane, so a few large primitives do not serialise their warps.
__global__ void __launch_bounds__(256) prim_emit_kernel(DrawParams P, uint32_t n_host, uint32_t n_launch,
                                                        const uint2* __restrict__ binrect,
                                                        const uint32_t* __restrict__ poff, uint32_t* __restrict__ keys,
                                                        uint32_t* __restrict__ vals, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = n_host ? n_host : (uint32_t)flags->n_gen_tris;
    const uint32_t lane = threadIdx.x & 31;
    uint2 br = make_uint2(RECT_EMPTY, RECT_EMPTY);
    if (t < n && t < n_launch) br = binrect[t];
    uint32_t bx0 = 1, by0 = 1, bx1 = 0, by1 = 0, nb = 0, o = 0;
    if (br.x != RECT_EMPTY) {
        bx0 = br.x & 0xffffu; by0 = br.x >> 16; bx1 = br.y & 0xffffu; by1 = br.y >> 16;
        nb = (bx1 - bx0 + 1) * (by1 - by0 + 1);
        o = poff[t];
    }
    if (nb && nb <= 16) {
        for (uint32_t by = by0; by <= by1; ++by)
            for (uint32_t bx = bx0; bx <= bx1; ++bx) {
                keys[o] = by * P.bins_x + bx;
                vals[o] = t;
                ++o;
            }
    }
    uint32_t big = __ballot_sync(0xffffffffu, nb > 16);
    while (big) {
        const uint32_t src = __ffs(big) - 1;
        big &= big - 1;
        const uint32_t sx0 = __shfl_sync(0xffffffffu, bx0, src), sy0 = __shfl_sync(0xffffffffu, by0, src);
        const uint32_t sw = __shfl_sync(0xffffffffu, bx1, src) - sx0 + 1;
        const uint32_t sn = __shfl_sync(0xffffffffu, nb, src), so = __shfl_sync(0xffffffffu, o, src);
        const uint32_t st = __shfl_sync(0xffffffffu, t, src);
        for (uint32_t i = lane; i < sn; i += 32) {
            keys[so + i] = (sy0 + i / sw) * P.bins_x + sx0 + i % sw;
            vals[so + i] = st;
        }
    }
}

// the extension pairs of unsafe primitives, after their rectangle's pairs
__global__ void __launch_bounds__(256) ext_emit_kernel(DrawParams P, const uint32_t* __restrict__ unsafe_list,
                                                       const float4* __restrict__ setup,
                                                       const uint2* __restrict__ binrect,
                                                       const uint32_t* __restrict__ poff, uint32_t* __restrict__ keys,
                                                       uint32_t* __restrict__ vals, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t nu = (uint32_t)flags->n_unsafe_list;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t k = warp; k < nu; k += nwarps) {
        const uint32_t t = unsafe_list[k];
        const uint2 br = binrect[t];
        uint32_t c = 0;
        ext_bins(P, setup, br, t, lane, [&](uint32_t) { ++c; });
        const uint32_t inc = warp_inclusive_scan(c);
        uint32_t o = poff[t] + rect_count(br) + (inc - c);
        ext_bins(P, setup, br, t, lane, [&](uint32_t b) {
            keys[o] = b;
            vals[o] = t;
            ++o;
        });
    }
}

// ------------------------------------------------------------ radix sort
// Per block and digit value: the number of the block's items with that digit
// (digit-major layout hist[d * nblocks + block]).
__global__ void __launch_bounds__(RADIX_THREADS) radix_hist_kernel(const uint32_t* __restrict__ keys,
                                                                   const uint32_t* __restrict__ count_ptr,
                                                                   uint32_t shift, uint32_t nblocks,
                                                                   uint32_t* __restrict__ hist,
                                                                   const DeviceFlags* flags) {
    __shared__ uint32_t h[256];
    const uint32_t n = flags->poison ? 0u : *count_ptr;
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * RADIX_TILE;
    for (uint32_t i = threadIdx.x; i < RADIX_TILE; i += RADIX_THREADS) {
        const uint32_t j = base + i;
        if (j < n) atomicAdd(&h[(keys[j] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: items keep their order among equal digits.  The block's
// tile is processed in rounds of 256 consecutive items (one per thread); an
// item's rank is the count of equal digits before it in earlier rounds
// (run[]), in earlier warps of this round (wc[][]), and in earlier lanes of
// its warp (match-any mask).
__global__ void __launch_bounds__(RADIX_THREADS) radix_scatter_kernel(const uint32_t* __restrict__ keys_in,
                                                                      const uint32_t* __restrict__ vals_in,
                                                                      const uint32_t* __restrict__ count_ptr,
                                                                      uint32_t shift, uint32_t nblocks,
                                                                      const uint32_t* __restrict__ hist_off,
                                                                      uint32_t* __restrict__ keys_out,
                                                                      uint32_t* __restrict__ vals_out,
                                                                      const DeviceFlags* flags) {
    __shared__ uint32_t run[256];
    __shared__ uint32_t wc[RADIX_THREADS / 32][256];
    const uint32_t n = flags->poison ? 0u : *count_ptr;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    run[threadIdx.x] = hist_off[threadIdx.x * nblocks + blockIdx.x];
    const uint32_t base = blockIdx.x * RADIX_TILE;
    for (uint32_t r = 0; r < RADIX_ITEMS; ++r) {
        for (uint32_t w = 0; w < RADIX_THREADS / 32; ++w) wc[w][threadIdx.x] = 0;
        __syncthreads();
        const uint32_t j = base + r * RADIX_THREADS + threadIdx.x;
        const bool valid = j < n;
        uint32_t key = 0, val = 0, d = 256;   // 256: no digit (invalid item)
        if (valid) {
            key = keys_in[j];
            val = vals_in[j];
            d = (key >> shift) & 255u;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = __popc(peers & ((1u << lane) - 1u));
        if (valid && before == 0) wc[wid][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = run[d] + before;
            for (uint32_t w = 0; w < wid; ++w) pos += wc[w][d];
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
        uint32_t tot = 0;
        for (uint32_t w = 0; w < RADIX_THREADS / 32; ++w) tot += wc[w][threadIdx.x];
        run[threadIdx.x] += tot;
        __syncthreads();
    }
}

// [begin, end) of every bin from the sorted keys (ranges[] zeroed before)
__global__ void bin_range_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ count_ptr,
                                 uint32_t* __restrict__ ranges, const DeviceFlags* flags) {
    const uint32_t n = flags->poison ? 0u : *count_ptr;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = keys[i];
    if (i == 0 || keys[i - 1] != k) ranges[2 * (size_t)k] = i;
    if (i + 1 == n || keys[i + 1] != k) ranges[2 * (size_t)k + 1] = i + 1;
}

// ---------------------------------------------------------------- launch
uint32_t radix_blocks(uint64_t cap) { return (uint32_t)((cap + RADIX_TILE - 1) / RADIX_TILE); }

uint32_t* launch_bins(const DrawParams& P, const uint2* binrect, const float4* setup, const uint32_t* unsafe_list,
                      const BinBuffers& B, DeviceFlags* flags, cudaStream_t st) {
    const uint32_t n_host = P.n_raster_host;
    const uint32_t n = n_host ? n_host : P.gen_tri_cap;   // launch bound; the device count is used inside
    const uint32_t n_bins = P.bins_x * P.bins_y;
    const dim3 blk(256), grd((n + 256) / 256);
    cudaMemsetAsync(B.pcount, 0, ((size_t)n + 1) * 4, st);
    prim_count_kernel<<<grd, blk, 0, st>>>(n_host, n, binrect, B.pcount, flags);
    ext_count_kernel<<<resident_grid(ext_count_kernel, 256, 4), 256, 0, st>>>(P, unsafe_list, setup, binrect,
                                                                             B.pcount, flags);
    exclusive_scan<uint32_t>(B.pcount, n + 1, B.poff, B.scan_tmp, st);
    check_pairs_kernel<<<1, 1, 0, st>>>(n, B.poff, B.cap, P.draw_id, flags);
    prim_emit_kernel<<<grd, blk, 0, st>>>(P, n_host, n, binrect, B.poff, B.keys[0], B.vals[0], flags);
    ext_emit_kernel<<<resident_grid(ext_emit_kernel, 256, 4), 256, 0, st>>>(P, unsafe_list, setup, binrect, B.poff,
                                                                           B.keys[0], B.vals[0], flags);
    // radix passes over the bin id bits; the pair count lives at poff[n]
    uint32_t bits = 1;
    while ((1ull << bits) < n_bins) ++bits;
    const uint32_t passes = (bits + 7) / 8;
    const uint32_t nblocks = radix_blocks(B.cap);
    const uint32_t* count_ptr = B.poff + n;
    int cur = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        radix_hist_kernel<<<nblocks, RADIX_THREADS, 0, st>>>(B.keys[cur], count_ptr, 8 * p, nblocks, B.hist, flags);
        exclusive_scan<uint32_t>(B.hist, 256 * nblocks, B.hist_off, B.scan_tmp, st);
        radix_scatter_kernel<<<nblocks, RADIX_THREADS, 0, st>>>(B.keys[cur], B.vals[cur], count_ptr, 8 * p, nblocks,
                                                                B.hist_off, B.keys[cur ^ 1], B.vals[cur ^ 1], flags);
        cur ^= 1;
    }
    cudaMemsetAsync(B.ranges, 0, (size_t)n_bins * 8, st);
    bin_range_kernel<<<(uint32_t)((B.cap + 255) / 256), 256, 0, st>>>(B.keys[cur], count_ptr, B.ranges, flags);
    return B.vals[cur];
}

}  // namespace sr
