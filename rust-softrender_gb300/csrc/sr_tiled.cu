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
//   5. the bin raster kernel seeds its 1024 keys (from the global buffer where
//      the bitmap says so), walks its primitive list -- a cheap sign pre-test
//      on every bbox pixel, the reference's exact arithmetic on the pixels it
//      keeps, a shared-memory atomicMax of the key -- and writes each pixel's
//      winner (the key's low word) to the bin's 1024 slots;
//   6. the bin resolve kernel shades every pixel with a winner: start depth,
//      the winner's barycentrics, varyings, shading, one colour and depth
//      write.
// Per pixel, global memory sees the framebuffer and one 32-bit winner slot
// written and read once (and the rare extension keys); no global atomics are
// taken per fragment.
#include "sr_internal.cuh"
#include "sr_scan.cuh"
#include "sr_shade.cuh"
#include "sr_opaque.cuh"
#include "sr_setup.cuh"
#include "sr_binraster.cuh"

namespace sr {

// Exclusive scans, in one CTA, of the n bins' primitive counts (list offsets)
// and of their work items: ceil(count / TL_CHUNK) chunks per bin, one for a
// bin with only extension keys, none for an empty bin.  4096 bins at a time:
// coalesced loads into shared memory, each thread scans 4 consecutive bins,
// a CTA-wide scan of the thread sums, coalesced stores.  off[n] and
// chunk_off[n] are the totals.  A draw whose lists outgrow the entry buffer
// (the total summed in 64 bits) poisons the pipeline: sr_sync grows the
// buffer and replays.
constexpr uint32_t BS_TILE = 4096;
__device__ __forceinline__ uint32_t bs_slot(uint32_t i) { return i + (i >> 5); }
__global__ void __launch_bounds__(1024) bin_scan_kernel(const uint32_t* __restrict__ counts,
                                                        const uint32_t* __restrict__ bitmap, uint32_t n,
                                                        uint32_t* __restrict__ off, uint32_t* __restrict__ chunk_off,
                                                        uint64_t cap, uint32_t draw_id, DeviceFlags* flags) {
    __shared__ uint32_t te[BS_TILE + BS_TILE / 32], tc[BS_TILE + BS_TILE / 32];
    if (flags->poison) return;
    unsigned long long carry_e = 0;
    uint32_t carry_c = 0;
    for (uint32_t base = 0; base < n; base += BS_TILE) {
        const uint32_t m = min(BS_TILE, n - base);
        for (uint32_t i = threadIdx.x; i < BS_TILE; i += 1024) {
            const uint32_t b = base + i;
            const uint32_t e = i < m ? counts[b] : 0u;
            const bool ext = i < m && ((bitmap[b >> 5] >> (b & 31)) & 1u);
            te[bs_slot(i)] = e;
            tc[bs_slot(i)] = e ? (e + TL_CHUNK - 1) / TL_CHUNK : (ext ? 1u : 0u);
        }
        __syncthreads();
        constexpr uint32_t PER = BS_TILE / 1024;
        uint32_t ve[PER], vc[PER];
        unsigned long long se = 0;
        uint32_t sc = 0;
#pragma unroll
        for (uint32_t k = 0; k < PER; ++k) {
            ve[k] = te[bs_slot(threadIdx.x * PER + k)];
            vc[k] = tc[bs_slot(threadIdx.x * PER + k)];
            se += ve[k];
            sc += vc[k];
        }
        unsigned long long tot_e;
        uint32_t tot_c;
        unsigned long long xe = block_exclusive_scan<unsigned long long, 1024>(se, &tot_e) + carry_e;
        uint32_t xc = block_exclusive_scan<uint32_t, 1024>(sc, &tot_c) + carry_c;
#pragma unroll
        for (uint32_t k = 0; k < PER; ++k) {
            te[bs_slot(threadIdx.x * PER + k)] = (uint32_t)min(xe, 0xffffffffull);
            tc[bs_slot(threadIdx.x * PER + k)] = xc;
            xe += ve[k];
            xc += vc[k];
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < m; i += 1024) {
            off[base + i] = te[bs_slot(i)];
            chunk_off[base + i] = tc[bs_slot(i)];
        }
        carry_e += tot_e;
        carry_c += tot_c;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        off[n] = (uint32_t)min(carry_e, 0xffffffffull);
        chunk_off[n] = carry_c;
        if (carry_e > cap) {
            if (carry_e > flags->need_entries) flags->need_entries = carry_e;
            atomicOr(&flags->overflow_bits, (unsigned)OVF_ENTRIES);
            atomicOr(&flags->poison, 1u);
            atomicMin(&flags->poison_draw, draw_id);
        }
    }
}

// Writes every primitive into the list of each bin its clamped bbox meets.
// `cursor` (n_bins, zero) counts the slots taken per bin.  One-bin primitives
// of a warp that share a bin take their slots with one atomic.
__global__ void __launch_bounds__(256) bin_scatter_kernel(uint32_t n_host, uint32_t n_launch, uint32_t bins_x,
                                                          const uint2* __restrict__ binrect,
                                                          const uint32_t* __restrict__ bin_off, uint32_t n_bins,
                                                          uint32_t* __restrict__ cursor, uint32_t* __restrict__ entries,
                                                          DeviceFlags* flags) {
    if (flags->poison) return;   // also when the lists outgrow the entry buffer (bin_scan_kernel)
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
    const uint32_t nb = br.x != RECT_EMPTY ? (bx1 - bx0 + 1) * (by1 - by0 + 1) : 0u;
    if (single != 0xffffffffu) {
        entries[bin_off[single] + base + __popc(peers & ((1u << lane) - 1u))] = t;
    } else if (nb && nb <= 16) {
        for (uint32_t by = by0; by <= by1; ++by)
            for (uint32_t bx = bx0; bx <= bx1; ++bx) {
                const uint32_t b = by * bins_x + bx;
                entries[bin_off[b] + atomicAdd(cursor + b, 1u)] = t;
            }
    }
    // rectangles of more than 16 bins: the warp's lanes share each one's bins
    uint32_t big = __ballot_sync(0xffffffffu, nb > 16);
    while (big) {
        const uint32_t src = __ffs(big) - 1;
        big &= big - 1;
        const uint32_t sx0 = __shfl_sync(0xffffffffu, bx0, src), sy0 = __shfl_sync(0xffffffffu, by0, src);
        const uint32_t sw = __shfl_sync(0xffffffffu, bx1, src) - sx0 + 1;
        const uint32_t sn = __shfl_sync(0xffffffffu, nb, src), st = __shfl_sync(0xffffffffu, t, src);
        for (uint32_t i = lane; i < sn; i += 32) {
            const uint32_t b = (sy0 + i / sw) * bins_x + sx0 + i % sw;
            entries[bin_off[b] + atomicAdd(cursor + b, 1u)] = st;
        }
    }
}

// Persistent CTAs take work items (bin_scan_kernel numbers them: chunks of
// TL_CHUNK primitives of one bin's list) from a counter and reduce each with
// bin_item (sr_binraster.cuh): a bin in one item writes its winners to its
// slots of `gids` (seeded with its extension keys when it has some), a bin in
// several items merges its keys into `gkeys`, where bin_resolve_kernel finds
// them.
__global__ void __launch_bounds__(TL_THREADS, 6) bin_raster_kernel(
    DrawParams P, const float4* __restrict__ setup, const uint32_t* __restrict__ bin_off,
    const uint32_t* __restrict__ chunk_off, const uint32_t* __restrict__ entries, const uint8_t* __restrict__ stencil,
    uint32_t gate_with_stencil, unsigned long long* __restrict__ gkeys, const uint32_t* __restrict__ bitmap,
    uint32_t* __restrict__ gids, DeviceFlags* flags) {
    __shared__ BinSmem sm;
    __shared__ unsigned long long sfrags;
    __shared__ uint32_t sitem;
    if (flags->poison) return;
    const uint32_t n_bins = P.bins_x * P.bins_y;
    const uint32_t n_items = chunk_off[n_bins];
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t lane = threadIdx.x & 31;
    if (threadIdx.x == 0) sfrags = 0;
    unsigned long long frags = 0;
    for (;;) {
        if (threadIdx.x == 0) sitem = (uint32_t)atomicAdd(&flags->work_raster, 1ull);
        __syncthreads();   // the previous item is done with the shared arrays
        const uint32_t item = sitem;
        if (item >= n_items) break;
        // the item's bin: the last bin whose first item is <= item
        uint32_t b = 0;
        {
            uint32_t lo = 0, hi = n_bins;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (__ldg(chunk_off + mid) <= item) lo = mid; else hi = mid;
            }
            b = lo;
        }
        const uint32_t c_first = __ldg(chunk_off + b), n_chunks = __ldg(chunk_off + b + 1) - c_first;
        const bool whole = n_chunks == 1;   // the bin's only item: it owns the pixels' keys
        const uint32_t e_bin = __ldg(bin_off + b), cnt_bin = __ldg(bin_off + b + 1) - e_bin;
        const uint32_t c0 = (item - c_first) * TL_CHUNK;
        const uint32_t n = cnt_bin > c0 ? min(cnt_bin - c0, TL_CHUNK) : 0u;
        const bool ext = (bitmap[b >> 5] >> (b & 31)) & 1u;
        const uint32_t X0 = (b % P.bins_x) << TL_BIN_LOG2, Y0 = (b / P.bins_x) << TL_BIN_LOG2;
        bin_item(sm, P, X0, Y0, setup, entries + e_bin + c0, n, N, stencil, gate_with_stencil, whole, whole && ext,
                 gkeys, gids + ((size_t)b << (2 * TL_BIN_LOG2)), frags);
    }
    // one atomic per CTA for the fragment count
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if (lane == 0 && frags) atomicAdd(&sfrags, frags);
    __syncthreads();
    if (threadIdx.x == 0 && sfrags) atomicAdd(&flags->fragments, sfrags);
}

// One CTA per 32x32 bin: each pixel with a winner is resolved -- start depth,
// the winner's barycentrics, varyings, shading, one colour and depth write.
// A bin raster in one work item left its winners in `gids`; one raster in
// several left its keys in the global key buffer (read here, then zeroed).
// The bin's extension-key bit is cleared.
template <int FS, int FMT>
__global__ void __launch_bounds__(TL_THREADS, 5) bin_resolve_kernel(
    DrawParams P, sr_uniforms U, const float4* __restrict__ setup, const uint32_t* __restrict__ chunk_off,
    const uint32_t* __restrict__ gids, unsigned long long* __restrict__ gkeys, const uint32_t* __restrict__ vidx,
    const float* __restrict__ vary, const uint32_t* __restrict__ tex, void* __restrict__ color,
    float* __restrict__ depth, const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil,
    uint32_t* __restrict__ bitmap, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t b = blockIdx.x;
    const uint32_t n_chunks = chunk_off[b + 1] - chunk_off[b];
    if (n_chunks == 0) return;
    const bool ext = (bitmap[b >> 5] >> (b & 31)) & 1u;
    __syncthreads();   // every thread has read the bit before it is cleared
    if (ext && threadIdx.x == 0) atomicAnd(bitmap + (b >> 5), ~(1u << (b & 31)));
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t X0 = (b % P.bins_x) << TL_BIN_LOG2, Y0 = (b / P.bins_x) << TL_BIN_LOG2;
    const uint32_t* in = gids + ((size_t)b << (2 * TL_BIN_LOG2));
    for (uint32_t i = threadIdx.x; i < (1u << (2 * TL_BIN_LOG2)); i += TL_THREADS) {
        const uint32_t px = X0 + (i & 31), py = Y0 + (i >> TL_BIN_LOG2);
        uint32_t id;
        if (n_chunks == 1) {
            id = in[i];   // 0 also for every slot outside the frame
        } else {
            if (px >= P.W || py >= P.H) continue;
            const size_t gi = (size_t)py * P.W + px;
            const unsigned long long k = gkeys[gi];
            if (k) gkeys[gi] = 0;
            id = (uint32_t)(k & 0xffffffffull);
        }
        if (!id) continue;
        const float d0 = P.has_depth ? depth[(size_t)py * P.W + px] : 0.0f;
        resolve_winner<FS, FMT>(P, U, px, py, id, d0, N, setup, vidx, vary, tex, color, depth, stencil,
                                gate_with_stencil);
    }
}

template <int FS>
static void launch_bin_resolve_fs(const DrawParams& P, const sr_uniforms& U, const TiledArgs& A, uint32_t n_bins,
                                  cudaStream_t st) {
#define SR_BR(FMT) bin_resolve_kernel<FS, FMT><<<n_bins, TL_THREADS, 0, st>>>(P, U, A.setup, A.chunk_off, A.gids, \
        A.gkeys, A.vidx, A.vary, A.tex, A.color, A.depth, A.stencil, A.gate, A.bitmap, A.flags)
    if (P.color_format == SR_COLOR_RGBA32F) SR_BR(SR_COLOR_RGBA32F);
    else if (P.color_format == SR_COLOR_RGBA8) SR_BR(SR_COLOR_RGBA8);
    else SR_BR(SR_COLOR_NONE);
#undef SR_BR
}

void ext_direct_launch(const DrawParams& P, const uint32_t* unsafe_list, const float4* unsafe_rect,
                       const float4* setup, unsigned long long* gkeys, uint32_t* bitmap, const uint8_t* stencil,
                       uint32_t gate, DeviceFlags* flags, cudaStream_t st);

// launches: extension keys, bin scan, scatter, bin raster, bin resolve
// (setup, with the bin counts, is launched by the caller)
int launch_tiled(const DrawParams& P, const sr_uniforms& U, const TiledArgs& A, cudaStream_t st) {
    const uint32_t n_bins = P.bins_x * P.bins_y;
    ext_direct_launch(P, A.unsafe_list, A.unsafe_rect, A.setup, A.gkeys, A.bitmap, A.stencil, A.gate, A.flags, st);
    bin_scan_kernel<<<1, 1024, 0, st>>>(A.bin_counts, A.bitmap, n_bins, A.bin_off, A.chunk_off, A.entry_cap,
                                        P.draw_id, A.flags);
    const uint32_t n_launch = P.n_raster_host ? P.n_raster_host : P.gen_tri_cap;
    bin_scatter_kernel<<<(n_launch + 255) / 256 ? (n_launch + 255) / 256 : 1, 256, 0, st>>>(
        P.n_raster_host, n_launch, P.bins_x, A.binrect, A.bin_off, n_bins, A.cursor, A.entries, A.flags);
    bin_raster_kernel<<<resident_grid(bin_raster_kernel, TL_THREADS, 6), TL_THREADS, 0, st>>>(
        P, A.setup, A.bin_off, A.chunk_off, A.entries, A.stencil, A.gate, A.gkeys, A.bitmap, A.gids, A.flags);
    switch (P.fs) {
    case FS_BLINN_PHONG_DIR: launch_bin_resolve_fs<FS_BLINN_PHONG_DIR>(P, U, A, n_bins, st); break;
    case FS_TEXTURED_BLINN_PHONG: launch_bin_resolve_fs<FS_TEXTURED_BLINN_PHONG>(P, U, A, n_bins, st); break;
    case FS_VERTEX_COLOR: launch_bin_resolve_fs<FS_VERTEX_COLOR>(P, U, A, n_bins, st); break;
    case FS_ACES_LIGHTS: launch_bin_resolve_fs<FS_ACES_LIGHTS>(P, U, A, n_bins, st); break;
    default: launch_bin_resolve_fs<FS_CONSTANT_COLOR>(P, U, A, n_bins, st); break;
    }
    return 5;
}

}  // namespace sr
