// sr_batch.cu — batched rendering: many independent opaque draws (each into
// its own pipeline's framebuffer, meshes and resolutions of uneven sizes)
// rendered by one launch per stage instead of one set of launches per draw.
//
// Every stage is a persistent kernel (a fixed grid sized to the GPU) that
// pulls work items from the flattened (instance, item) space: vertices,
// primitives, 32x32 resolve blocks and 32x32 clear blocks.  An item's
// instance is found by binary search over per-instance exclusive prefix sums
// (once per warp where a warp's items are consecutive).  A cleared target is
// cleared after the raster passes, and only where no fragment landed: resolve
// writes the clear values into the rest of the blocks it visits.  Per-draw
// results are identical to sr_render's: the per-primitive, per-pixel and
// per-block device code is the same (sr_vertex.cuh, sr_setup.cuh,
// sr_opaque.cuh), only the indexing differs; each instance keeps its own
// primitive numbering, key buffer and touched-block bitmap (its pipeline's).
//
// The launch sequence reads every size from a device-resident table, so one
// CUDA graph serves every batch with the same table capacity and launch
// configuration; the host fills a pinned table per batch and replays.  The
// launch configuration (primitives per warp, large-primitive threshold,
// raster CTAs per SM) is picked per batch size class by measuring the
// candidates once (results do not depend on it: the opaque reduction is
// order independent).
#include <algorithm>
#include <cstdlib>
#include <map>
#include <unordered_set>
#include <vector>

#include "sr_host.h"
#include "sr_opaque.cuh"
#include "sr_scan.cuh"
#include "sr_setup.cuh"
#include "sr_vertex.cuh"
#include "sr_binraster.cuh"

namespace sr {

// One draw of a batch (device table entry).
struct BInst {
    DrawParams P;                 // as sr_render derives it; P.n_raster_host = triangle count
    VpMatrix vpm;                 // viewport matrix of ClipVertex::normalize
    const float* planes;
    const uint32_t* indices;
    const uint32_t* tex;
    void* color;
    float* depth;
    unsigned long long* gkeys;    // the target pipeline's per-pixel key buffer
    uint32_t* bitmap;             // the target pipeline's touched-block bitmap
    uint32_t n_pad;               // plane stride of the mesh
    uint32_t vbase, tbase;        // first batch vertex slot / first batch primitive
    uint32_t clear;               // clear colour and depth before drawing
    uint4 clear_color;            // colour clear pattern (one pixel of RGBA32F, four of RGBA8)
    uint32_t mx, my;              // division magics of the semantic tile size
};

// Device table layout for a capacity of NB draws (all offsets 256-aligned).
struct BTables {
    const uint32_t* n;            // number of draws in this batch
    const BInst* inst;
    const sr_uniforms* U;
    const uint32_t* qbase;        // exclusive prefix of vertices            (NB + 1)
    const uint32_t* tbase;        // exclusive prefix of primitives          (NB + 1)
    const uint32_t* bbase;        // exclusive prefix of 32x32 resolve blocks (NB + 1)
    const uint32_t* cbase;        // exclusive prefix of 32x32 clear blocks  (NB + 1)
};

constexpr uint32_t BIG_CHUNK = 4096;     // bbox pixels per work item of a large primitive
// Work-queue counters of a batch (device array of 32 u64):
//   [fs * 3 + format]  resolve launch of that (fragment shader, colour format)
constexpr int Q_TOUCHED = 16;            // entries on the touched-block list
constexpr int Q_BIG = 17;                // large primitives (count << 40 | chunks)
constexpr int Q_BIGCHUNK = 18;           // next large-primitive chunk to hand out
constexpr int N_QUEUES = 32;

// The touched-block list is built after the raster passes (which only set
// bitmap bits with fire-and-forget atomics): one thread per (draw, block).
__global__ void __launch_bounds__(256) batch_collect_kernel(BTables T, unsigned long long* __restrict__ tlist,
                                                            unsigned long long* __restrict__ queues);

// Largest i in [0, n) with base[i] <= j (base[0] = 0, j < base[n]).
__device__ __forceinline__ uint32_t owner_of(const uint32_t* __restrict__ base, uint32_t n, uint32_t j) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(base + mid) <= j) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Owner of item j when the owner of an item j0 <= j is known to be i0 (the
// items of a warp are consecutive, so this is usually 0 or 1 step).
__device__ __forceinline__ uint32_t owner_from(const uint32_t* __restrict__ base, uint32_t n, uint32_t i0, uint32_t j) {
    uint32_t i = i0;
    while (i + 1 < n && __ldg(base + i + 1) <= j) ++i;
    return i;
}

// ---------------------------------------------------------------- clear
// The clears of the batch's cleared targets, deferred until after the raster
// passes: one warp per 32x32 block of a cleared target.  A block with
// fragments (its bitmap bit set) is left to resolve, which writes every pixel
// of it (the winner's shade or the clear values).
__global__ void __launch_bounds__(256) batch_clear_kernel(BTables T) {
    const uint32_t n = *T.n;
    const uint32_t total = __ldg(T.cbase + n);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < total; j += warps) {
        const uint32_t i = owner_of(T.cbase, n, j);
        const BInst& I = T.inst[i];
        const uint32_t b = j - __ldg(T.cbase + i);
        if ((I.bitmap[b >> 5] >> (b & 31)) & 1u) continue;
        const uint32_t W = I.P.W, H = I.P.H;
        const uint32_t bx = (W + 31) >> 5;
        const uint32_t x = ((b % bx) << 5) + lane, y0 = (b / bx) << 5;
        if (x >= W) continue;
        const uint32_t y1 = min(y0 + 32u, H);
        const uint4 cv = I.clear_color;
        for (uint32_t y = y0; y < y1; ++y) {
            const size_t gi = (size_t)y * W + x;
            if (I.P.color_format == SR_COLOR_RGBA32F) reinterpret_cast<uint4*>(I.color)[gi] = cv;
            else if (I.P.color_format == SR_COLOR_RGBA8) reinterpret_cast<uint32_t*>(I.color)[gi] = cv.x;
            if (I.P.has_depth) I.depth[gi] = F32_LOWEST;
        }
    }
}

// ---------------------------------------------------------------- vertex
__global__ void __launch_bounds__(128) batch_vertex_kernel(BTables T, float4* __restrict__ scr4,
                                                           float* __restrict__ vary) {
    const uint32_t n = *T.n;
    const uint32_t total = __ldg(T.qbase + n);
    const uint32_t lane = threadIdx.x & 31;
    // a warp takes 32 consecutive vertices per round; lane 0 finds the draw
    for (uint32_t jw = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); jw < total; jw += gridDim.x * blockDim.x) {
        uint32_t i0 = 0;
        if (lane == 0) i0 = owner_of(T.qbase, n, jw);
        i0 = __shfl_sync(0xffffffffu, i0, 0);
        const uint32_t j = jw + lane;
        if (j >= total) continue;
        const uint32_t i = owner_from(T.qbase, n, i0, j);
        const BInst& I = T.inst[i];
        const uint32_t v = j - __ldg(T.qbase + i);
        float4* s4 = scr4 + I.vbase;
        float* vy = vary + (size_t)I.vbase * VSTRIDE;
        switch (I.P.vs) {
        case VS_MVP_POS_NRM: vertex_one<VS_MVP_POS_NRM>(v, I.P.n_verts, I.n_pad, T.U[i], I.vpm, I.planes, nullptr, s4, vy); break;
        case VS_MVP_POS_NRM_UV: vertex_one<VS_MVP_POS_NRM_UV>(v, I.P.n_verts, I.n_pad, T.U[i], I.vpm, I.planes, nullptr, s4, vy); break;
        case VS_CLIP_COLOR: vertex_one<VS_CLIP_COLOR>(v, I.P.n_verts, I.n_pad, T.U[i], I.vpm, I.planes, nullptr, s4, vy); break;
        default: vertex_one<VS_CLIP_RGBA8>(v, I.P.n_verts, I.n_pad, T.U[i], I.vpm, I.planes, nullptr, s4, vy); break;
        }
    }
}

// ---------------------------------------------------------------- setup
// The opaque branch of setup_kernel (sr_setup.cu) per batch primitive g:
// cull, det, bbox, safety class, record, bbox pixel count, unsafe list.  A
// primitive whose bbox meets at most `bin_limit` of its target's 32x32 bins
// and `big_threshold` pixels is listed in those bins (its bin rectangle, and
// a count per (draw, bin)); a larger one goes to the large-primitive list,
// whose chunks batch_raster_big_kernel reduces through the key buffer.
__global__ void __launch_bounds__(256) batch_setup_kernel(BTables T, const float4* __restrict__ scr4,
                                                          float4* __restrict__ setup,
                                                          unsigned long long* __restrict__ area,
                                                          uint32_t* __restrict__ unsafe_list, uint2* __restrict__ binrect,
                                                          uint32_t* __restrict__ bin_cnt, uint32_t bin_limit,
                                                          uint32_t big_threshold, uint32_t* __restrict__ big_list,
                                                          uint32_t* __restrict__ big_base,
                                                          unsigned long long* __restrict__ queues, DeviceFlags* flags) {
    const uint32_t n = *T.n;
    const uint32_t total = __ldg(T.tbase + n);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t n_raster = 0, n_unsafe = 0, nan_cnt = 0;
    // a warp takes 32 consecutive primitives per round: lane 0 finds the draw
    // of the first, the others step forward from it
    for (uint32_t gw = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); gw < total; gw += stride) {
        uint32_t i0 = 0;
        if (lane == 0) i0 = owner_of(T.tbase, n, gw);
        i0 = __shfl_sync(0xffffffffu, i0, 0);
        const uint32_t g = gw + lane;
        uint32_t single_fb = 0xffffffffu;   // the (draw, bin) of a one-bin listed primitive
        if (g < total) {
            const uint32_t i = owner_from(T.tbase, n, i0, g);
            const BInst& I = T.inst[i];
            const DrawParams& P = I.P;
            const uint32_t t = g - I.tbase;
            uint32_t ia, ib, ic;
            tri_slots(t, I.indices, ia, ib, ic);
            const bool bad = ia >= P.n_verts || ib >= P.n_verts || ic >= P.n_verts;
            if (bad) { atomicOr(&flags->bad_index, 1u); ia = ib = ic = 0; }
            const float4* sv = scr4 + I.vbase;
            const float4 s0 = __ldg(sv + ia), s1 = __ldg(sv + ib), s2 = __ldg(sv + ic);
            const float x1 = s0.x, y1 = s0.y, x2 = s1.x, y2 = s1.y, x3 = s2.x, y3 = s2.y;
            bool culled = false;
            if (P.cull) {
                const float ar = x1 * y2 + x2 * y3 + x3 * y1 - x2 * y1 - x3 * y2 - x1 * y3;
                const bool neg = !isnan(ar) && signbit(ar);
                culled = (neg ? 1u : 2u) == P.cull;
            }
            culled = culled || bad;
            area[g] = 0;
            binrect[g] = make_uint2(RECT_EMPTY, RECT_EMPTY);
            setup[4 * (size_t)g + 2] = make_float4(0.0f, 0.0f, __uint_as_float(0u), 0.0f);
            if (!culled) {
                const float det = (y2 - y3) * (x1 - x3) + (x3 - x2) * (y1 - y3);
                const float mnx = sr_min(sr_min(x1, x2), x3), mny = sr_min(sr_min(y1, y2), y3);
                const float mxx = sr_max(sr_max(x1, x2), x3), mxy = sr_max(sr_max(y1, y2), y3);
                if (isnan(mnx) || isnan(mny)) {
                    ++nan_cnt;
                } else {
                    const int W = (int)P.W, H = (int)P.H;
                    const int ix0 = floor_sat(mnx, -1, W), ix1 = floor_sat(mxx, -1, W);
                    const int iy0 = floor_sat(mny, -1, H), iy1 = floor_sat(mxy, -1, H);
                    const bool no_frag = det == 0.0f || isnan(det) || (s0.z >= 0.0f && s1.z >= 0.0f && s2.z >= 0.0f);
                    if (!no_frag) {
                        const bool safe = !P.force_unsafe &&
                                          inflated_region(x1, y1, x2, y2, x3, y3, det, P.W, P.H, ix0, iy0, ix1, iy1);
                        const int qx0 = max(ix0, 0), qy0 = max(iy0, 0), qx1 = min(ix1, W - 1), qy1 = min(iy1, H - 1);
                        const bool b_in = qx0 <= qx1 && qy0 <= qy1;
                        if (b_in || !safe) {
                            float4* rr = setup + 4 * (size_t)g;
                            rr[0] = make_float4(y2 - y3, x3 - x2, y3 - y1, x1 - x3);
                            rr[1] = make_float4(x3, y3, det, s0.z);
                            rr[2] = make_float4(s1.z, s2.z, __uint_as_float(REC_RASTER | (safe ? 0u : REC_UNSAFE)),
                                                det_sign(det));
                            rr[3] = make_float4(__int_as_float(ix0), __int_as_float(iy0), __int_as_float(ix1),
                                                __int_as_float(iy1));
                            ++n_raster;
                            if (!safe) {
                                ++n_unsafe;
                                unsafe_list[atomicAdd(&flags->n_unsafe_list, 1ull)] = g;
                            }
                            const unsigned long long at =
                                b_in ? (unsigned long long)(qx1 - qx0 + 1) * (unsigned long long)(qy1 - qy0 + 1) : 0ull;
                            area[g] = at;
                            if (b_in) {
                                const uint32_t rx0 = (uint32_t)qx0 >> TL_BIN_LOG2, rx1 = (uint32_t)qx1 >> TL_BIN_LOG2;
                                const uint32_t ry0 = (uint32_t)qy0 >> TL_BIN_LOG2, ry1 = (uint32_t)qy1 >> TL_BIN_LOG2;
                                const uint32_t nb = (rx1 - rx0 + 1) * (ry1 - ry0 + 1);
                                if (nb <= bin_limit && at <= big_threshold) {
                                    binrect[g] = make_uint2(rx0 | (ry0 << 16), rx1 | (ry1 << 16));
                                    const uint32_t fb0 = __ldg(T.bbase + i);
                                    if (nb == 1) {
                                        single_fb = fb0 + ry0 * P.bins_x + rx0;   // counted per warp below
                                    } else {
                                        for (uint32_t by = ry0; by <= ry1; ++by)
                                            for (uint32_t bx = rx0; bx <= rx1; ++bx)
                                                atomicAdd(bin_cnt + fb0 + by * P.bins_x + bx, 1u);
                                    }
                                } else {
                                    // one packed counter keeps list order and chunk offsets consistent
                                    const unsigned long long nch = (at + BIG_CHUNK - 1) / BIG_CHUNK;
                                    const unsigned long long old = atomicAdd(queues + Q_BIG, (1ull << 40) | nch);
                                    big_list[old >> 40] = g;
                                    big_base[old >> 40] = (uint32_t)(old & ((1ull << 40) - 1));
                                    // the count has 24 bits: past them the batch reports SR_EOVERFLOW
                                    if ((old >> 40) >= (1ull << 24) - 1) atomicOr(&flags->overflow_bits, 1u);
                                }
                            }
                        }
                    }
                }
            }
        }
        // one atomic per warp and bin for the one-bin primitives (a mesh's
        // consecutive primitives mostly share bins)
        const uint32_t peers = __match_any_sync(0xffffffffu, single_fb);
        if (single_fb != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(bin_cnt + single_fb, (uint32_t)__popc(peers));
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_raster += __shfl_down_sync(0xffffffffu, n_raster, o);
        n_unsafe += __shfl_down_sync(0xffffffffu, n_unsafe, o);
        nan_cnt += __shfl_down_sync(0xffffffffu, nan_cnt, o);
    }
    if (lane == 0) {
        if (n_raster) atomicAdd(&flags->triangles_raster, (unsigned long long)n_raster);
        if (n_unsafe) atomicAdd(&flags->unsafe, (unsigned long long)n_unsafe);
        if (nan_cnt) { atomicAdd(&flags->nan_bbox, nan_cnt); atomicAdd(&flags->nan_total, nan_cnt); }
    }
}

// ---------------------------------------------------------------- bins
// The listed primitives are reduced per (draw, 32x32 bin) as in sr_render's
// binned path (sr_tiled.cu, sr_binraster.cuh): the draws' bins are numbered
// consecutively (bin j of draw i is T.bbase[i] + j), each bin's count becomes
// its list offset and its number of work items (chunks of TL_CHUNK
// primitives) in one scan of packed u64 values (entries << 32 | items), the
// primitives scatter into the lists, and persistent CTAs reduce the work
// items in shared memory.  The winners land in each target's per-pixel key
// buffer, where the large primitives (batch_raster_big_kernel) and the
// extension fragments (batch_ext_kernel) already left theirs, and every bin
// with keys is marked in the target's bitmap, so batch_collect_kernel,
// batch_clear_kernel and batch_resolve_kernel work on them unchanged.

// Packed count of bin j (< cap): entries << 32 | work items; zero past the
// batch's bins.  The counts are reset for the next batch here (and the
// slot cursors by the bin raster), so a batch needs no clearing launches.
__global__ void __launch_bounds__(256) batch_bin_pack_kernel(BTables T, uint32_t cap, uint32_t* __restrict__ bin_cnt,
                                                             unsigned long long* __restrict__ packed) {
    const uint32_t total = __ldg(T.bbase + *T.n);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < cap; j += gridDim.x * blockDim.x) {
        unsigned long long v = 0;
        if (j < total) {
            const uint32_t e = bin_cnt[j];
            if (e) bin_cnt[j] = 0;
            v = ((unsigned long long)e << 32) | ((e + TL_CHUNK - 1) / TL_CHUNK);
        }
        packed[j] = v;
    }
}

// The work-item table: the (draw, bin) of every work item, from the scanned
// item offsets.
__global__ void __launch_bounds__(256) batch_bin_items_kernel(BTables T, const unsigned long long* __restrict__ off,
                                                              uint32_t* __restrict__ item_bin, uint64_t item_cap) {
    const uint32_t total = __ldg(T.bbase + *T.n);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += gridDim.x * blockDim.x) {
        const uint32_t c0 = (uint32_t)(off[j] & 0xffffffffull), c1 = (uint32_t)(off[j + 1] & 0xffffffffull);
        for (uint32_t k = c0; k < c1 && k < item_cap; ++k) item_bin[k] = j;
    }
}

// Every listed primitive into the list of each bin of its rectangle (draw-
// local primitive numbers; order within a list is free).  `cursor` (cap
// entries, zero) counts the slots taken per bin.
__global__ void __launch_bounds__(256) batch_bin_scatter_kernel(BTables T, const uint2* __restrict__ binrect,
                                                                const unsigned long long* __restrict__ off,
                                                                uint32_t* __restrict__ cursor,
                                                                uint32_t* __restrict__ entries, uint64_t entry_cap,
                                                                DeviceFlags* flags) {
    const uint32_t n = *T.n;
    const uint32_t total = __ldg(T.tbase + n);
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t gw = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); gw < total; gw += gridDim.x * blockDim.x) {
        uint32_t i0 = 0;
        if (lane == 0) i0 = owner_of(T.tbase, n, gw);
        i0 = __shfl_sync(0xffffffffu, i0, 0);
        const uint32_t g = gw + lane;
        uint32_t single = 0xffffffffu, t = 0;
        uint2 br = make_uint2(RECT_EMPTY, RECT_EMPTY);
        uint32_t fb0 = 0, bins_x = 0;
        if (g < total) {
            br = binrect[g];
            if (br.x != RECT_EMPTY) {
                const uint32_t i = owner_from(T.tbase, n, i0, g);
                fb0 = __ldg(T.bbase + i);
                bins_x = T.inst[i].P.bins_x;
                t = g - __ldg(T.tbase + i);
                if (br.x == br.y) single = fb0 + (br.x >> 16) * bins_x + (br.x & 0xffffu);
            }
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, single);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (single != 0xffffffffu && lane == leader) base = atomicAdd(cursor + single, (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        // (the lists were sized on the host; a slot past them is reported
        // as SR_EOVERFLOW rather than written)
        if (single != 0xffffffffu) {
            const uint64_t k = (off[single] >> 32) + base + __popc(peers & ((1u << lane) - 1u));
            if (k < entry_cap) entries[k] = t;
            else atomicOr(&flags->overflow_bits, 1u);
        } else if (br.x != RECT_EMPTY) {
            for (uint32_t by = br.x >> 16; by <= (br.y >> 16); ++by)
                for (uint32_t bx = br.x & 0xffffu; bx <= (br.y & 0xffffu); ++bx) {
                    const uint32_t fb = fb0 + by * bins_x + bx;
                    const uint64_t k = (off[fb] >> 32) + atomicAdd(cursor + fb, 1u);
                    if (k < entry_cap) entries[k] = t;
                    else atomicOr(&flags->overflow_bits, 1u);
                }
        }
    }
}

// Persistent CTAs take work items from a counter: the work-item table gives
// the item's (draw, bin), and bin_item reduces it.  A bin in one item starts
// from the keys already in the key buffer when its bitmap bit says so, and
// stores its non-zero keys there; a bin in several items merges them with
// atomicMax.  Each item marks its bin in the bitmap.  The next item is fetched
// while the current one is reduced.
__global__ void __launch_bounds__(TL_THREADS, 6) batch_bin_raster_kernel(
    BTables T, const float4* __restrict__ setup, const unsigned long long* __restrict__ off, uint32_t cap,
    const uint32_t* __restrict__ item_bin, uint64_t item_cap, const uint32_t* __restrict__ entries,
    uint64_t entry_cap, uint32_t* __restrict__ cursor, DeviceFlags* flags) {
    __shared__ BinSmem sm;
    __shared__ DrawParams sP;
    __shared__ uint4 snext[2];   // per parity: item, (draw, bin), draw, 0
    __shared__ ulonglong2 soff[2];   // per parity: the bin's packed offsets and the next bin's
    __shared__ bool sext;
    __shared__ unsigned long long sfrags;
    const uint32_t n = *T.n;
    const uint32_t n_items = (uint32_t)(off[cap] & 0xffffffffull);
    auto fetch = [&](uint32_t item, uint32_t par) {
        uint4 v = make_uint4(item, 0, 0, 0);
        ulonglong2 o = make_ulonglong2(0, 0);
        if (item < n_items && item < item_cap) {
            const uint32_t fb = min(__ldg(item_bin + item), cap - 1);
            v = make_uint4(item, fb, owner_of(T.bbase, n, fb), 0);
            o = make_ulonglong2(off[fb], off[fb + 1]);
        }
        snext[par] = v;
        soff[par] = o;
    };
    if (threadIdx.x == 0) {
        sfrags = 0;
        fetch((uint32_t)min(atomicAdd(&flags->work_raster, 1ull), 0xffffffffull), 0);
    }
    __syncthreads();
    unsigned long long frags = 0;
    for (uint32_t par = 0;; par ^= 1u) {
        const uint4 it = snext[par];
        const ulonglong2 oo = soff[par];
        const uint32_t item = it.x;
        if (item >= n_items) break;
        uint32_t nxt = 0;
        if (threadIdx.x == 0) nxt = (uint32_t)min(atomicAdd(&flags->work_raster, 1ull), 0xffffffffull);
        const uint32_t fb = it.y, i = it.z;
        const BInst& I = T.inst[i];
        for (uint32_t k = threadIdx.x; k < sizeof(DrawParams) / 4; k += blockDim.x)
            reinterpret_cast<uint32_t*>(&sP)[k] = reinterpret_cast<const uint32_t*>(&I.P)[k];
        const uint32_t b = fb - __ldg(T.bbase + i);
        const uint32_t e_bin = (uint32_t)(oo.x >> 32), cnt_bin = (uint32_t)(oo.y >> 32) - e_bin;
        const uint32_t c_first = (uint32_t)(oo.x & 0xffffffffull), n_chunks = (uint32_t)(oo.y & 0xffffffffull) - c_first;
        const uint32_t c0 = (item - c_first) * TL_CHUNK;
        uint32_t cnt = cnt_bin > c0 ? min(cnt_bin - c0, TL_CHUNK) : 0u;
        if ((uint64_t)e_bin + c0 + cnt > entry_cap) cnt = 0;   // flagged by the scatter
        const bool whole = n_chunks == 1;
        if (threadIdx.x == 0) {
            if (c0 == 0) cursor[fb] = 0;   // the bin's scatter is done: reset for the next batch
            const uint32_t word = I.bitmap[b >> 5], bit = 1u << (b & 31);
            sext = (word & bit) != 0;   // keys of large primitives or extension fragments
            if (!(word & bit)) atomicOr(I.bitmap + (b >> 5), bit);
        }
        __syncthreads();
        const bool seed = whole && sext;
        const uint32_t X0 = (b % sP.bins_x) << TL_BIN_LOG2, Y0 = (b / sP.bins_x) << TL_BIN_LOG2;
        bin_item(sm, sP, X0, Y0, setup + 4 * (size_t)I.tbase, entries + e_bin + c0, cnt, sP.n_raster_host, nullptr,
                 0u, whole, seed, I.gkeys, nullptr, frags);
        if (threadIdx.x == 0) fetch(nxt, par ^ 1u);
        __syncthreads();   // the next item is known, and this one is done with the shared arrays
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&sfrags, frags);
    __syncthreads();
    if (threadIdx.x == 0 && sfrags) atomicAdd(&flags->fragments, sfrags);
}

// raster_big_kernel over the batch's large primitives, split into chunks of
// BIG_CHUNK bbox pixels taken from a work queue (a huge primitive spreads
// over many CTAs).
__global__ void __launch_bounds__(256) batch_raster_big_kernel(BTables T, const float4* __restrict__ setup,
                                                               const unsigned long long* __restrict__ area,
                                                               const uint32_t* __restrict__ big_list,
                                                               const uint32_t* __restrict__ big_base,
                                                               unsigned long long* __restrict__ tlist,
                                                               unsigned long long* __restrict__ queues,
                                                               DeviceFlags* flags) {
    __shared__ uint32_t s_item;
    const uint32_t n = *T.n;
    const unsigned long long packed = queues[Q_BIG];
    const uint32_t nb = (uint32_t)(packed >> 40);
    const uint32_t total = (uint32_t)min(packed & ((1ull << 40) - 1), 0xffffffffull);
    unsigned long long frags = 0;
    for (;;) {
        if (threadIdx.x == 0) s_item = (uint32_t)min(atomicAdd(queues + Q_BIGCHUNK, 1ull), 0xffffffffull);
        __syncthreads();
        const uint32_t j = s_item;
        __syncthreads();
        if (j >= total) break;
        // the large primitive owning chunk j: largest k with big_base[k] <= j
        uint32_t lo = 0, hi = nb - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (big_base[mid] <= j) lo = mid; else hi = mid - 1;
        }
        const uint32_t g = big_list[lo];
        const uint32_t c = j - big_base[lo];
        const uint32_t i = owner_of(T.tbase, n, g);
        const BInst& I = T.inst[i];
        const float4* r = setup + 4 * (size_t)g;
        const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
        const uint32_t W = I.P.W, H = I.P.H;
        const uint32_t x0 = (uint32_t)max(__float_as_int(r3.x), 0);
        const uint32_t y0 = (uint32_t)max(__float_as_int(r3.y), 0);
        const uint32_t x1 = (uint32_t)min(__float_as_int(r3.z), (int)W - 1);
        const uint32_t y1 = (uint32_t)min(__float_as_int(r3.w), (int)H - 1);
        const uint32_t w = x1 - x0 + 1;
        if (c == 0) {   // the first chunk marks the whole bbox
            const uint32_t blocks_x = (W + 31) >> 5;
            const uint32_t bx0 = x0 >> TOUCH_LOG2, by0 = y0 >> TOUCH_LOG2;
            const uint32_t nbx = (x1 >> TOUCH_LOG2) - bx0 + 1, nby = (y1 >> TOUCH_LOG2) - by0 + 1;
            for (uint32_t q = threadIdx.x; q < nbx * nby; q += blockDim.x) {
                const uint32_t bb = (by0 + q / nbx) * blocks_x + bx0 + q % nbx, bit = 1u << (bb & 31);
                if (!(I.bitmap[bb >> 5] & bit)) atomicOr(I.bitmap + (bb >> 5), bit);
            }
        }
        const uint32_t sb = seam_bits(x0, y0, x1, y1, I.P);
        // bbox pixels of the chunk, row-major; each thread steps its (row,
        // column) by blockDim pixels instead of dividing per pixel
        const uint32_t at = (uint32_t)area[g];
        const uint32_t p0 = c * BIG_CHUNK;
        const uint32_t p1 = min(at, p0 + BIG_CHUNK);
        const uint32_t t = g - I.tbase;
        const uint32_t q0 = p0 + threadIdx.x;
        uint32_t row = q0 / w, col = q0 - row * w;
        const uint32_t drow = blockDim.x / w, dcol = blockDim.x - drow * w;
        for (uint32_t q = q0; q < p1; q += blockDim.x) {
            frag_emit(W, H, I.P.tile_w, I.P.tile_h, I.mx, I.my, sb, I.P.has_depth != 0, r0, r1, r2, t, x0 + col,
                      y0 + row, I.P.n_raster_host, I.gkeys, nullptr, 0u, 0u, 0u, frags);
            row += drow;
            col += dcol;
            if (col >= w) { col -= w; ++row; }
        }
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// ext_direct_kernel over the batch's unsafe primitives (one warp each).
__global__ void __launch_bounds__(256) batch_ext_kernel(BTables T, const float4* __restrict__ setup,
                                                        const uint32_t* __restrict__ unsafe_list,
                                                        unsigned long long* __restrict__ tlist,
                                                        unsigned long long* __restrict__ queues, DeviceFlags* flags) {
    const uint32_t n = *T.n;
    const uint32_t nu = (uint32_t)flags->n_unsafe_list;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long frags = 0;
    for (uint32_t k = warp; k < nu; k += nwarps) {
        const uint32_t g = unsafe_list[k];
        const BInst& I = T.inst[owner_of(T.tbase, n, g)];
        ext_prim(I.P, g - I.tbase, I.P.n_raster_host, setup + 4 * (size_t)I.tbase, I.gkeys, I.bitmap, nullptr, 0u,
                 lane, frags);
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// ---------------------------------------------------------------- collect
__global__ void __launch_bounds__(256) batch_collect_kernel(BTables T, unsigned long long* __restrict__ tlist,
                                                            unsigned long long* __restrict__ queues) {
    const uint32_t n = *T.n;
    const uint32_t total = __ldg(T.bbase + n);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (total + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t j = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool set = false;
        unsigned long long e = 0;
        if (j < total) {
            const uint32_t i = owner_of(T.bbase, n, j);
            const uint32_t b = j - __ldg(T.bbase + i);
            set = (T.inst[i].bitmap[b >> 5] >> (b & 31)) & 1u;
            e = ((unsigned long long)i << 32) | b;
        }
        const uint32_t m = __ballot_sync(0xffffffffu, set);
        if (!m) continue;
        unsigned long long base = 0;
        if (lane == __ffs(m) - 1) base = atomicAdd(queues + Q_TOUCHED, (unsigned long long)__popc(m));
        base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
        if (set) tlist[base + __popc(m & ((1u << lane) - 1u))] = e;
    }
}

// ---------------------------------------------------------------- resolve
// resolve_kernel over (draw, touched 32x32 block) items, one launch per
// (fragment shader, colour format) pair present in the batch; a launch skips
// the draws of other pairs.  CTAs take items from a work queue.
template <int FS, int FMT>
// 6 resident CTAs per SM (at most 40 registers) measured faster than the
// unconstrained 64 registers (4 CTAs)
__global__ void __launch_bounds__(256, 6) batch_resolve_kernel(BTables T, const float4* __restrict__ setup,
                                                            const float* __restrict__ vary,
                                                            const unsigned long long* __restrict__ tlist,
                                                            unsigned long long* __restrict__ queues, int qi) {
    __shared__ uint32_t s_item;
    const uint32_t total = (uint32_t)min(queues[Q_TOUCHED], 0xffffffffull);
    for (;;) {
        if (threadIdx.x == 0) s_item = (uint32_t)min(atomicAdd(queues + qi, 1ull), 0xffffffffull);
        __syncthreads();
        const uint32_t j = s_item;
        __syncthreads();
        if (j >= total) break;
        const unsigned long long e = tlist[j];
        const uint32_t i = (uint32_t)(e >> 32), b = (uint32_t)e;
        const BInst& I = T.inst[i];
        if (I.P.fs != FS || (int)I.P.color_format != FMT) continue;
        resolve_block<FS, FMT>(I.P, T.U[i], b, I.P.n_raster_host, setup + 4 * (size_t)I.tbase, I.indices,
                               vary + (size_t)I.vbase * VSTRIDE, I.tex, I.color, I.depth, nullptr, 0u, I.gkeys,
                               I.bitmap, I.clear != 0, I.clear_color);
    }
}

}  // namespace sr

// ================================================================== host
using namespace sr;

namespace {

struct BatchConfig {
    uint32_t G = 8;           // bins a listed primitive may cover (more: the large-primitive pass)
    uint32_t big = 8192;      // bbox pixels above which a primitive takes the large-primitive pass
    uint32_t ctas = 8;        // bin raster CTAs per SM (at most the kernel's resident count)
    bool operator==(const BatchConfig& o) const { return G == o.G && big == o.big && ctas == o.ctas; }
};

struct Layout {
    size_t off_n, off_inst, off_U, off_q, off_t, off_b, off_c, bytes;
};

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

Layout layout_for(uint32_t NB) {
    Layout L;
    L.off_n = 0;
    L.off_inst = 256;
    L.off_U = al256(L.off_inst + (size_t)NB * sizeof(BInst));
    L.off_q = al256(L.off_U + (size_t)NB * sizeof(sr_uniforms));
    L.off_t = al256(L.off_q + (size_t)(NB + 1) * 4);
    L.off_b = al256(L.off_t + (size_t)(NB + 1) * 4);
    L.off_c = al256(L.off_b + (size_t)(NB + 1) * 4);
    L.bytes = al256(L.off_c + (size_t)(NB + 1) * 4);
    return L;
}

uint32_t bucket_of(uint32_t n) {
    uint32_t b = 16;
    while (b < n) b <<= 1;
    return b;
}

int batch_min_varyings(int fs) {
    switch (fs) {
    case FS_TEXTURED_BLINN_PHONG: return 10;
    case FS_VERTEX_COLOR: return 4;
    case FS_CONSTANT_COLOR: return 0;
    default: return 8;
    }
}

uint32_t log2_floor(uint64_t x) {
    uint32_t r = 0;
    while (x > 1) { x >>= 1; ++r; }
    return r;
}

}  // namespace

struct sr_batch {
    cudaStream_t own_stream = nullptr, stream = nullptr;
    DevBuf<unsigned char> dtab;
    unsigned char* htab = nullptr;
    size_t htab_cap = 0;
    DevBuf<float4> scr4;
    DevBuf<float> vary;
    DevBuf<float4> setup;
    DevBuf<unsigned long long> area;
    DevBuf<uint32_t> big_list, big_base, unsafe_list;
    DevBuf<unsigned long long> tlist;       // touched (draw, block) list
    DevBuf<uint2> binrect;                  // per primitive: its bin rectangle, or RECT_EMPTY
    DevBuf<uint32_t> bin_cnt, bin_cursor;   // per (draw, bin): listed primitives, slots taken
    DevBuf<unsigned long long> bin_pack, bin_off, bin_tmp;   // packed counts, their exclusive scan, scan scratch
    DevBuf<uint32_t> entries;               // the bins' primitive lists
    DevBuf<uint32_t> item_bin;              // the (draw, bin) of each work item
    uint32_t bin_cap = 0;                   // (draw, bin) capacity the graphs were recorded for
    DeviceFlags* flags = nullptr;
    DeviceFlags* hflags = nullptr;
    unsigned long long* queues = nullptr;   // work-queue counters of the resolve launches
    uint32_t combos = 0;                    // (fragment shader, colour format) pairs of the current batch
    cudaEvent_t done = nullptr, ev0 = nullptr, ev1 = nullptr;
    bool in_flight = false;
    bool use_graphs = true, autotune = true;
    BatchConfig forced{0, 0, 0};
    std::map<uint64_t, BatchConfig> tuned;
    struct Graph { uint32_t NB; BatchConfig cfg; uint64_t gen; uint32_t combos; uint32_t bin_cap; cudaGraphExec_t exec; };
    std::vector<Graph> graphs;
    uint64_t gen = 1;            // bumped whenever a device buffer moves
    BatchConfig last_cfg;
    uint64_t last_tris = 0;
    sr_stats last{};
    bool stats_valid = false;
};

namespace {

void drop_graphs(sr_batch* b) {
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
    b->graphs.clear();
}

template <typename T>
int grow(sr_batch* b, DevBuf<T>& buf, size_t n) {
    if (n <= buf.cap) return SR_OK;
    // a buffer that moves invalidates the recorded graphs; wait for users
    if (b->in_flight) cudaEventSynchronize(b->done);
    drop_graphs(b);
    ++b->gen;
    return buf.ensure(n);
}

BTables tables_at(unsigned char* base, const Layout& L) {
    BTables T;
    T.n = reinterpret_cast<const uint32_t*>(base + L.off_n);
    T.inst = reinterpret_cast<const BInst*>(base + L.off_inst);
    T.U = reinterpret_cast<const sr_uniforms*>(base + L.off_U);
    T.qbase = reinterpret_cast<const uint32_t*>(base + L.off_q);
    T.tbase = reinterpret_cast<const uint32_t*>(base + L.off_t);
    T.bbase = reinterpret_cast<const uint32_t*>(base + L.off_b);
    T.cbase = reinterpret_cast<const uint32_t*>(base + L.off_c);
    return T;
}

// The launch sequence of one batch (also what a graph records).
void enqueue_batch(sr_batch* b, uint32_t NB, const BatchConfig& c) {
    const Layout L = layout_for(NB);
    cudaStream_t st = b->stream;
    const BTables T = tables_at(b->dtab.p, L);
    cudaMemcpyAsync(b->dtab.p, b->htab, L.bytes, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(b->flags, 0, sizeof(DeviceFlags), st);
    cudaMemsetAsync(b->queues, 0, N_QUEUES * sizeof(unsigned long long), st);
    batch_vertex_kernel<<<resident_grid(batch_vertex_kernel, 128, 16), 128, 0, st>>>(T, b->scr4.p, b->vary.p);
    const uint32_t cap = b->bin_cap;
    batch_setup_kernel<<<resident_grid(batch_setup_kernel, 256, 8), 256, 0, st>>>(
        T, b->scr4.p, b->setup.p, b->area.p, b->unsafe_list.p, b->binrect.p, b->bin_cnt.p, c.G, c.big, b->big_list.p,
        b->big_base.p, b->queues, b->flags);
    batch_raster_big_kernel<<<resident_grid(batch_raster_big_kernel, 256, 8), 256, 0, st>>>(
        T, b->setup.p, b->area.p, b->big_list.p, b->big_base.p, b->tlist.p, b->queues, b->flags);
    batch_ext_kernel<<<resident_grid(batch_ext_kernel, 256, 4), 256, 0, st>>>(T, b->setup.p, b->unsafe_list.p,
                                                                             b->tlist.p, b->queues, b->flags);
    batch_bin_pack_kernel<<<resident_grid(batch_bin_pack_kernel, 256, 8), 256, 0, st>>>(T, cap, b->bin_cnt.p,
                                                                                        b->bin_pack.p);
    exclusive_scan<unsigned long long>(b->bin_pack.p, cap, b->bin_off.p, b->bin_tmp.p, st);
    batch_bin_items_kernel<<<resident_grid(batch_bin_items_kernel, 256, 8), 256, 0, st>>>(T, b->bin_off.p,
                                                                                          b->item_bin.p,
                                                                                          b->item_bin.cap);
    batch_bin_scatter_kernel<<<resident_grid(batch_bin_scatter_kernel, 256, 8), 256, 0, st>>>(
        T, b->binrect.p, b->bin_off.p, b->bin_cursor.p, b->entries.p, b->entries.cap, b->flags);
    batch_bin_raster_kernel<<<resident_grid(batch_bin_raster_kernel, TL_THREADS, (int)c.ctas), TL_THREADS, 0, st>>>(
        T, b->setup.p, b->bin_off.p, cap, b->item_bin.p, b->item_bin.cap, b->entries.p, b->entries.cap,
        b->bin_cursor.p, b->flags);
    batch_collect_kernel<<<resident_grid(batch_collect_kernel, 256, 8), 256, 0, st>>>(T, b->tlist.p, b->queues);
    batch_clear_kernel<<<resident_grid(batch_clear_kernel, 256, 8), 256, 0, st>>>(T);
    for (int fs = 0; fs < FS_COUNT; ++fs)
        for (int fmt = 0; fmt < 3; ++fmt) {
            if (!(b->combos & (1u << (fs * 3 + fmt)))) continue;
            const int qi = fs * 3 + fmt;
#define SR_BRES(FS, FMT) batch_resolve_kernel<FS, FMT><<<resident_grid(batch_resolve_kernel<FS, FMT>, 256, 8), 256, 0, st>>>( \
                T, b->setup.p, b->vary.p, b->tlist.p, b->queues, qi)
#define SR_BRES_FS(FS)                                        \
            if (fmt == SR_COLOR_RGBA8) SR_BRES(FS, SR_COLOR_RGBA8);   \
            else if (fmt == SR_COLOR_RGBA32F) SR_BRES(FS, SR_COLOR_RGBA32F); \
            else SR_BRES(FS, SR_COLOR_NONE);
            switch (fs) {
            case FS_BLINN_PHONG_DIR: SR_BRES_FS(FS_BLINN_PHONG_DIR) break;
            case FS_TEXTURED_BLINN_PHONG: SR_BRES_FS(FS_TEXTURED_BLINN_PHONG) break;
            case FS_VERTEX_COLOR: SR_BRES_FS(FS_VERTEX_COLOR) break;
            case FS_ACES_LIGHTS: SR_BRES_FS(FS_ACES_LIGHTS) break;
            default: SR_BRES_FS(FS_CONSTANT_COLOR) break;
            }
#undef SR_BRES_FS
#undef SR_BRES
        }
}

int launch_batch(sr_batch* b, uint32_t NB, const BatchConfig& c) {
    if (!b->use_graphs) {
        enqueue_batch(b, NB, c);
        SR_CK(cudaGetLastError());
        return SR_OK;
    }
    cudaGraphExec_t exec = nullptr;
    for (auto& g : b->graphs)
        if (g.NB == NB && g.cfg == c && g.gen == b->gen && g.combos == b->combos && g.bin_cap == b->bin_cap)
            exec = g.exec;
    if (!exec) {
        cudaGraph_t graph = nullptr;
        SR_CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_batch(b, NB, c);
        cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
        if (e != cudaSuccess) { last_cuda_error() = e; return SR_ECUDA; }
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { last_cuda_error() = e; return SR_ECUDA; }
        if (b->graphs.size() >= 32) { cudaGraphExecDestroy(b->graphs.front().exec); b->graphs.erase(b->graphs.begin()); }
        b->graphs.push_back({NB, c, b->gen, b->combos, b->bin_cap, exec});
    }
    SR_CK(cudaGraphLaunch(exec, b->stream));
    return SR_OK;
}

// Measures every candidate configuration on this batch (rendering it is
// idempotent: same inputs, same winners) and returns the fastest.
BatchConfig tune(sr_batch* b, uint32_t NB, uint32_t g_max) {
    static const uint32_t Gs[] = {4, 16, 32};
    static const uint32_t bigs[] = {4096, 16384, 65536};
    static const uint32_t ctas[] = {4, 8};
    BatchConfig best;
    float best_ms = 1e30f;
    for (uint32_t g : Gs)
        for (uint32_t bg : bigs)
            for (uint32_t ct : ctas) {
                BatchConfig c{std::min(g, g_max), bg, ct};
                enqueue_batch(b, NB, c);   // warm
                cudaEventRecord(b->ev0, b->stream);
                enqueue_batch(b, NB, c);
                enqueue_batch(b, NB, c);
                cudaEventRecord(b->ev1, b->stream);
                if (cudaEventSynchronize(b->ev1) != cudaSuccess) return best;
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, b->ev0, b->ev1);
                if (ms < best_ms) { best_ms = ms; best = c; }
            }
    return best;
}

}  // namespace

extern "C" SR_API int sr_batch_create(sr_batch** out) {
    if (!out) return SR_EINVAL;
    *out = nullptr;
    sr_batch* b = new (std::nothrow) sr_batch();
    if (!b) return SR_ENOMEM;
    cudaError_t e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->flags, sizeof(DeviceFlags));
    if (e == cudaSuccess) e = cudaMallocHost(&b->hflags, sizeof(DeviceFlags));
    if (e == cudaSuccess) e = cudaMalloc(&b->queues, N_QUEUES * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e != cudaSuccess) {
        last_cuda_error() = e;
        sr_batch_destroy(b);
        return e == cudaErrorMemoryAllocation ? SR_ENOMEM : SR_ECUDA;
    }
    b->stream = b->own_stream;
    *out = b;
    return SR_OK;
}

extern "C" SR_API int sr_batch_destroy(sr_batch* b) {
    if (!b) return SR_EINVAL;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    b->dtab.release(); b->scr4.release(); b->vary.release(); b->setup.release();
    b->area.release(); b->big_list.release(); b->big_base.release(); b->unsafe_list.release(); b->tlist.release();
    b->binrect.release(); b->bin_cnt.release(); b->bin_cursor.release(); b->bin_pack.release();
    b->bin_off.release(); b->bin_tmp.release(); b->entries.release(); b->item_bin.release();
    if (b->htab) cudaFreeHost(b->htab);
    if (b->flags) cudaFree(b->flags);
    if (b->hflags) cudaFreeHost(b->hflags);
    if (b->queues) cudaFree(b->queues);
    if (b->done) cudaEventDestroy(b->done);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return SR_OK;
}

extern "C" SR_API int sr_batch_set_stream(sr_batch* b, void* stream) {
    if (!b) return SR_EINVAL;
    if (b->in_flight) cudaEventSynchronize(b->done);
    b->stream = stream ? (cudaStream_t)stream : b->own_stream;
    return SR_OK;
}

extern "C" SR_API int sr_batch_set_options(sr_batch* b, int use_graphs, int autotune) {
    if (!b) return SR_EINVAL;
    b->use_graphs = use_graphs != 0;
    b->autotune = autotune != 0;
    return SR_OK;
}

extern "C" SR_API int sr_batch_set_config(sr_batch* b, uint32_t ppw, uint32_t big, uint32_t ctas) {
    if (!b) return SR_EINVAL;
    if (ppw == 0 && big == 0 && ctas == 0) { b->forced = BatchConfig{0, 0, 0}; return SR_OK; }
    if (ppw == 0 || ppw > 32 || (ppw & (ppw - 1)) || big == 0 || ctas == 0 || ctas > 8) return SR_EINVAL;
    b->forced = BatchConfig{ppw, big, ctas};
    return SR_OK;
}

extern "C" SR_API int sr_batch_get_config(sr_batch* b, uint32_t* ppw, uint32_t* big, uint32_t* ctas) {
    if (!b || !ppw || !big || !ctas) return SR_EINVAL;
    *ppw = b->last_cfg.G; *big = b->last_cfg.big; *ctas = b->last_cfg.ctas;
    return SR_OK;
}

// The checks of one draw that sr_batch_render makes independently of its
// target; the server makes them when a request is submitted, so that an
// ineligible request is refused alone instead of failing its whole batch.
int sr::batch_draw_check(const sr_draw* d) {
    const sr_mesh* m = d ? d->mesh : nullptr;
    if (!m) return SR_EINVAL;
    if (d->prim != SR_PRIM_TRIANGLE || d->gs_mode != SR_GS_NONE || d->blend != BLEND_REPLACE) return SR_EINVAL;
    if (d->reuse != SR_REUSE_NONE) return SR_EINVAL;
    if (m->n_indices % 3 != 0) return SR_EINVAL;                            // mod.rs:148
    if (d->vs < 0 || d->vs >= VS_COUNT || d->fs < 0 || d->fs >= FS_COUNT) return SR_EINVAL;
    if (d->tile_w == 0 || d->tile_h == 0 || d->tile_w > 65535 || d->tile_h > 65535) return SR_EINVAL;
    if (d->tex_filter > SR_SAMPLE_BILINEAR || d->tex_edge > SR_SAMPLE_BORDER) return SR_EINVAL;
    if (d->cull > SR_CULL_COUNTER_CLOCKWISE) return SR_EINVAL;
    if (m->n_planes < (uint32_t)vs_planes(d->vs)) return SR_EINVAL;
    if (vs_nk(d->vs) < batch_min_varyings(d->fs)) return SR_EINVAL;
    if (d->fs == FS_TEXTURED_BLINN_PHONG && !d->texture) return SR_EINVAL;
    if (d->texture && d->texture->view) return SR_EINVAL;   // another target of the batch may write it
    return SR_OK;
}

extern "C" SR_API int sr_batch_render(sr_batch* b, const sr_batch_item* items, uint32_t n) {
    if (!b || (n && !items)) return SR_EINVAL;
    if (n == 0) return SR_OK;
    if (n > (1u << 20)) return SR_EINVAL;
    // ---- validation (nothing is enqueued unless every item is acceptable)
    std::unordered_set<const sr_pipeline*> seen;
    uint64_t slots = 0, tris = 0, blocks = 0, clear_blocks = 0, px = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const sr_batch_item& it = items[i];
        const sr_pipeline* p = it.target;
        const sr_draw* d = &it.draw;
        const sr_mesh* m = d->mesh;
        if (!p || !m) return SR_EINVAL;
        if (!p->pending.empty()) return SR_EBUSY;
        if (!seen.insert(p).second) return SR_EINVAL;                       // targets must be distinct
        const int rc = batch_draw_check(d);
        if (rc != SR_OK) return rc;
        if (p->stencil && !(p->stencil_test == SR_STENCIL_ALWAYS && p->stencil_op == SR_STENCIL_KEEP)) return SR_EINVAL;
        const uint64_t npx = (uint64_t)p->fb.width * p->fb.height;
        slots += m->n_pad;
        tris += m->n_indices / 3;
        blocks += (uint64_t)((p->fb.width + 31) / 32) * ((p->fb.height + 31) / 32);
        if (it.clear) clear_blocks += (uint64_t)((p->fb.width + 31) / 32) * ((p->fb.height + 31) / 32);
        px += npx;
    }
    if (slots >= (1ull << 31) || tris >= (1ull << 31) || blocks >= (1ull << 31) || clear_blocks >= (1ull << 31))
        return SR_EINVAL;
    // the host table is reused: the previous batch must have consumed it
    if (b->in_flight) {
        SR_CK(cudaEventSynchronize(b->done));
        b->in_flight = false;
    }
    const uint32_t NB = bucket_of(n);
    const Layout L = layout_for(NB);
    int rc;
    if (L.bytes > b->htab_cap) {
        if (b->htab) cudaFreeHost(b->htab);
        b->htab = nullptr;
        b->htab_cap = 0;
        SR_CK(cudaMallocHost(&b->htab, L.bytes));
        b->htab_cap = L.bytes;
    }
    if ((rc = grow(b, b->dtab, L.bytes)) || (rc = grow(b, b->scr4, slots + 4)) ||
        (rc = grow(b, b->vary, (slots + 4) * VSTRIDE)) || (rc = grow(b, b->setup, 4 * (tris + 1))) ||
        (rc = grow(b, b->area, tris + 1)) || (rc = grow(b, b->big_list, tris + 1)) ||
        (rc = grow(b, b->big_base, tris + 1)) || (rc = grow(b, b->unsafe_list, tris + 1)) ||
        (rc = grow(b, b->tlist, blocks + 1)) || (rc = grow(b, b->binrect, tris + 1)))
        return rc;
    // (draw, bin) buffers for a power-of-two capacity of bins (the graphs are
    // recorded per capacity); the lists hold up to `bins per listed
    // primitive` entries per primitive, so they are sized for the largest
    // value this batch may use (the tuner's candidates go up to 32)
    uint32_t bin_cap = 1024;
    while (bin_cap < blocks) bin_cap <<= 1;
    BatchConfig pre;
    const uint64_t cls = ((uint64_t)bucket_of(n) << 40) | ((uint64_t)log2_floor(tris + 1) << 20) | log2_floor(px + 1);
    const auto tuned_it = b->tuned.find(cls);
    uint32_t g_max = pre.G;
    if (b->forced.G) g_max = b->forced.G;
    else if (tuned_it != b->tuned.end()) g_max = tuned_it->second.G;
    else if (b->autotune) g_max = 32;
    while (g_max > 1 && (uint64_t)g_max * tris >= 0xffffffffull) g_max >>= 1;
    const size_t cnt_cap0 = b->bin_cnt.cap, cur_cap0 = b->bin_cursor.cap;
    if ((rc = grow(b, b->bin_cnt, bin_cap)) || (rc = grow(b, b->bin_cursor, bin_cap)) ||
        (rc = grow(b, b->bin_pack, bin_cap)) || (rc = grow(b, b->bin_off, (size_t)bin_cap + 1)) ||
        (rc = grow(b, b->bin_tmp, (size_t)scan_blocks(bin_cap) + 2)) ||
        (rc = grow(b, b->entries, (size_t)g_max * tris + 1)) ||
        (rc = grow(b, b->item_bin, bin_item_cap((uint64_t)g_max * tris, bin_cap))))
        return rc;
    // the counts and cursors are zeroed whenever they are (re)allocated (a
    // new allocation may reuse the old address, so the capacity tells); the
    // batch's own kernels reset what they used
    if (b->bin_cnt.cap != cnt_cap0) SR_CK(cudaMemsetAsync(b->bin_cnt.p, 0, b->bin_cnt.cap * 4, b->stream));
    if (b->bin_cursor.cap != cur_cap0) SR_CK(cudaMemsetAsync(b->bin_cursor.p, 0, b->bin_cursor.cap * 4, b->stream));
    b->bin_cap = bin_cap;
    // ---- host table
    std::memset(b->htab, 0, L.bytes);
    *reinterpret_cast<uint32_t*>(b->htab + L.off_n) = n;
    BInst* hi = reinterpret_cast<BInst*>(b->htab + L.off_inst);
    sr_uniforms* hu = reinterpret_cast<sr_uniforms*>(b->htab + L.off_U);
    uint32_t* qb = reinterpret_cast<uint32_t*>(b->htab + L.off_q);
    uint32_t* tb = reinterpret_cast<uint32_t*>(b->htab + L.off_t);
    uint32_t* bb = reinterpret_cast<uint32_t*>(b->htab + L.off_b);
    uint32_t* cb = reinterpret_cast<uint32_t*>(b->htab + L.off_c);
    uint32_t vbase = 0;
    uint32_t combos = 0;
    qb[0] = tb[0] = bb[0] = cb[0] = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const sr_batch_item& it = items[i];
        sr_pipeline* p = it.target;
        const sr_draw* d = &it.draw;
        const sr_mesh* m = d->mesh;
        const uint32_t W = p->fb.width, H = p->fb.height;
        const size_t npx = (size_t)W * H;
        const size_t nblk = (size_t)((W + 31) / 32) * ((H + 31) / 32);
        // the target's opaque scratch (zero between draws; zeroed when allocated)
        const bool fresh = p->gkeys.cap < npx || p->bitmap.cap < (nblk + 31) / 32;
        if ((rc = p->gkeys.ensure(npx)) || (rc = p->bitmap.ensure((nblk + 31) / 32))) return rc;
        if (fresh) {
            SR_CK(cudaMemsetAsync(p->gkeys.p, 0, p->gkeys.cap * 8, b->stream));
            SR_CK(cudaMemsetAsync(p->bitmap.p, 0, p->bitmap.cap * 4, b->stream));
        }
        p->have_prev = false;   // sr_draw.reuse after a batch has no previous sr_render to refer to
        BInst& I = hi[i];
        DrawParams& P = I.P;
        P.W = W; P.H = H;
        P.tile_w = d->tile_w; P.tile_h = d->tile_h;
        P.magic_w = div_magic(d->tile_w); P.magic_h = div_magic(d->tile_h);
        P.ncols = W >= 2 ? (W - 1 + d->tile_w - 1) / d->tile_w : 0;
        P.nrows = H >= 2 ? (H - 1 + d->tile_h - 1) / d->tile_h : 0;
        P.n_verts = m->n_verts;
        P.gen_base = m->n_pad;
        P.n_in = (uint32_t)(m->n_indices / 3);
        P.cull = d->cull;
        P.vs = d->vs; P.fs = d->fs; P.blend = BLEND_REPLACE;
        std::memcpy(P.vp, &d->viewport, sizeof(P.vp));
        P.has_depth = p->depth != nullptr;
        P.has_stencil = 0;
        P.color_format = p->fb.color_format;
        P.stencil_test = SR_STENCIL_ALWAYS; P.stencil_op = SR_STENCIL_KEEP; P.stencil_wrap = 1;
        P.force_unsafe = p->force_unsafe ? 1u : 0u;
        uint32_t tex_f32 = 0;
        const uint32_t* tex_data = sampled_texels(d->texture, &tex_f32);
        if (d->texture) { P.tex_w = d->texture->w; P.tex_h = d->texture->h; P.tex_f32 = tex_f32; }
        P.tex_filter = d->tex_filter; P.tex_edge = d->tex_edge;
        P.bin_w_log2 = 5; P.bin_h_log2 = 5;
        P.bins_x = (W + 31) >> 5; P.bins_y = (H + 31) >> 5;
        // the draw renders nothing when the frame has no semantic tile or a
        // missing stencil attachment fails the test (as in sr_render)
        const bool nothing = W < 2 || H < 2 || (!p->stencil && !stencil_test(p->stencil_test, 0, 0));
        const uint32_t nt = nothing ? 0u : P.n_in;
        P.n_raster_host = nt;
        I.vpm = viewport_matrix(P.vp);
        I.planes = m->planes;
        I.indices = m->indices;
        I.tex = tex_data;
        I.color = p->color;
        I.depth = p->depth;
        I.gkeys = p->gkeys.p;
        I.bitmap = p->bitmap.p;
        I.n_pad = m->n_pad;
        I.vbase = vbase;
        I.tbase = tb[i];
        I.clear = it.clear ? 1u : 0u;
        if (p->fb.color_format == SR_COLOR_RGBA32F) {
            std::memcpy(&I.clear_color, it.clear_color, 16);
        } else {
            uint32_t c;
            std::memcpy(&c, it.clear_color, 4);
            I.clear_color = make_uint4(c, c, c, c);
        }
        I.mx = div_magic(d->tile_w);
        I.my = div_magic(d->tile_h);
        hu[i] = p->U;
        if (!nothing) combos |= 1u << (d->fs * 3 + (int)p->fb.color_format);
        vbase += m->n_pad;
        qb[i + 1] = qb[i] + (nothing ? 0u : m->n_verts);
        tb[i + 1] = tb[i] + nt;
        bb[i + 1] = bb[i] + (nothing ? 0u : (uint32_t)nblk);
        cb[i + 1] = cb[i] + (it.clear ? (uint32_t)nblk : 0u);
    }
    b->combos = combos;
    // ---- configuration: forced, tuned for this size class, or the default
    BatchConfig cfg;
    if (b->forced.G) {
        cfg = b->forced;
    } else if (tuned_it != b->tuned.end()) {
        cfg = tuned_it->second;
    } else if (b->autotune) {
        cfg = tune(b, NB, g_max);
        b->tuned[cls] = cfg;
    }
    // the lists were sized for g_max entries per primitive
    if (cfg.G > g_max) cfg.G = g_max;
    if ((rc = launch_batch(b, NB, cfg))) return rc;
    SR_CK(cudaEventRecord(b->done, b->stream));
    b->in_flight = true;
    b->last_cfg = cfg;
    b->last_tris = tris;
    b->stats_valid = false;
    return SR_OK;
}

extern "C" SR_API int sr_batch_sync(sr_batch* b) {
    if (!b) return SR_EINVAL;
    SR_CK(cudaStreamSynchronize(b->stream));
    if (!b->in_flight && b->stats_valid) return SR_OK;
    b->in_flight = false;
    SR_CK(cudaMemcpyAsync(b->hflags, b->flags, sizeof(DeviceFlags), cudaMemcpyDeviceToHost, b->stream));
    SR_CK(cudaStreamSynchronize(b->stream));
    const DeviceFlags& f = *b->hflags;
    sr_stats& s = b->last;
    std::memset(&s, 0, sizeof(s));
    s.triangles_in = b->last_tris;
    s.triangles_generated = b->last_tris;
    s.triangles_raster = f.triangles_raster;
    s.unsafe_triangles = f.unsafe;
    s.fragments = f.fragments;
    s.nan_bbox = f.nan_bbox;
    s.kernel_launches = 13 + (uint32_t)__builtin_popcount(b->combos);
    b->stats_valid = true;
    if (f.bad_index) return SR_EINVAL;
    if (f.overflow_bits) return SR_EOVERFLOW;
    if (f.nan_total) return SR_ENAN;
    return SR_OK;
}

extern "C" SR_API int sr_batch_get_stats(sr_batch* b, sr_stats* out) {
    if (!b || !out) return SR_EINVAL;
    *out = b->last;
    return SR_OK;
}
