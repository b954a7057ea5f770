// sr_scan.cuh — exclusive prefix sums (reduce / scan-of-block-sums / apply),
// used for order-preserving compaction of geometry-shader output and for bin
// offsets.  Three launches, no inter-block waiting.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sr {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;   // 4096 elements per block
constexpr int SCAN_MAX_BLOCKS = 8192;                    // block sums scanned in registers (33.5M elements)

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// Block-wide exclusive scan; returns the block total through *total.
template <typename T, int NT>
__device__ __forceinline__ T block_exclusive_scan(T v, T* total) {
    __shared__ T warp_sums[NT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T s = lane < NT / 32 ? warp_sums[lane] : T(0);
        s = warp_inclusive_scan(s);
        if (lane < NT / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    T base = warp ? warp_sums[warp - 1] : T(0);
    *total = warp_sums[NT / 32 - 1];
    __syncthreads();
    return base + inc - v;
}

template <typename T>
__global__ void scan_reduce_kernel(const T* __restrict__ in, uint64_t n, T* __restrict__ block_sums) {
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    T s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t j = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        if (j < n) s += in[j];
    }
    T tot;
    block_exclusive_scan<T, SCAN_THREADS>(s, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// One block scans up to SCAN_MAX_BLOCKS block sums in place (exclusive) and
// stores the grand total at block_sums[nb].
template <typename T>
__global__ void scan_blocks_kernel(T* block_sums, uint32_t nb) {
    constexpr int NT = 1024;
    constexpr int PER = SCAN_MAX_BLOCKS / NT;
    T v[PER];
    T s = 0;
    for (int i = 0; i < PER; ++i) {
        uint32_t j = threadIdx.x * PER + i;
        v[i] = j < nb ? block_sums[j] : T(0);
        s += v[i];
    }
    T tot;
    T ex = block_exclusive_scan<T, NT>(s, &tot);
    for (int i = 0; i < PER; ++i) {
        uint32_t j = threadIdx.x * PER + i;
        if (j < nb) block_sums[j] = ex;
        ex += v[i];
    }
    if (threadIdx.x == 0) block_sums[nb] = tot;
}

// The same for any number of block sums (scans of more than SCAN_MAX_BLOCKS
// tiles): each thread takes a contiguous run of ceil(nb / 1024) sums and reads
// it twice from global memory instead of holding it in registers.  The block
// scan's barriers order every read before the first write.
template <typename T>
__global__ void scan_blocks_large_kernel(T* block_sums, uint32_t nb) {
    constexpr int NT = 1024;
    const uint32_t per = (nb + NT - 1) / NT;
    const uint64_t j0 = (uint64_t)threadIdx.x * per;
    T s = 0;
    for (uint32_t i = 0; i < per; ++i) {
        const uint64_t j = j0 + i;
        if (j < nb) s += block_sums[j];
    }
    T tot;
    T ex = block_exclusive_scan<T, NT>(s, &tot);
    for (uint32_t i = 0; i < per; ++i) {
        const uint64_t j = j0 + i;
        if (j < nb) {
            const T v = block_sums[j];
            block_sums[j] = ex;
            ex += v;
        }
    }
    if (threadIdx.x == 0) block_sums[nb] = tot;
}

// Shared-memory slot of tile element e, padded by one element per 128 bytes
// so that the blocked-per-thread accesses (thread t reads elements
// t * SCAN_ITEMS ..) fall into distinct banks.
template <typename T>
__device__ __forceinline__ int scan_slot(int e) { return e + (e >> (sizeof(T) == 8 ? 4 : 5)); }
template <typename T>
constexpr int scan_tile_slots() { return SCAN_TILE + (SCAN_TILE >> (sizeof(T) == 8 ? 4 : 5)); }

// out[j] = exclusive prefix of in; out[n] = total.  Loads and stores are
// coalesced; in between, each thread scans SCAN_ITEMS consecutive values.
template <typename T>
__global__ void scan_apply_kernel(const T* __restrict__ in, uint64_t n, const T* __restrict__ block_sums,
                                  uint32_t nb, T* __restrict__ out) {
    __shared__ T tile[scan_tile_slots<T>()];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t j = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        tile[scan_slot<T>(i * SCAN_THREADS + threadIdx.x)] = j < n ? in[j] : T(0);
    }
    __syncthreads();
    T v[SCAN_ITEMS];
    T s = 0;
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = tile[scan_slot<T>(threadIdx.x * SCAN_ITEMS + i)];
        s += v[i];
    }
    T tot;
    T ex = block_exclusive_scan<T, SCAN_THREADS>(s, &tot) + block_sums[blockIdx.x];
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        tile[scan_slot<T>(threadIdx.x * SCAN_ITEMS + i)] = ex;
        ex += v[i];
    }
    __syncthreads();
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t j = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        if (j < n) out[j] = tile[scan_slot<T>(i * SCAN_THREADS + threadIdx.x)];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = block_sums[nb];
}

inline uint32_t scan_blocks(uint64_t n) { return (uint32_t)((n + SCAN_TILE - 1) / SCAN_TILE); }

// tmp must hold scan_blocks(n) + 1 elements; out must hold n + 1.
// Returns false if n exceeds the supported size (2^40 elements).
template <typename T>
inline bool exclusive_scan(const T* in, uint64_t n, T* out, T* tmp, cudaStream_t st) {
    if (n > (1ull << 40)) return false;
    uint32_t nb = scan_blocks(n);
    if (nb == 0) nb = 1;
    scan_reduce_kernel<T><<<nb, SCAN_THREADS, 0, st>>>(in, n, tmp);
    if (nb <= (uint32_t)SCAN_MAX_BLOCKS)
        scan_blocks_kernel<T><<<1, 1024, 0, st>>>(tmp, nb);
    else
        scan_blocks_large_kernel<T><<<1, 1024, 0, st>>>(tmp, nb);
    scan_apply_kernel<T><<<nb, SCAN_THREADS, 0, st>>>(in, n, tmp, nb, out);
    return true;
}

}  // namespace sr
