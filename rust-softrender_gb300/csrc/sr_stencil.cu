// sr_stencil.cu — stencil events of a draw counted in closed form.
//
// rasterize_triangle applies `if test(s, ref) { s = op(s, ref) }` to EVERY
// pixel of the primitive's bounding box clamped to the current tile
// (triangle.rs:66-99), covered or not, once per semantic tile pass.  A bbox
// outside the tile collapses onto the tile's edge row / column, so each
// primitive touches every tile (edge pixels receive events from primitives
// far away), and seam pixels are visited by 2 or 4 tile passes.
//
// When the stencil test is Always (and the op is not Keep), every event is the
// same map g = op, so the final value is g^K(s0) with K(p) the number of
// events on the pixel, and fragments are never gated.  With the floor-rounded
// bbox [ix0, ix1] x [iy0, iy1] and the tiles containing a pixel forming a
// product of tile columns and tile rows, K(p) = sum_t X(t, px) * Y(t, py) where
//   X = [ix0 <= px <= ix1]                      px inside a tile column
//   X = 1 + [ix0 <= px <= ix1]                  px on a seam column (2 tiles)
//   X = [ix0 <= 0]  = f + [ix1 < 0]             px = 0
//   X = [ix1 >= W-1] = f + [ix0 > W-1]          px = W-1
// (and the same in y), which expands into a 2D bbox-coverage count, 1D column
// and row interval counts and a few global counts, all gathered with
// difference arrays in the setup pass and prefix-summed here.
#include "sr_internal.cuh"

namespace sr {

// inclusive prefix along rows of a (rows x cols) int array, one block per row
__global__ void __launch_bounds__(256) row_prefix_kernel(int* a, uint32_t cols) {
    int* row = a + (size_t)blockIdx.x * cols;
    __shared__ int carry;
    __shared__ int wsum[8];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < cols; base += 256) {
        uint32_t i = base + threadIdx.x;
        int v = i < cols ? row[i] : 0;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            int n = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += n;
        }
        if (lane == 31) wsum[w] = v;
        __syncthreads();
        int add = carry;
        for (int k = 0; k < w; ++k) add += wsum[k];
        if (i < cols) row[i] = v + add;
        __syncthreads();
        if (threadIdx.x == 255) carry = v + add;
        __syncthreads();
    }
}

// Inclusive prefix down the columns of a (rows x cols) int array, in two
// passes over segments of STENCIL_SEG rows: the first sums each (segment,
// column), the second starts each (segment, column) from the sums of the
// segments above it and walks its rows.  One thread per (segment, column),
// consecutive threads on consecutive columns (coalesced rows).
__global__ void __launch_bounds__(256) col_seg_sum_kernel(const int* __restrict__ a, uint32_t rows, uint32_t cols,
                                                          int* __restrict__ seg) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y;
    if (c >= cols) return;
    const uint32_t r0 = g * STENCIL_SEG, r1 = min(r0 + STENCIL_SEG, rows);
    int acc = 0;
    for (uint32_t r = r0; r < r1; ++r) acc += a[(size_t)r * cols + c];
    seg[(size_t)g * cols + c] = acc;
}

__global__ void __launch_bounds__(256) col_seg_apply_kernel(int* __restrict__ a, uint32_t rows, uint32_t cols,
                                                            const int* __restrict__ seg) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y;
    if (c >= cols) return;
    int acc = 0;
    for (uint32_t k = 0; k < g; ++k) acc += seg[(size_t)k * cols + c];
    const uint32_t r0 = g * STENCIL_SEG, r1 = min(r0 + STENCIL_SEG, rows);
    for (uint32_t r = r0; r < r1; ++r) {
        acc += a[(size_t)r * cols + c];
        a[(size_t)r * cols + c] = acc;
    }
}

__device__ __forceinline__ uint32_t stencil_power(uint32_t op, uint32_t wrap, uint32_t s0, uint32_t ref, long long K) {
    if (K <= 0) return s0;
    switch (op) {
    case 1: return (K & 1) ? (~s0 & 0xffu) : s0;
    case 2: return 0;
    case 3: return ref;
    case 4: return wrap ? (uint32_t)((s0 + (unsigned long long)K) & 0xffu) : (uint32_t)min((long long)s0 + K, 255ll);
    case 5: return wrap ? (uint32_t)((s0 - (unsigned long long)K) & 0xffu) : (uint32_t)max((long long)s0 - K, 0ll);
    default: return s0;
    }
}

__global__ void __launch_bounds__(256) stencil_apply_kernel(DrawParams P, StencilCountArgs S, uint8_t* stencil,
                                                            DeviceFlags* flags) {
    if (flags->poison) return;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.W * P.H) return;
    const uint32_t W = P.W, H = P.H;
    uint32_t px = i % W, py = i / W;
    const int* CX = S.lines;
    const int* CXa = CX + (W + 1);
    const int* CXb = CXa + (W + 1);
    const int* CY = CXb + (W + 1);
    const int* CYl = CY + (H + 1);
    const int* CYr = CYl + (H + 1);
    const unsigned long long* G = S.globals;
    bool seam_x = px > 0 && px < W - 1 && (px % P.tile_w) == 0;
    bool seam_y = py > 0 && py < H - 1 && (py % P.tile_h) == 0;
    int ex = seam_x ? 1 : (px == 0 ? 2 : (px == W - 1 ? 3 : 0));   // 1 seam, 2 first, 3 last
    int ey = seam_y ? 1 : (py == 0 ? 2 : (py == H - 1 ? 3 : 0));
    long long K = S.diff2d[(size_t)py * (W + 1) + px];
    if (ey == 1) K += CX[px];
    else if (ey == 2) K += CXa[px];
    else if (ey == 3) K += CXb[px];
    if (ex == 1) K += CY[py];
    else if (ex == 2) K += CYl[py];
    else if (ex == 3) K += CYr[py];
    if (ex && ey) {
        // global counts: 0 all, 1 L, 2 R, 3 A, 4 B, 5 LA, 6 LB, 7 RA, 8 RB
        unsigned long long g;
        if (ex == 1 && ey == 1) g = G[0];
        else if (ex == 1) g = ey == 2 ? G[3] : G[4];
        else if (ey == 1) g = ex == 2 ? G[1] : G[2];
        else if (ex == 2) g = ey == 2 ? G[5] : G[6];
        else g = ey == 2 ? G[7] : G[8];
        K += (long long)g;
    }
    uint32_t s0 = stencil[i];
    stencil[i] = (uint8_t)stencil_power(P.stencil_op, P.stencil_wrap, s0, P.sref, K);
}

void launch_stencil_apply(const DrawParams& P, const StencilCountArgs& S, uint8_t* stencil, DeviceFlags* flags,
                          cudaStream_t st) {
    uint32_t W = P.W, H = P.H;
    row_prefix_kernel<<<H + 1, 256, 0, st>>>(S.diff2d, W + 1);
    const dim3 cg((W + 1 + 255) / 256, stencil_colseg_rows(H));
    col_seg_sum_kernel<<<cg, 256, 0, st>>>(S.diff2d, H + 1, W + 1, S.colseg);
    col_seg_apply_kernel<<<cg, 256, 0, st>>>(S.diff2d, H + 1, W + 1, S.colseg);
    // the line counts: CX, CXa, CXb (W+1 each), then CY, CYl, CYr (H+1 each)
    row_prefix_kernel<<<3, 256, 0, st>>>(S.lines, W + 1);
    row_prefix_kernel<<<3, 256, 0, st>>>(S.lines + 3 * (size_t)(W + 1), H + 1);
    uint32_t n = W * H;
    stencil_apply_kernel<<<(n + 255) / 256, 256, 0, st>>>(P, S, stencil, flags);
}

}  // namespace sr
