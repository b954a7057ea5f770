// sr_setup.cu — triangle setup and binning.
//
// Setup restates the per-primitive part of rasterize_triangle
// (stages/rasterization/triangle.rs:48-78): back-face culling by the shoelace
// sum, the determinant, the NaN-ignoring f32 min/max bounding box and its
// integer extent.  clamp_as_int(v, lo, hi) of the reference equals
// clamp(floor(v), lo, hi) for non-NaN v, so the floor-rounded bbox
// [ix0, ix1] x [iy0, iy1] determines every tile's clamped pixel range.
//
// The reference visits every primitive in every 128x128 tile
// (fragment.rs:268-311).  Here a primitive is binned only into the internal
// bins its pixels can produce fragments in:
//   * primitives whose computed det is 0 or NaN, or whose three screen z are
//     >= 0, can never produce a fragment (the covered branch then always
//     yields a NaN or non-negative z) and are not binned;
//   * for the rest, a conservative floating-point error bound (the "inflated
//     triangle": each edge pushed out by the worst-case rounding of the
//     reference's barycentric expressions over the frame) bounds every pixel
//     centre whose computed coverage can be true.  If that region lies inside
//     the integer bbox the primitive is "safe" and binned by its bbox; else it
//     is binned by the inflated region ("unsafe") and the raster evaluates the
//     reference's clamped tile-edge events for pixels outside the bbox.
// Stencil events of the clamped bbox (which hit tile edges from every
// primitive) are counted analytically in sr_stencil.cu.
#include "sr_internal.cuh"
#include "sr_scan.cuh"
#include "sr_setup.cuh"

namespace sr {


// Returns the set of global counters (bits 0..8 of S.globals) this primitive
// increments; the caller adds them up per warp.  The column and row interval
// counts every primitive inside the frame adds to (CX, CY) go to `sx` / `sy`:
// the CTA's shared copies when the frame is small enough, else the global
// arrays.
__device__ __forceinline__ uint32_t stencil_count_tri(const DrawParams& P, const StencilCountArgs& S, int ix0,
                                                  int iy0, int ix1, int iy1, int* sx, int* sy) {
    const int W = (int)P.W, H = (int)P.H;
    int x0 = max(ix0, 0), x1 = min(ix1, W - 1), y0 = max(iy0, 0), y1 = min(iy1, H - 1);
    bool xin = x0 <= x1, yin = y0 <= y1;
    int* CX = sx;
    int* CXa = S.lines + (W + 1);
    int* CXb = CXa + (W + 1);
    int* CY = sy;
    int* CYl = S.lines + 3 * (W + 1) + (H + 1);
    int* CYr = CYl + (H + 1);
    bool L = ix1 < 0, R = ix0 > W - 1, A = iy1 < 0, B = iy0 > H - 1;
    if (xin && yin) {
        size_t st = (size_t)W + 1;
        atomicAdd(S.diff2d + (size_t)y0 * st + x0, 1);
        atomicAdd(S.diff2d + (size_t)y0 * st + x1 + 1, -1);
        atomicAdd(S.diff2d + (size_t)(y1 + 1) * st + x0, -1);
        atomicAdd(S.diff2d + (size_t)(y1 + 1) * st + x1 + 1, 1);
    }
    if (xin) {
        atomicAdd(CX + x0, 1); atomicAdd(CX + x1 + 1, -1);
        if (A) { atomicAdd(CXa + x0, 1); atomicAdd(CXa + x1 + 1, -1); }
        if (B) { atomicAdd(CXb + x0, 1); atomicAdd(CXb + x1 + 1, -1); }
    }
    if (yin) {
        atomicAdd(CY + y0, 1); atomicAdd(CY + y1 + 1, -1);
        if (L) { atomicAdd(CYl + y0, 1); atomicAdd(CYl + y1 + 1, -1); }
        if (R) { atomicAdd(CYr + y0, 1); atomicAdd(CYr + y1 + 1, -1); }
    }
    return 1u | (L ? 2u : 0u) | (R ? 4u : 0u) | (A ? 8u : 0u) | (B ? 16u : 0u) | ((L && A) ? 32u : 0u) |
           ((L && B) ? 64u : 0u) | ((R && A) ? 128u : 0u) | ((R && B) ? 256u : 0u);
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;   // the sum in lane 0
}

// One thread per raster triangle: setup record, bin rectangle, bin counts,
// and (when the stencil changes under Always) the stencil event counts.  The
// grid covers the primitives in strides of the whole grid.  With `shared_lines`
// the column and row interval counts of the stencil events (one +1 / -1 pair
// per primitive on W+1 and H+1 counters, which every primitive of a dense
// frame hits) accumulate in shared memory over the CTA's primitives and are
// added to the global arrays once per CTA.
__global__ void __launch_bounds__(256) setup_kernel(DrawParams P, uint32_t n_host, const uint32_t* __restrict__ vidx,
                                                    const float4* __restrict__ scr4, float4* __restrict__ setup,
                                                    uint2* __restrict__ binrect, uint32_t* __restrict__ bin_counts,
                                                    uint32_t* __restrict__ unsafe_list,
                                                    float4* __restrict__ unsafe_rect,
                                                    unsigned long long* __restrict__ area, StencilCountArgs S,
                                                    uint32_t shared_lines, DeviceFlags* flags) {
    extern __shared__ int s_lines[];   // CX (W+1), CY (H+1) with shared_lines
    if (flags->poison) return;
    const uint32_t n = n_host ? n_host : (uint32_t)flags->n_gen_tris;
    const uint32_t n_launch = n_host ? n_host : P.gen_tri_cap;
    const bool counting = P.stencil_active && !P.mode_b;
    int* sx = S.lines;
    int* sy = S.lines + 3 * (P.W + 1);
    if (counting && shared_lines) {
        sx = s_lines;
        sy = s_lines + (P.W + 1);
        for (uint32_t i = threadIdx.x; i < P.W + P.H + 2; i += blockDim.x) s_lines[i] = 0;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    unsigned long long n_raster = 0, n_unsafe = 0, n_entries = 0;
    uint32_t nan_cnt = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n_launch; base += gridDim.x * blockDim.x) {
        const uint32_t t = base + threadIdx.x;
        // opaque path: bbox pixel counts instead of bins (zero past the last primitive)
        if (area && t >= n && t < n_launch) area[t] = 0;
        uint32_t single_bin = 0xfffffffeu;   // bin of a one-bin primitive (warp aggregation key)
        uint32_t entries_t = 0;
        uint32_t gmask = 0;   // stencil global counters this primitive increments
        uint32_t rx0 = 1, ry0 = 1, rx1 = 0, ry1 = 0;
        if (t < n) {
            uint32_t ia, ib, ic;
            tri_slots(t, vidx, ia, ib, ic);
            bool bad = n_host && (ia >= P.n_verts || ib >= P.n_verts || ic >= P.n_verts);
            if (bad) { atomicOr(&flags->bad_index, 1u); ia = ib = ic = 0; }
            float4 s0 = __ldg(scr4 + ia), s1 = __ldg(scr4 + ib), s2 = __ldg(scr4 + ic);
            float x1 = s0.x, y1 = s0.y, x2 = s1.x, y2 = s1.y, x3 = s2.x, y3 = s2.y;
            bool culled = false;
            if (P.cull) {
                float ar = x1 * y2 + x2 * y3 + x3 * y1 - x2 * y1 - x3 * y2 - x1 * y3;
                bool neg = !isnan(ar) && signbit(ar);
                uint32_t winding = neg ? 1u : 2u;
                culled = winding == P.cull;
            }
            culled = culled || bad;
            uint2 rect = make_uint2(RECT_EMPTY, RECT_EMPTY);
            if (area) area[t] = 0;
            // every primitive gets a record flag word (mode B walks all of them)
            setup[4 * (size_t)t + 2] = make_float4(0.0f, 0.0f, __uint_as_float(0u), 0.0f);
            if (!culled) {
                float det = (y2 - y3) * (x1 - x3) + (x3 - x2) * (y1 - y3);
                float mnx = sr_min(sr_min(x1, x2), x3), mny = sr_min(sr_min(y1, y2), y3);
                float mxx = sr_max(sr_max(x1, x2), x3), mxy = sr_max(sr_max(y1, y2), y3);
                if (isnan(mnx) || isnan(mny)) {
                    nan_cnt += 1;
                } else {
                    const int W = (int)P.W, H = (int)P.H;
                    int ix0 = floor_sat(mnx, -1, W), ix1 = floor_sat(mxx, -1, W);
                    int iy0 = floor_sat(mny, -1, H), iy1 = floor_sat(mxy, -1, H);
                    if (counting) gmask = stencil_count_tri(P, S, ix0, iy0, ix1, iy1, sx, sy);
                    bool no_frag = det == 0.0f || isnan(det) || (s0.z >= 0.0f && s1.z >= 0.0f && s2.z >= 0.0f);
                    if (!no_frag || P.mode_b) {
                        // the coverage region of an unsafe primitive bounds its
                        // fragments outside the bbox (the SR_FORCE_UNSAFE test hook
                        // leaves it unbounded, so every tile's segment is evaluated)
                        float4 region = make_float4(NAN, NAN, NAN, NAN);
                        bool safe = !P.mode_b && !P.force_unsafe &&
                                    inflated_region(x1, y1, x2, y2, x3, y3, det, P.W, P.H, ix0, iy0, ix1, iy1, &region);
                        if (P.force_unsafe) region = make_float4(NAN, NAN, NAN, NAN);
                        int qx0 = max(ix0, 0), qy0 = max(iy0, 0), qx1 = min(ix1, W - 1), qy1 = min(iy1, H - 1);
                        bool b_in = qx0 <= qx1 && qy0 <= qy1;
                        if (b_in || !safe) {
                            float4* r = setup + 4 * (size_t)t;
                            r[0] = make_float4(y2 - y3, x3 - x2, y3 - y1, x1 - x3);
                            r[1] = make_float4(x3, y3, det, s0.z);
                            uint32_t fl = REC_RASTER | (safe ? 0u : REC_UNSAFE);
                            r[2] = make_float4(s1.z, s2.z, __uint_as_float(fl), det_sign(det));
                            r[3] = make_float4(__int_as_float(ix0), __int_as_float(iy0), __int_as_float(ix1),
                                               __int_as_float(iy1));
                            n_raster += 1;
                            n_unsafe += safe ? 0 : 1;
                            if (area) {
                                area[t] = b_in ? (unsigned long long)(qx1 - qx0 + 1) * (unsigned long long)(qy1 - qy0 + 1) : 0ull;
                                if (!safe) {
                                    unsigned long long k = atomicAdd(&flags->n_unsafe_list, 1ull);
                                    unsafe_list[k] = t;
                                    if (unsafe_rect) unsafe_rect[k] = region;
                                }
                            } else if (!P.mode_b) {
                                if (b_in) {
                                    rx0 = (uint32_t)qx0 >> P.bin_w_log2; rx1 = (uint32_t)qx1 >> P.bin_w_log2;
                                    ry0 = (uint32_t)qy0 >> P.bin_h_log2; ry1 = (uint32_t)qy1 >> P.bin_h_log2;
                                    rect = make_uint2(rx0 | (ry0 << 16), rx1 | (ry1 << 16));
                                    entries_t = (rx1 - rx0 + 1) * (ry1 - ry0 + 1);
                                    n_entries += entries_t;
                                    if (rx0 == rx1 && ry0 == ry1) single_bin = ry0 * P.bins_x + rx0;
                                }
                                if (!safe) {
                                    unsigned long long k = atomicAdd(&flags->n_unsafe_list, 1ull);
                                    unsafe_list[k] = t;
                                    if (unsafe_rect) unsafe_rect[k] = region;
                                }
                            }
                        }
                    }
                }
            }
            binrect[t] = rect;
        }
        // bin counts: warp-aggregated for one-bin primitives
        if (bin_counts) {
            const unsigned peers = __match_any_sync(0xffffffffu, single_bin);
            if (single_bin < 0xfffffffeu) {
                if (lane == __ffs(peers) - 1) atomicAdd(bin_counts + single_bin, (uint32_t)__popc(peers));
            } else if (entries_t && entries_t <= 16) {
                for (uint32_t by = ry0; by <= ry1; ++by)
                    for (uint32_t bx = rx0; bx <= rx1; ++bx) atomicAdd(bin_counts + by * P.bins_x + bx, 1u);
            }
            // bin rectangles of more than 16 bins: the warp's lanes share each one's bins
            uint32_t big = __ballot_sync(0xffffffffu, entries_t > 16);
            while (big) {
                const uint32_t src = __ffs(big) - 1;
                big &= big - 1;
                const uint32_t bx0 = __shfl_sync(0xffffffffu, rx0, src), by0 = __shfl_sync(0xffffffffu, ry0, src);
                const uint32_t bw = __shfl_sync(0xffffffffu, rx1, src) - bx0 + 1;
                const uint32_t nb = __shfl_sync(0xffffffffu, entries_t, src);
                for (uint32_t i = lane; i < nb; i += 32)
                    atomicAdd(bin_counts + (by0 + i / bw) * P.bins_x + bx0 + i % bw, 1u);
            }
        }
        // stencil global counters, one atomic per warp and counter
        if (counting) {
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const unsigned m = __ballot_sync(0xffffffffu, (gmask >> k) & 1u);
                if (lane == 0 && m) atomicAdd(S.globals + k, (unsigned long long)__popc(m));
            }
        }
    }
    if (counting && shared_lines) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i <= P.W; i += blockDim.x)
            if (s_lines[i]) atomicAdd(S.lines + i, s_lines[i]);
        for (uint32_t i = threadIdx.x; i <= P.H; i += blockDim.x)
            if (s_lines[P.W + 1 + i]) atomicAdd(S.lines + 3 * (P.W + 1) + i, s_lines[P.W + 1 + i]);
    }
    // statistics: per-warp sums
    const unsigned long long w_raster = warp_sum_u64(n_raster);
    const unsigned long long w_unsafe = warp_sum_u64(n_unsafe);
    const unsigned long long w_entries = warp_sum_u64(n_entries);
    const uint32_t w_nan = __reduce_add_sync(0xffffffffu, nan_cnt);
    if (lane == 0) {
        if (w_raster) atomicAdd(&flags->triangles_raster, w_raster);
        if (w_unsafe) atomicAdd(&flags->unsafe, w_unsafe);
        if (w_entries) atomicAdd(&flags->entries, w_entries);
        if (w_nan) { atomicAdd(&flags->nan_bbox, w_nan); atomicAdd(&flags->nan_total, w_nan); }
    }
}

// CX and CY in shared memory while the frame's W + H + 2 counters fit in this
// many bytes (a 6,142 x 6,142 frame); larger frames add to the global arrays.
constexpr size_t SETUP_LINES_SMEM = 48 * 1024;

void launch_setup_bin(const DrawParams& P, const uint32_t* vidx, VertexStore vs, float4* setup, uint32_t* binrect,
                      uint32_t* bin_counts, uint32_t* bin_off, uint32_t* bin_cursor, uint32_t* entries,
                      uint32_t* scan_tmp, uint32_t* unsafe_list, float4* unsafe_rect, unsigned long long* area,
                      const StencilCountArgs& S, DeviceFlags* flags, cudaStream_t st) {
    uint32_t n_host = P.n_raster_host;
    uint32_t n_launch = n_host ? n_host : P.gen_tri_cap;
    dim3 block(256), grid((n_launch + 255) / 256 ? (n_launch + 255) / 256 : 1);
    const bool counting = P.stencil_active && !P.mode_b;
    const size_t smem = counting ? ((size_t)P.W + P.H + 2) * sizeof(int) : 0;
    uint32_t shared_lines = 0;
    if (counting && smem <= SETUP_LINES_SMEM) {
        // a resident grid, so each CTA adds its counters once over many primitives
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, setup_kernel, 256, smem) != cudaSuccess || nb <= 0)
            nb = 1;
        const uint32_t g = (uint32_t)nb * (uint32_t)sm_count();
        if (grid.x > g) grid.x = g;
        shared_lines = 1;
    }
    const size_t dyn = shared_lines ? smem : 0;
    // opaque key-buffer path: bbox pixel counts, no bins; binned opaque path:
    // setup counts each bin's primitives; ordered path (bin_counts null):
    // setup only, bins are built by launch_bins (sr_bins.cu)
    setup_kernel<<<grid, block, dyn, st>>>(P, n_host, vidx, vs.scr4, setup, reinterpret_cast<uint2*>(binrect),
                                           area ? nullptr : bin_counts, unsafe_list, unsafe_rect, area, S,
                                           shared_lines, flags);
    (void)bin_off; (void)bin_cursor; (void)entries; (void)scan_tmp;
}


}  // namespace sr
