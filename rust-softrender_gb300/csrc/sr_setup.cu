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

constexpr uint32_t RECT_EMPTY = 0xffffffffu;

__device__ __forceinline__ void stencil_count_tri(const DrawParams& P, const StencilCountArgs& S, int ix0,
                                                  int iy0, int ix1, int iy1) {
    const int W = (int)P.W, H = (int)P.H;
    int x0 = max(ix0, 0), x1 = min(ix1, W - 1), y0 = max(iy0, 0), y1 = min(iy1, H - 1);
    bool xin = x0 <= x1, yin = y0 <= y1;
    int* CX = S.lines;
    int* CXa = CX + (W + 1);
    int* CXb = CXa + (W + 1);
    int* CY = CXb + (W + 1);
    int* CYl = CY + (H + 1);
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
    atomicAdd(S.globals + 0, 1ull);
    if (L) atomicAdd(S.globals + 1, 1ull);
    if (R) atomicAdd(S.globals + 2, 1ull);
    if (A) atomicAdd(S.globals + 3, 1ull);
    if (B) atomicAdd(S.globals + 4, 1ull);
    if (L && A) atomicAdd(S.globals + 5, 1ull);
    if (L && B) atomicAdd(S.globals + 6, 1ull);
    if (R && A) atomicAdd(S.globals + 7, 1ull);
    if (R && B) atomicAdd(S.globals + 8, 1ull);
}

// One thread per raster triangle: setup record, bin rectangle, bin counts,
// and (when the stencil changes under Always) the stencil event counts.
__global__ void __launch_bounds__(256) setup_kernel(DrawParams P, uint32_t n_host, const uint32_t* __restrict__ vidx,
                                                    const float4* __restrict__ scr4, float4* __restrict__ setup,
                                                    uint2* __restrict__ binrect, uint32_t* __restrict__ bin_counts,
                                                    uint32_t* __restrict__ unsafe_list,
                                                    unsigned long long* __restrict__ area, StencilCountArgs S,
                                                    DeviceFlags* flags) {
    if (flags->poison) return;
    uint32_t n = n_host ? n_host : (uint32_t)flags->n_gen_tris;
    if (area) {   // opaque path: bbox pixel counts instead of bins (zero past the last primitive)
        const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
        const uint32_t n_launch = n_host ? n_host : P.gen_tri_cap;
        if (t0 >= n && t0 < n_launch) area[t0] = 0;
    }
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint32_t single_bin = 0xfffffffeu;   // bin of a one-bin primitive (warp aggregation key)
    unsigned long long n_raster = 0, n_unsafe = 0, n_entries = 0;
    uint32_t nan_cnt = 0;
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
                nan_cnt = 1;
            } else {
                const int W = (int)P.W, H = (int)P.H;
                int ix0 = floor_sat(mnx, -1, W), ix1 = floor_sat(mxx, -1, W);
                int iy0 = floor_sat(mny, -1, H), iy1 = floor_sat(mxy, -1, H);
                if (P.stencil_active && !P.mode_b) stencil_count_tri(P, S, ix0, iy0, ix1, iy1);
                bool no_frag = det == 0.0f || isnan(det) || (s0.z >= 0.0f && s1.z >= 0.0f && s2.z >= 0.0f);
                if (!no_frag || P.mode_b) {
                    bool safe = !P.mode_b && !P.force_unsafe && inflated_region(x1, y1, x2, y2, x3, y3, det, P.W, P.H, ix0, iy0, ix1, iy1);
                    int qx0 = max(ix0, 0), qy0 = max(iy0, 0), qx1 = min(ix1, W - 1), qy1 = min(iy1, H - 1);
                    bool b_in = qx0 <= qx1 && qy0 <= qy1;
                    if (b_in || !safe) {
                        float4* r = setup + 4 * (size_t)t;
                        r[0] = make_float4(y2 - y3, x3 - x2, y3 - y1, x1 - x3);
                        r[1] = make_float4(x3, y3, det, s0.z);
                        uint32_t fl = REC_RASTER | (safe ? 0u : REC_UNSAFE);
                        r[2] = make_float4(s1.z, s2.z, __uint_as_float(fl), 0.0f);
                        r[3] = make_float4(__int_as_float(ix0), __int_as_float(iy0), __int_as_float(ix1),
                                           __int_as_float(iy1));
                        n_raster = 1;
                        n_unsafe = safe ? 0 : 1;
                        if (area) {
                            area[t] = b_in ? (unsigned long long)(qx1 - qx0 + 1) * (unsigned long long)(qy1 - qy0 + 1) : 0ull;
                            if (!safe) {
                                unsigned long long k = atomicAdd(&flags->n_unsafe_list, 1ull);
                                unsafe_list[k] = t;
                            }
                        } else if (!P.mode_b) {
                            if (b_in) {
                                rx0 = (uint32_t)qx0 >> P.bin_w_log2; rx1 = (uint32_t)qx1 >> P.bin_w_log2;
                                ry0 = (uint32_t)qy0 >> P.bin_h_log2; ry1 = (uint32_t)qy1 >> P.bin_h_log2;
                                rect = make_uint2(rx0 | (ry0 << 16), rx1 | (ry1 << 16));
                                n_entries = (unsigned long long)(rx1 - rx0 + 1) * (ry1 - ry0 + 1);
                                if (rx0 == rx1 && ry0 == ry1) single_bin = ry0 * P.bins_x + rx0;
                            }
                            if (!safe) {
                                unsigned long long k = atomicAdd(&flags->n_unsafe_list, 1ull);
                                unsafe_list[k] = t;
                            }
                        }
                    }
                }
            }
        }
        binrect[t] = rect;
    }
    // bin counts: warp-aggregated for one-bin primitives
    unsigned peers = __match_any_sync(0xffffffffu, single_bin);
    if (single_bin < 0xfffffffeu) {
        if (lane == __ffs(peers) - 1) atomicAdd(bin_counts + single_bin, (uint32_t)__popc(peers));
    } else if (n_entries) {
        for (uint32_t by = ry0; by <= ry1; ++by)
            for (uint32_t bx = rx0; bx <= rx1; ++bx) atomicAdd(bin_counts + by * P.bins_x + bx, 1u);
    }
    // statistics
    for (int o = 16; o > 0; o >>= 1) {
        n_raster += __shfl_down_sync(0xffffffffu, n_raster, o);
        n_unsafe += __shfl_down_sync(0xffffffffu, n_unsafe, o);
        n_entries += __shfl_down_sync(0xffffffffu, n_entries, o);
        nan_cnt += __shfl_down_sync(0xffffffffu, nan_cnt, o);
    }
    if (lane == 0) {
        if (n_raster) atomicAdd(&flags->triangles_raster, n_raster);
        if (n_unsafe) atomicAdd(&flags->unsafe, n_unsafe);
        if (n_entries) atomicAdd(&flags->entries, n_entries);
        if (nan_cnt) { atomicAdd(&flags->nan_bbox, nan_cnt); atomicAdd(&flags->nan_total, nan_cnt); }
    }
}

__global__ void __launch_bounds__(256) bin_fill_kernel(DrawParams P, uint32_t n_host, const uint2* __restrict__ binrect,
                                                       const uint32_t* __restrict__ bin_off, uint32_t* __restrict__ cursor,
                                                       uint32_t* __restrict__ entries, uint64_t entry_cap,
                                                       DeviceFlags* flags) {
    if (flags->poison) return;
    uint32_t n = n_host ? n_host : (uint32_t)flags->n_gen_tris;
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint2 rect = make_uint2(RECT_EMPTY, RECT_EMPTY);
    if (t < n) rect = binrect[t];
    uint32_t single_bin = 0xfffffffeu;
    uint32_t rx0 = 0, ry0 = 0, rx1 = 0, ry1 = 0;
    bool any = rect.x != RECT_EMPTY;
    if (any) {
        rx0 = rect.x & 0xffffu; ry0 = rect.x >> 16; rx1 = rect.y & 0xffffu; ry1 = rect.y >> 16;
        if (rx0 == rx1 && ry0 == ry1) single_bin = ry0 * P.bins_x + rx0;
    }
    unsigned peers = __match_any_sync(0xffffffffu, single_bin);
    if (single_bin < 0xfffffffeu) {
        int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(cursor + single_bin, (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        uint32_t pos = base + __popc(peers & ((1u << lane) - 1u));
        uint64_t at = (uint64_t)bin_off[single_bin] + pos;
        if (at < entry_cap) entries[at] = t;
    } else if (any) {
        for (uint32_t by = ry0; by <= ry1; ++by)
            for (uint32_t bx = rx0; bx <= rx1; ++bx) {
                uint32_t b = by * P.bins_x + bx;
                uint32_t pos = atomicAdd(cursor + b, 1u);
                uint64_t at = (uint64_t)bin_off[b] + pos;
                if (at < entry_cap) entries[at] = t;
            }
    }
}


// ------------------------------------------------------- extension pass
// An unsafe primitive can produce fragments outside its bbox, but only at
// the pixels where the reference evaluates it there: the projection of its
// bbox onto each semantic tile it does not overlap (a column segment, a row
// segment or a corner pixel on that tile's edge).  For each such segment a
// sound sign test clears the whole segment when one of u, v, w is certainly
// negative on it; remaining pixels are evaluated exactly (the reference's
// expressions), and the primitive is added to the bin of every pixel that
// yields a fragment, unless that bin already lists it.
//
// Sign test: the reference's numerator n_u(P) differs from the exact edge
// function N_u(P) by at most gamma_4 * S_u(P), S_u = |y2-y3||x-x3| + |x3-x2||y-y3|
// (convex on the segment, so its maximum is at an end point).  N_u is affine,
// so s*n_u(end) + 2 gamma_4 max S_u < 0 at both ends (s = sign of the computed
// det) makes u < 0 on the whole segment; v likewise.  For w = (1-u)-v the
// quantity det - N_u - N_v is affine and w < 0 follows when it is negative
// beyond the numerator errors plus 8 eps |det| (the roundings of the two
// quotients and two subtractions while u, v lie in [0, 2]; outside that range
// u < 0, v < 0 or w < 0 holds anyway).
__device__ __forceinline__ uint32_t clampu(int v, uint32_t lo, uint32_t hi) {
    return v < (int)lo ? lo : (v > (int)hi ? hi : (uint32_t)v);
}

template <bool FILL>
__global__ void __launch_bounds__(256) ext_kernel(DrawParams P, const uint32_t* __restrict__ unsafe_list,
                                                  const float4* __restrict__ setup, const uint2* __restrict__ binrect,
                                                  uint32_t* __restrict__ bin_counts, const uint32_t* __restrict__ bin_off,
                                                  uint32_t* __restrict__ cursor, uint32_t* __restrict__ entries,
                                                  uint64_t entry_cap, DeviceFlags* flags) {
    if (flags->poison) return;
    const uint32_t nu = (uint32_t)flags->n_unsafe_list;
    const uint32_t ntiles = P.ncols * P.nrows;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long emitted = 0;
    for (uint32_t k = warp; k < nu; k += nwarps) {
        const uint32_t t = unsafe_list[k];
        const float4* r = setup + 4 * (size_t)t;
        const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
        const int ix0 = __float_as_int(r3.x), iy0 = __float_as_int(r3.y);
        const int ix1 = __float_as_int(r3.z), iy1 = __float_as_int(r3.w);
        const uint2 br = binrect[t];
        const bool has_rect = br.x != RECT_EMPTY;
        const uint32_t bx0 = br.x & 0xffffu, by0 = br.x >> 16, bx1 = br.y & 0xffffu, by1 = br.y >> 16;
        for (uint32_t ti = lane; ti < ntiles; ti += 32) {
            const uint32_t C = ti % P.ncols, R = ti / P.ncols;
            const uint32_t lx = C * P.tile_w, hx = min((C + 1) * P.tile_w, P.W - 1);
            const uint32_t ly = R * P.tile_h, hy = min((R + 1) * P.tile_h, P.H - 1);
            const bool ox = ix1 >= (int)lx && ix0 <= (int)hx;
            const bool oy = iy1 >= (int)ly && iy0 <= (int)hy;
            if (ox && oy) continue;   // bbox meets the tile: those pixels lie in the bbox bins
            const uint32_t cx0 = clampu(ix0, lx, hx), cx1 = clampu(ix1, lx, hx);
            const uint32_t cy0 = clampu(iy0, ly, hy), cy1 = clampu(iy1, ly, hy);
            if (segment_cleared(r0, r1, cx0, cy0, cx1, cy1)) continue;
            uint32_t last_b = 0xffffffffu;
            for (uint32_t py = cy0; py <= cy1; ++py) {
                for (uint32_t px = cx0; px <= cx1; ++px) {
                    float x = (float)px + 0.5f, y = (float)py + 0.5f;
                    float dx = x - r1.x, dy = y - r1.y;
                    float u = (r0.x * dx + r0.y * dy) / r1.z;
                    float v = (r0.z * dx + r0.w * dy) / r1.z;
                    float w = 1.0f - u - v;
                    if (u < 0.0f || v < 0.0f || w < 0.0f) continue;
                    float z = (r1.w * u + r2.x * v) + r2.y * w;
                    if (!(z < 0.0f)) continue;
                    const uint32_t bxx = px >> P.bin_w_log2, byy = py >> P.bin_h_log2;
                    if (has_rect && bxx >= bx0 && bxx <= bx1 && byy >= by0 && byy <= by1) continue;
                    const uint32_t b = byy * P.bins_x + bxx;
                    if (b == last_b) continue;
                    last_b = b;
                    if (FILL) {
                        uint32_t pos = atomicAdd(cursor + b, 1u);
                        uint64_t at = (uint64_t)bin_off[b] + pos;
                        if (at < entry_cap) entries[at] = t;
                    } else {
                        atomicAdd(bin_counts + b, 1u);
                        ++emitted;
                    }
                }
            }
        }
    }
    if (!FILL && emitted) atomicAdd(&flags->entries, emitted);
}

__global__ void check_entries_kernel(uint32_t n_bins, const uint32_t* bin_off, uint64_t entry_cap, uint32_t draw_id,
                                     DeviceFlags* flags) {
    if (flags->poison) return;
    unsigned long long tot = bin_off[n_bins];
    if (tot > flags->need_entries) flags->need_entries = tot;
    if (tot > entry_cap) {
        atomicOr(&flags->overflow_bits, (unsigned)OVF_ENTRIES);
        atomicOr(&flags->poison, 1u); atomicMin(&flags->poison_draw, draw_id);
    }
}

void launch_setup_bin(const DrawParams& P, const uint32_t* vidx, VertexStore vs, float4* setup, uint32_t* binrect,
                      uint32_t* bin_counts, uint32_t* bin_off, uint32_t* bin_cursor, uint32_t* entries,
                      uint32_t* scan_tmp, uint32_t* unsafe_list, unsigned long long* area, const StencilCountArgs& S,
                      DeviceFlags* flags, cudaStream_t st) {
    uint32_t n_bins = P.bins_x * P.bins_y;
    uint32_t n_host = P.n_raster_host;
    uint32_t n_launch = n_host ? n_host : P.gen_tri_cap;
    dim3 block(256), grid((n_launch + 255) / 256 ? (n_launch + 255) / 256 : 1);
    if (area) {   // opaque path: no bins
        setup_kernel<<<grid, block, 0, st>>>(P, n_host, vidx, vs.scr4, setup, reinterpret_cast<uint2*>(binrect),
                                             bin_counts, unsafe_list, area, S, flags);
        return;
    }
    cudaMemsetAsync(bin_counts, 0, (size_t)n_bins * 4, st);
    cudaMemsetAsync(bin_cursor, 0, (size_t)n_bins * 4, st);
    setup_kernel<<<grid, block, 0, st>>>(P, n_host, vidx, vs.scr4, setup, reinterpret_cast<uint2*>(binrect),
                                         bin_counts, unsafe_list, nullptr, S, flags);
    const uint2* br = reinterpret_cast<const uint2*>(binrect);
    const dim3 ext_grid(4 * 152);
    if (!P.mode_b)
        ext_kernel<false><<<ext_grid, block, 0, st>>>(P, unsafe_list, setup, br, bin_counts, bin_off, bin_cursor,
                                                      entries, P.entry_cap, flags);
    exclusive_scan<uint32_t>(bin_counts, n_bins, bin_off, scan_tmp, st);
    check_entries_kernel<<<1, 1, 0, st>>>(n_bins, bin_off, P.entry_cap, P.draw_id, flags);
    bin_fill_kernel<<<grid, block, 0, st>>>(P, n_host, br, bin_off, bin_cursor, entries, P.entry_cap, flags);
    if (!P.mode_b)
        ext_kernel<true><<<ext_grid, block, 0, st>>>(P, unsafe_list, setup, br, bin_counts, bin_off, bin_cursor,
                                                     entries, P.entry_cap, flags);
}

}  // namespace sr
