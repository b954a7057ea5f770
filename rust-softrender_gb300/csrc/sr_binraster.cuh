// sr_binraster.cuh — one work item of the binned opaque raster: a chunk of
// up to 256 primitives of one 32x32 screen bin, reduced to each pixel's
// winner key in shared memory.  Shared by the per-draw kernel (sr_tiled.cu)
// and the batched one (sr_batch.cu).
#pragma once
#include "sr_internal.cuh"
#include "sr_scan.cuh"
#include "sr_opaque.cuh"

namespace sr {

constexpr uint32_t TL_THREADS = 256;
constexpr uint32_t TL_WARPS = TL_THREADS / 32;
constexpr uint32_t TL_BIN_LOG2 = 5;   // bins of 32 x 32 pixels (the touched-block bitmap's granularity)
static_assert(TL_BIN_LOG2 == TOUCH_LOG2, "the extension keys' bitmap marks bins");
constexpr uint32_t TL_CHUNK = TL_THREADS;   // primitives a raster work item stages (one per thread)
static_assert(TL_CHUNK == BIN_CHUNK, "work items of the bin scans");
constexpr uint32_t TL_QCAP = 64;            // pixels a warp's stack holds: 31 waiting + 32 pushed

// Per staged primitive, the sign pre-test's three rejection thresholds (see
// bin_item); the edge coefficients, anchor and det come from the setup
// record, the sign s from its last word.
struct PreRec {
    float tu, tv, tw;
};

// The shared memory of one CTA working on a bin item.
struct BinSmem {
    unsigned long long keys[1u << (2 * TL_BIN_LOG2)];   // the bin's winner keys
    float4 srec[TL_CHUNK][3];
    PreRec spre[TL_CHUNK];
    uint32_t sst[TL_CHUNK + 1];            // first row of each primitive; [n] = rows
    uint32_t sxy[TL_CHUNK];                // x0 | y0 << 16 (bin-relative) | seam bits 15, 31
    uint32_t sw[TL_CHUNK];                 // clipped width
    uint32_t st[TL_CHUNK];                 // primitive index
    uint32_t squeue[TL_WARPS][TL_QCAP];    // pixels waiting for the exact test: chunk slot << 10 | y << 5 | x
    uint32_t next_row;                     // the next window of rows a warp takes
};

// Work item = one chunk of up to TL_CHUNK primitives of one 32x32 bin's list.
// For the item the CTA reduces the winner key of each pixel of the bin in
// shared memory; a bin with one item (`whole`) writes the keys' low words
// (pass * N + primitive + 1, 0 for no fragment) to its 1024 slots `gids`, or,
// without slots, its non-zero keys to the per-pixel key buffer `gkeys`; a bin
// with several items -- a long list, as a dense mesh on a small frame gives --
// merges each non-zero key into `gkeys` with a 64-bit atomicMax.  With `seed`
// (a bin in one item whose pixels already hold keys in `gkeys`: extension
// fragments, large primitives) the reduction starts from those keys.
//
// Rows.  Each chunk primitive's bbox clipped to the bin gives its rows; a
// CTA-wide scan numbers them, and the warps take windows of 32 rows from a
// shared counter.  Every listed primitive's bbox meets its bin, so every
// primitive of a chunk has rows and their first rows are strictly increasing:
// a warp finds the owner of its window's first row by binary search and the
// primitives starting inside the window from one load per lane.  Each lane reduces its row to the span of pixels that can be
// covered; the window's spans go onto a per-warp stack in shared memory, and
// whenever 32 wait the whole warp evaluates them exactly (frag_key: the
// reference's divisions, z, the key) with every lane busy.
//
// Spans.  With s = det_sign(det) (non-zero for 0 < |det| < 1e18) and the
// edge coefficients A, B (u) and C, D (v), the reference's numerators differ
// from the exact edge functions Nu = A (x - x3) + B (y - y3) (Nv alike) by at
// most 3.0001 2^-24 S, S = |A| Xr + |B| Yr over the clipped bbox (Xr, Yr
// bounding |x - x3|, |y - y3|): the rounding of x - x3, of the two products
// and of the sum.  At the row's first pixel, eu0 = (sA) dx + (sB) dy with the
// reference's operations is exactly s nu there, so along the row (pixel k)
//   covered  =>  s nu >= -1e-18            (else u = nu/det rounds below 0)
//            =>  s Nu(k) >= -1e-18 - 3.0001 2^-24 Su
//            =>  eu0 + k sA >= -(1e-18 + 6.0002 2^-24 Su) >= -tu,
// tu = 1e-18 + 2^-20 Su, in real arithmetic (s Nu steps by exactly sA); v
// alike.  For w = (1-u)-v, covered means w's unrounded value is at least
// -2^-150 (a w of -0 passes), so s (det - nu - nv) >= -2^-24 (|det| + 2|nu| +
// |nv|) - 2^-140 |det| (frag_key's third-edge argument) and, with
// ew0 = (|det| - eu0) - ev0 evaluated in f32,
//   ew0 - k (sA + sC) >= -(2^-24 (3|det| + 10.0002 Su + 9.0002 Sv) + 2^-140 |det|)
//                     >= -tw,  tw = 2^-20 (|det| + Su + Sv) + 2^-140 |det|.
// Each of the three conditions bounds k on one side: k >= (-T - e0) / g for
// g > 0, k <= (-T - e0) / g for g < 0, nothing or no pixel for g = 0.  The
// bound is computed in f32 (two roundings: at most 2^-22 |k| off for |k| <=
// 64, and the rounded slope of the w edge shifts it by at most 31 2^-24) and
// moved outwards by 10^-4 pixel, so the span holds every pixel of the row
// that can be covered; a non-finite value keeps the whole row.
__device__ __forceinline__ void bin_item(BinSmem& sm, const DrawParams& P, uint32_t X0, uint32_t Y0,
                                         const float4* __restrict__ setup, const uint32_t* __restrict__ list,
                                         uint32_t n, uint32_t N, const uint8_t* __restrict__ stencil,
                                         uint32_t gate_with_stencil, bool whole, bool seed,
                                         unsigned long long* __restrict__ gkeys, uint32_t* __restrict__ gids,
                                         unsigned long long& frags) {
    const uint32_t lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;   // lanes below this one
    const uint32_t mx = P.magic_w, my = P.magic_h;
    const uint32_t X1 = min(X0 + (1u << TL_BIN_LOG2) - 1, P.W - 1), Y1 = min(Y0 + (1u << TL_BIN_LOG2) - 1, P.H - 1);
    for (uint32_t i = threadIdx.x; i < (1u << (2 * TL_BIN_LOG2)); i += TL_THREADS) {
        unsigned long long k = 0;
        if (seed) {   // seed with the bin's keys already in gkeys (they stay there otherwise)
            const uint32_t px = X0 + (i & 31), py = Y0 + (i >> TL_BIN_LOG2);
            if (px <= X1 && py <= Y1) {
                const size_t gi = (size_t)py * P.W + px;
                k = gkeys[gi];
                if (k && gids) gkeys[gi] = 0;
            }
        }
        sm.keys[i] = k;
    }
    uint32_t a = 0;
    if (threadIdx.x < n) {
        const uint32_t t = __ldg(list + threadIdx.x);
        const float4* r = setup + 4 * (size_t)t;
        const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
        const uint32_t x0 = (uint32_t)max(__float_as_int(r3.x), (int)X0);
        const uint32_t y0 = (uint32_t)max(__float_as_int(r3.y), (int)Y0);
        const uint32_t x1 = (uint32_t)min(__float_as_int(r3.z), (int)X1);
        const uint32_t y1 = (uint32_t)min(__float_as_int(r3.w), (int)Y1);
        const uint32_t w = x1 - x0 + 1;
        a = y1 - y0 + 1;   // the primitive's rows in the bin
        sm.srec[threadIdx.x][0] = r0;
        sm.srec[threadIdx.x][1] = r1;
        sm.srec[threadIdx.x][2] = r2;
        PreRec pr;
        if (r2.w != 0.0f) {
            // bounds of |x - x3| and |y - y3| over the clipped bbox's pixel centres
            const float xr = fmaxf(fabsf(((float)x0 + 0.5f) - r1.x), fabsf(((float)x1 + 0.5f) - r1.x)) * 1.001f;
            const float yr = fmaxf(fabsf(((float)y0 + 0.5f) - r1.y), fabsf(((float)y1 + 0.5f) - r1.y)) * 1.001f;
            const float su = fabsf(r0.x) * xr + fabsf(r0.y) * yr, sv = fabsf(r0.z) * xr + fabsf(r0.w) * yr;
            const float ad = fabsf(r1.z);
            pr.tu = 1.0e-18f + 0x1p-20f * su;
            pr.tv = 1.0e-18f + 0x1p-20f * sv;
            pr.tw = 0x1p-20f * ((ad + su) + sv) + 0x1p-140f * ad;
        } else {   // no sign information: keep every pixel for the exact test
            const float INF = __int_as_float(0x7f800000);
            pr.tu = INF; pr.tv = INF; pr.tw = INF;
        }
        sm.spre[threadIdx.x] = pr;
        const uint32_t sb = seam_bits(x0, y0, x1, y1, P);
        sm.sxy[threadIdx.x] = (x0 - X0) | ((y0 - Y0) << 16) | ((sb & 1u) << 15) | ((sb & 2u) << 30);
        sm.sw[threadIdx.x] = w;
        sm.st[threadIdx.x] = t;
    }
    uint32_t total;
    const uint32_t ex = block_exclusive_scan<uint32_t, TL_THREADS>(a, &total);
    if (threadIdx.x < n) sm.sst[threadIdx.x] = ex;
    if (threadIdx.x == 0) {
        sm.sst[n] = total;
        sm.next_row = 0;
    }
    __syncthreads();
    // windows of 32 rows, taken by the warps one at a time from a shared
    // counter (rows differ in cost, so equal shares would leave warps waiting)
    const uint32_t q1 = total;
    uint32_t qn = 0;   // pixels waiting on the warp's stack (warp-uniform, < 32 between rounds)
    const float INF = __int_as_float(0x7f800000);
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&sm.next_row, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= q1) break;
        // the owner of row `base`: the last primitive whose first row is <= base
        uint32_t cur = 0;
        {
            uint32_t lo = 0, hi = n;   // sm.sst[lo] <= base < sm.sst[hi]
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (sm.sst[mid] <= base) lo = mid; else hi = mid;
            }
            cur = lo;
        }
        // primitives cur+1 .. cur+32 that start inside [base, base + 32)
        const uint32_t j = cur + 1 + lane;
        const uint32_t sj = j < n ? sm.sst[j] : 0xffffffffu;
        const uint32_t starts = __reduce_or_sync(0xffffffffu, sj - base < 32u ? (1u << (sj - base)) : 0u);
        const uint32_t o = cur + __popc(starts & (lt | (1u << lane)));
        const uint32_t q = base + lane;
        // this lane's row: the span [ka, kb] of its pixels that can be covered
        uint32_t len = 0, pinfo = 0;
        if (q < q1) {
            const uint32_t w = sm.sw[o], xy = sm.sxy[o];
            const uint32_t lx0 = xy & 0x7fffu, ly = ((xy >> 16) & 0x7fffu) + (q - sm.sst[o]);
            const PreRec pr = sm.spre[o];
            float klo = 0.0f, khi = (float)(w - 1);
            if (pr.tu < INF) {
                const float4 r0 = sm.srec[o][0], r1 = sm.srec[o][1];
                const float sg = sm.srec[o][2].w;   // det_sign(det)
                const float sa = sg * r0.x, sb = sg * r0.y, sc = sg * r0.z, sd = sg * r0.w, ad = sg * r1.z;
                const float dx = ((float)(X0 + lx0) + 0.5f) - r1.x;
                const float dy = ((float)(Y0 + ly) + 0.5f) - r1.y;
                const float eu0 = sa * dx + sb * dy, ev0 = sc * dx + sd * dy;
                const float ew0 = (ad - eu0) - ev0, gw = -(sa + sc);
                if (fabsf(eu0) < INF && fabsf(ev0) < INF && fabsf(ew0) < INF && fabsf(gw) < INF) {
                    // pixel k of the row can be covered only if e0 + k g >= -T on
                    // every edge (real arithmetic; see the span argument above)
                    const float e0[3] = {eu0, ev0, ew0}, g[3] = {sa, sc, gw}, T[3] = {pr.tu, pr.tv, pr.tw};
#pragma unroll
                    for (int e = 0; e < 3; ++e) {
                        if (g[e] > 0.0f) klo = fmaxf(klo, (-T[e] - e0[e]) / g[e] - 1.0e-4f);
                        else if (g[e] < 0.0f) khi = fminf(khi, (-T[e] - e0[e]) / g[e] + 1.0e-4f);
                        else if (e0[e] < -T[e]) khi = -1.0f;
                    }
                }
            }
            const uint32_t ka = (uint32_t)ceilf(fminf(klo, 64.0f));
            const int kb = (int)floorf(fmaxf(khi, -1.0f));
            len = kb >= (int)ka ? (uint32_t)(kb - (int)ka + 1) : 0u;
            pinfo = (o << 10) | (ly << 5) | (lx0 + ka);
        }
        // the window's spans onto the stack, 32 pixels per round, each round
        // followed by exact evaluation of the full 32s (lanes spread over the
        // pixels: a pixel's span is the last lane starting at or before it)
        const uint32_t incl = warp_inclusive_scan(len);
        const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31), st_l = incl - len;
        for (uint32_t done = 0; done < tot; ) {
            const uint32_t m = min(tot - done, 32u);
            const uint32_t p = done + lane;
            uint32_t jl = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, st_l, jl + step) <= p) jl += step;
            const uint32_t info = __shfl_sync(0xffffffffu, pinfo, jl), sjl = __shfl_sync(0xffffffffu, st_l, jl);
            if (lane < m) sm.squeue[wl][qn + lane] = info + (p - sjl);
            qn += m;
            done += m;
            __syncwarp();
            // exact evaluation, 32 pixels at a time from the top of the stack
            while (qn >= 32) {
                const uint32_t e = sm.squeue[wl][qn - 32 + lane];
                const uint32_t oo = e >> 10, ex_ = e & 31u, ey = (e >> 5) & 31u;
                const uint32_t xy = sm.sxy[oo];
                const uint32_t seams = ((xy >> 15) & 1u) | ((xy >> 30) & 2u);
                const unsigned long long k =
                    frag_key(P.W, P.H, P.tile_w, P.tile_h, mx, my, seams, P.has_depth != 0, sm.srec[oo][0],
                             sm.srec[oo][1], sm.srec[oo][2], sm.st[oo], X0 + ex_, Y0 + ey, N, stencil, gate_with_stencil,
                             P.stencil_test, P.sref, frags);
                if (k) atomicMax(sm.keys + (ey << TL_BIN_LOG2) + ex_, k);
                qn -= 32;
                __syncwarp();
            }
        }
    }
    // what is left on the stack after the warp's last window
    if (qn) {
        if (lane < qn) {
            const uint32_t e = sm.squeue[wl][lane];
            const uint32_t oo = e >> 10, ex_ = e & 31u, ey = (e >> 5) & 31u;
            const uint32_t xy = sm.sxy[oo];
            const uint32_t seams = ((xy >> 15) & 1u) | ((xy >> 30) & 2u);
            const unsigned long long k =
                frag_key(P.W, P.H, P.tile_w, P.tile_h, mx, my, seams, P.has_depth != 0, sm.srec[oo][0],
                         sm.srec[oo][1], sm.srec[oo][2], sm.st[oo], X0 + ex_, Y0 + ey, N, stencil, gate_with_stencil,
                         P.stencil_test, P.sref, frags);
            if (k) atomicMax(sm.keys + (ey << TL_BIN_LOG2) + ex_, k);
        }
        __syncwarp();
    }
    __syncthreads();   // every warp's keys are final
    if (whole && gids) {
        for (uint32_t i = threadIdx.x; i < (1u << (2 * TL_BIN_LOG2)); i += TL_THREADS)
            gids[i] = (uint32_t)(sm.keys[i] & 0xffffffffull);
    } else if (whole) {
        for (uint32_t i = threadIdx.x; i < (1u << (2 * TL_BIN_LOG2)); i += TL_THREADS) {
            const unsigned long long k = sm.keys[i];
            if (k) gkeys[(size_t)(Y0 + (i >> TL_BIN_LOG2)) * P.W + X0 + (i & 31)] = k;
        }
    } else {
        for (uint32_t i = threadIdx.x; i < (1u << (2 * TL_BIN_LOG2)); i += TL_THREADS) {
            const unsigned long long k = sm.keys[i];
            if (k) atomicMax(gkeys + (size_t)(Y0 + (i >> TL_BIN_LOG2)) * P.W + X0 + (i & 31), k);
        }
    }
}

}  // namespace sr
