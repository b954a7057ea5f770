// sr_raster.cu — the per-pixel part of rasterize_triangle
// (stages/rasterization/triangle.rs:80-155) over the binned primitives.
//
// Per pixel centre (x, y) = (px + 0.5, py + 0.5) the reference computes, in
// FP32 without contraction:
//   u = ((y2-y3)*(x-x3) + (x3-x2)*(y-y3)) / det
//   v = ((y3-y1)*(x-x3) + (x1-x3)*(y-y3)) / det
//   w = (1 - u) - v;   covered iff !(u < 0 || v < 0 || w < 0)
//   z = (z1*u + z2*v) + z3*w;  fragment iff z < 0 and z >= depth[p]
// and the semantic tiles (fragment.rs:188-216) overlap by one pixel, so a seam
// pixel is processed once per tile containing it, in row-major tile order.
//
// raster_opaque_kernel (blend `()`, shaders that never discard): the final
// colour of a pixel is the shade of the LAST fragment in submission order
// whose z equals the maximum z (ties pass `>=`).  That winner is the
// lexicographic maximum of (zkey(z), pass, primitive), so fragments are tested
// fragment-parallel, reduced with 64-bit shared-memory atomicMax, and only the
// winner is shaded (deferred): the result equals the reference's sequential
// loop bit for bit.
//
// raster_ordered_kernel (blending, stencil-gated draws): one thread per pixel
// walks the bin's primitives in submission order (sorted in shared memory),
// once per semantic tile containing the pixel, applying the reference's
// sequence literally.
#include "sr_internal.cuh"
#include "sr_scan.cuh"

namespace sr {

template <int FS>
struct FsTraits { static constexpr int NK = 8; };
template <> struct FsTraits<FS_TEXTURED_BLINN_PHONG> { static constexpr int NK = 10; };
template <> struct FsTraits<FS_VERTEX_COLOR> { static constexpr int NK = 4; };
template <> struct FsTraits<FS_CONSTANT_COLOR> { static constexpr int NK = 0; };

// The fragment closures compiled into the library (RGBA f32 result).
template <int FS>
__device__ __forceinline__ sr_v4 shade(const sr_uniforms& U, const float* k, const uint32_t* tex, const DrawParams& P) {
    if (FS == FS_BLINN_PHONG_DIR)
        return sr_blinn_phong(&U, sr_make_v4(k[0], k[1], k[2], k[3]), sr_make_v4(k[4], k[5], k[6], k[7]),
                              sr_make_v4(U.color[0], U.color[1], U.color[2], U.color[3]));
    if (FS == FS_TEXTURED_BLINN_PHONG) {
        sr_v4 t = sr_sample_rgba8(tex, P.tex_w, P.tex_h, k[8], k[9], (int)P.tex_filter, (int)P.tex_edge);
        t = sr_decode_gamma(t, U.gamma);
        return sr_blinn_phong(&U, sr_make_v4(k[0], k[1], k[2], k[3]), sr_make_v4(k[4], k[5], k[6], k[7]), t);
    }
    if (FS == FS_VERTEX_COLOR) return sr_make_v4(k[0], k[1], k[2], k[3]);
    if (FS == FS_ACES_LIGHTS)
        return sr_aces_lights(&U, sr_make_v4(k[0], k[1], k[2], k[3]), sr_make_v4(k[4], k[5], k[6], k[7]));
    return sr_make_v4(U.color[0], U.color[1], U.color[2], U.color[3]);
}

// Barycentric varyings (interpolate.rs:43-52): (ka*u + kb*v) + kc*w
template <int NK>
__device__ __forceinline__ void interp_varyings(const float* __restrict__ vary, uint32_t a, uint32_t b, uint32_t c,
                                                float u, float v, float w, float* k) {
    const float4* ka = reinterpret_cast<const float4*>(vary + (size_t)a * VSTRIDE);
    const float4* kb = reinterpret_cast<const float4*>(vary + (size_t)b * VSTRIDE);
    const float4* kc = reinterpret_cast<const float4*>(vary + (size_t)c * VSTRIDE);
#pragma unroll
    for (int q = 0; q < (NK + 3) / 4; ++q) {
        float4 x = __ldg(ka + q), y = __ldg(kb + q), z = __ldg(kc + q);
        k[4 * q + 0] = (x.x * u + y.x * v) + z.x * w;
        k[4 * q + 1] = (x.y * u + y.y * v) + z.y * w;
        k[4 * q + 2] = (x.z * u + y.z * v) + z.z * w;
        k[4 * q + 3] = (x.w * u + y.w * v) + z.w * w;
    }
}

struct Bary {
    float u, v, w, z;
    bool covered;
};

__device__ __forceinline__ Bary barycentric(float4 r0, float4 r1, float4 r2, uint32_t px, uint32_t py) {
    Bary b;
    float x = (float)px + 0.5f;
    float y = (float)py + 0.5f;
    float dx = x - r1.x, dy = y - r1.y;
    b.u = (r0.x * dx + r0.y * dy) / r1.z;
    b.v = (r0.z * dx + r0.w * dy) / r1.z;
    b.w = 1.0f - b.u - b.v;
    b.covered = !(b.u < 0.0f || b.v < 0.0f || b.w < 0.0f);
    b.z = (r1.w * b.u + r2.x * b.v) + r2.y * b.w;
    return b;
}

// Highest-rank semantic tile containing (px, py) whose clamped bbox of the
// primitive contains the pixel; -1 if none.  Ranks are row-major among the
// (1, 2 or 4) tiles containing the pixel.
__device__ __forceinline__ int clamped_rank(const DrawParams& P, int ix0, int iy0, int ix1, int iy1, uint32_t px,
                                            uint32_t py, TileSpan cs, TileSpan rs) {
    int best = -1;
    for (int ri = 0; ri < rs.count; ++ri) {
        if (!clamp_axis(iy0, iy1, py, (uint32_t)(rs.first + ri), P.tile_h, P.H - 1)) continue;
        for (int ci = 0; ci < cs.count; ++ci)
            if (clamp_axis(ix0, ix1, px, (uint32_t)(cs.first + ci), P.tile_w, P.W - 1)) best = ri * cs.count + ci;
    }
    return best;
}

template <int FMT>
__device__ __forceinline__ void store_color(void* color, size_t idx, sr_v4 c) {
    if (FMT == SR_COLOR_RGBA32F) reinterpret_cast<float4*>(color)[idx] = make_float4(c.x, c.y, c.z, c.w);
    else if (FMT == SR_COLOR_RGBA8) reinterpret_cast<uint32_t*>(color)[idx] = sr_to_rgba8(c);
}

constexpr int OPQ_THREADS = 256;
constexpr int OPQ_CHUNK = 256;
constexpr unsigned long long KEY_BLOCK = ~0ull;

template <int FS, int FMT>
__global__ void __launch_bounds__(OPQ_THREADS) raster_opaque_kernel(
    DrawParams P, sr_uniforms U, const float4* __restrict__ setup, const uint32_t* __restrict__ bin_off,
    const uint32_t* __restrict__ entries, const uint32_t* __restrict__ vidx, const float* __restrict__ vary,
    const uint32_t* __restrict__ tex, void* __restrict__ color, float* __restrict__ depth,
    const uint8_t* __restrict__ stencil, uint32_t gate_with_stencil, DeviceFlags* flags) {
    extern __shared__ unsigned long long keys[];   // bin pixels
    __shared__ float4 rec[OPQ_CHUNK][3];
    __shared__ int4 rbb[OPQ_CHUNK];
    __shared__ uint32_t rtri[OPQ_CHUNK];
    __shared__ uint32_t rrect[OPQ_CHUNK];          // x0 | y0 << 8 | w << 16 | h << 24 (bin-local)
    __shared__ uint32_t pre[OPQ_CHUNK + 1];
    __shared__ uint8_t gate[1024];                 // stencil gate per bin pixel
    if (flags->poison) return;
    const uint32_t bin = blockIdx.x;
    const uint32_t beg = bin_off[bin], end = bin_off[bin + 1];
    if (beg == end) return;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    const uint32_t bx = bin % P.bins_x, by = bin / P.bins_x;
    const uint32_t BW = 1u << P.bin_w_log2, BH = 1u << P.bin_h_log2;
    const uint32_t X0 = bx * BW, Y0 = by * BH;
    const uint32_t bw = min(BW, P.W - X0), bh = min(BH, P.H - Y0);
    const uint32_t npx = bw * bh;
    for (uint32_t i = threadIdx.x; i < npx; i += OPQ_THREADS) {
        uint32_t gx = X0 + i % bw, gy = Y0 + i / bw;
        size_t gi = (size_t)gy * P.W + gx;
        unsigned long long k = 0;
        if (P.has_depth) {
            float d0 = depth[gi];
            k = isnan(d0) ? KEY_BLOCK : ((unsigned long long)zkey(d0) << 32);
        }
        bool g = !gate_with_stencil || stencil_test(P.stencil_test, stencil[gi], P.sref);
        if (!g) k = KEY_BLOCK;
        keys[i] = k;
        gate[i] = g ? 1 : 0;
    }
    unsigned long long frags = 0;
    for (uint32_t cb = beg; cb < end; cb += OPQ_CHUNK) {
        uint32_t m = min((uint32_t)OPQ_CHUNK, end - cb);
        uint32_t cnt = 0;
        if (threadIdx.x < m) {
            uint32_t t = entries[cb + threadIdx.x];
            const float4* r = setup + 4 * (size_t)t;
            float4 r2 = __ldg(r + 2), r3 = __ldg(r + 3);
            rec[threadIdx.x][0] = __ldg(r);
            rec[threadIdx.x][1] = __ldg(r + 1);
            rec[threadIdx.x][2] = r2;
            int4 bb = make_int4(__float_as_int(r3.x), __float_as_int(r3.y), __float_as_int(r3.z), __float_as_int(r3.w));
            rbb[threadIdx.x] = bb;
            rtri[threadIdx.x] = t;
            bool unsafe = __float_as_uint(r2.z) & REC_UNSAFE;
            int x0 = 0, y0 = 0, x1 = (int)bw - 1, y1 = (int)bh - 1;
            if (!unsafe) {
                x0 = max(bb.x - (int)X0, 0); y0 = max(bb.y - (int)Y0, 0);
                x1 = min(bb.z - (int)X0, (int)bw - 1); y1 = min(bb.w - (int)Y0, (int)bh - 1);
            }
            if (x0 <= x1 && y0 <= y1) {
                uint32_t w = (uint32_t)(x1 - x0 + 1), h = (uint32_t)(y1 - y0 + 1);
                rrect[threadIdx.x] = (uint32_t)x0 | ((uint32_t)y0 << 8) | ((w - 1) << 16) | ((h - 1) << 24);
                cnt = w * h;
            }
        }
        uint32_t total;
        uint32_t ex = block_exclusive_scan<uint32_t, OPQ_THREADS>(cnt, &total);
        if (threadIdx.x < OPQ_CHUNK) pre[threadIdx.x] = ex;
        if (threadIdx.x == 0) pre[OPQ_CHUNK] = total;
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < total; j += OPQ_THREADS) {
            // owning entry: largest i with pre[i] <= j
            int lo = 0, hi = (int)m - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (pre[mid] <= j) lo = mid; else hi = mid - 1;
            }
            uint32_t rr = rrect[lo];
            uint32_t w = ((rr >> 16) & 0xffu) + 1;
            uint32_t local = j - pre[lo];
            uint32_t lx = (rr & 0xffu) + local % w, ly = ((rr >> 8) & 0xffu) + local / w;
            uint32_t px = X0 + lx, py = Y0 + ly;
            int4 bb = rbb[lo];
            float4 r0 = rec[lo][0], r1 = rec[lo][1], r2 = rec[lo][2];
            bool in_b = bb.x <= (int)px && (int)px <= bb.z && bb.y <= (int)py && (int)py <= bb.w;
            TileSpan cs = tiles_of(px, P.tile_w, P.ncols, P.W - 1);
            TileSpan rs = tiles_of(py, P.tile_h, P.nrows, P.H - 1);
            int kp = cs.count * rs.count;
            int prank = in_b ? kp - 1 : clamped_rank(P, bb.x, bb.y, bb.z, bb.w, px, py, cs, rs);
            if (prank < 0) continue;
            Bary b = barycentric(r0, r1, r2, px, py);
            if (!b.covered || !(b.z < 0.0f)) continue;
            if (!gate[ly * bw + lx]) continue;
            if (prank == kp - 1) ++frags;
            uint32_t zk = P.has_depth ? zkey(b.z) : 0u;
            unsigned long long key = ((unsigned long long)zk << 32) |
                                     (unsigned long long)((uint32_t)prank * N + rtri[lo] + 1u);
            atomicMax(&keys[ly * bw + lx], key);
        }
        __syncthreads();
    }
    // resolve: shade the winner of each pixel once
    for (uint32_t i = threadIdx.x; i < npx; i += OPQ_THREADS) {
        unsigned long long k = keys[i];
        uint32_t seq = (uint32_t)(k & 0xffffffffull);
        if (k == KEY_BLOCK || seq == 0) continue;
        uint32_t t = (seq - 1u) % N;
        uint32_t px = X0 + i % bw, py = Y0 + i / bw;
        size_t gi = (size_t)py * P.W + px;
        const float4* r = setup + 4 * (size_t)t;
        Bary b = barycentric(__ldg(r), __ldg(r + 1), __ldg(r + 2), px, py);
        constexpr int NK = FsTraits<FS>::NK;
        float kv[NK > 0 ? ((NK + 3) / 4) * 4 : 4];
        if (NK > 0) {
            uint32_t a = __ldg(vidx + 3 * (size_t)t), bb = __ldg(vidx + 3 * (size_t)t + 1), c = __ldg(vidx + 3 * (size_t)t + 2);
            interp_varyings<NK>(vary, a, bb, c, b.u, b.v, b.w, kv);
        }
        sr_v4 col = shade<FS>(U, kv, tex, P);
        store_color<FMT>(color, gi, col);
        if (P.has_depth) depth[gi] = b.z;
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// ---------------------------------------------------------------- ordered
constexpr int ORD_THREADS = 256;      // 16 x 16 bin, one pixel per thread
constexpr int ORD_CHUNK = 128;        // setup records staged per step
constexpr int SORT_CAP = 16384;       // bin entries sortable in shared memory

template <int FMT>
struct PixelColor;
template <> struct PixelColor<SR_COLOR_RGBA32F> { float4 v; };
template <> struct PixelColor<SR_COLOR_RGBA8> { uint32_t v; };
template <> struct PixelColor<SR_COLOR_NONE> { uint32_t v; };

// Bitonic sort of n (power of two) keys in shared memory.
__device__ void block_bitonic_sort(uint32_t* a, uint32_t n) {
    for (uint32_t k = 2; k <= n; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                uint32_t l = i ^ j;
                if (l > i) {
                    uint32_t x = a[i], y = a[l];
                    bool up = (i & k) == 0;
                    if ((x > y) == up) { a[i] = y; a[l] = x; }
                }
            }
            __syncthreads();
        }
    }
}

template <int FS, int FMT, int BLEND>
__global__ void __launch_bounds__(ORD_THREADS) raster_ordered_kernel(
    DrawParams P, sr_uniforms U, const float4* __restrict__ setup, const uint32_t* __restrict__ bin_off,
    const uint32_t* __restrict__ entries, const uint32_t* __restrict__ vidx, const float* __restrict__ vary,
    const uint32_t* __restrict__ tex, void* __restrict__ color, float* __restrict__ depth, uint8_t* __restrict__ stencil,
    uint32_t gate_with_stencil, DeviceFlags* flags) {
    extern __shared__ uint32_t list[];              // sorted bin entries (not used in mode B)
    __shared__ float4 rec[ORD_CHUNK][3];
    __shared__ int4 rbb[ORD_CHUNK];
    __shared__ uint32_t rtri[ORD_CHUNK];
    if (flags->poison) return;
    const uint32_t bin = blockIdx.x;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    uint32_t beg = 0, cnt = N;
    if (!P.mode_b) {
        beg = bin_off[bin];
        cnt = bin_off[bin + 1] - beg;
        if (cnt == 0) return;
        if (cnt > (uint32_t)SORT_CAP) {
            if (threadIdx.x == 0) { atomicOr(&flags->overflow_bits, (unsigned)OVF_SORT); atomicOr(&flags->poison, 1u); atomicMin(&flags->poison_draw, P.draw_id); }
            return;
        }
        uint32_t n2 = 1;
        while (n2 < cnt) n2 <<= 1;
        for (uint32_t i = threadIdx.x; i < n2; i += ORD_THREADS) list[i] = i < cnt ? entries[beg + i] : 0xffffffffu;
        __syncthreads();
        block_bitonic_sort(list, n2);
    }
    const uint32_t bx = bin % P.bins_x, by = bin / P.bins_x;
    const uint32_t BW = 1u << P.bin_w_log2, BH = 1u << P.bin_h_log2;
    const uint32_t lx = threadIdx.x & (BW - 1), ly = threadIdx.x >> P.bin_w_log2;
    const uint32_t px = bx * BW + lx, py = by * BH + ly;
    const bool active = ly < BH && px < P.W && py < P.H;
    size_t gi = (size_t)py * P.W + px;
    PixelColor<FMT> pc;
    float d = 0.0f;
    uint32_t s = 0;
    if (active) {
        if (FMT == SR_COLOR_RGBA32F) *(float4*)&pc.v = reinterpret_cast<float4*>(color)[gi];
        else if (FMT == SR_COLOR_RGBA8) *(uint32_t*)&pc.v = reinterpret_cast<uint32_t*>(color)[gi];
        if (P.has_depth) d = depth[gi];
        if (P.has_stencil) s = stencil[gi];
    }
    bool gate = true;
    if (active && gate_with_stencil) gate = stencil_test(P.stencil_test, s, P.sref);
    TileSpan cs = tiles_of(px, P.tile_w, P.ncols, P.W - 1);
    TileSpan rs = tiles_of(py, P.tile_h, P.nrows, P.H - 1);
    const int kp = active ? cs.count * rs.count : 0;
    // the block streams its list once per pass; kp differs per pixel
    int max_kp = __syncthreads_or(kp > 1) ? (__syncthreads_or(kp > 2) ? 4 : 2) : 1;
    unsigned long long frags = 0;
    for (int pass = 0; pass < max_kp; ++pass) {
        const bool my_pass = pass < kp;
        const int ri = my_pass ? pass / cs.count : 0, ci = my_pass ? pass % cs.count : 0;
        for (uint32_t cb = 0; cb < cnt; cb += ORD_CHUNK) {
            uint32_t m = min((uint32_t)ORD_CHUNK, cnt - cb);
            __syncthreads();
            if (threadIdx.x < m) {
                uint32_t t = P.mode_b ? cb + threadIdx.x : list[cb + threadIdx.x];
                const float4* r = setup + 4 * (size_t)t;
                rec[threadIdx.x][0] = __ldg(r);
                rec[threadIdx.x][1] = __ldg(r + 1);
                float4 r2 = __ldg(r + 2), r3 = __ldg(r + 3);
                rec[threadIdx.x][2] = r2;
                rbb[threadIdx.x] = make_int4(__float_as_int(r3.x), __float_as_int(r3.y), __float_as_int(r3.z),
                                             __float_as_int(r3.w));
                rtri[threadIdx.x] = t;
            }
            __syncthreads();
            if (!my_pass) continue;
            for (uint32_t e = 0; e < m; ++e) {
                float4 r2 = rec[e][2];
                uint32_t fl = __float_as_uint(r2.z);
                if (!(fl & REC_RASTER)) continue;
                int4 bb = rbb[e];
                bool in_b = bb.x <= (int)px && (int)px <= bb.z && bb.y <= (int)py && (int)py <= bb.w;
                bool ev;
                if (P.mode_b || (!in_b && (fl & REC_UNSAFE))) {
                    ev = clamp_axis(bb.x, bb.z, px, (uint32_t)(cs.first + ci), P.tile_w, P.W - 1) &&
                         clamp_axis(bb.y, bb.w, py, (uint32_t)(rs.first + ri), P.tile_h, P.H - 1);
                } else {
                    ev = in_b;
                }
                if (!ev) continue;
                if (P.mode_b) {
                    if (!stencil_test(P.stencil_test, s, P.sref)) continue;
                    if (P.has_stencil) s = stencil_op(P.stencil_op, P.stencil_wrap, s, P.sref);
                } else if (!gate) {
                    continue;
                }
                Bary b = barycentric(rec[e][0], rec[e][1], r2, px, py);
                if (!b.covered || !(b.z < 0.0f)) continue;
                if (pass == kp - 1) ++frags;
                if (P.has_depth && !(b.z >= d)) continue;
                uint32_t t = rtri[e];
                constexpr int NK = FsTraits<FS>::NK;
                float kv[NK > 0 ? ((NK + 3) / 4) * 4 : 4];
                if (NK > 0) {
                    uint32_t a = __ldg(vidx + 3 * (size_t)t), bq = __ldg(vidx + 3 * (size_t)t + 1),
                             c = __ldg(vidx + 3 * (size_t)t + 2);
                    interp_varyings<NK>(vary, a, bq, c, b.u, b.v, b.w, kv);
                }
                sr_v4 col = shade<FS>(U, kv, tex, P);
                if (FMT == SR_COLOR_RGBA32F) {
                    float4 dst = *(float4*)&pc.v;
                    if (BLEND == BLEND_OVER) col = sr_blend_over_f32(col, sr_make_v4(dst.x, dst.y, dst.z, dst.w));
                    *(float4*)&pc.v = make_float4(col.x, col.y, col.z, col.w);
                } else if (FMT == SR_COLOR_RGBA8) {
                    uint32_t src = sr_to_rgba8(col);
                    *(uint32_t*)&pc.v = BLEND == BLEND_OVER ? sr_blend_over_rgba8(src, *(uint32_t*)&pc.v) : src;
                }
                if (P.has_depth) d = b.z;
            }
        }
    }
    if (active) {
        if (FMT == SR_COLOR_RGBA32F) reinterpret_cast<float4*>(color)[gi] = *(float4*)&pc.v;
        else if (FMT == SR_COLOR_RGBA8) reinterpret_cast<uint32_t*>(color)[gi] = *(uint32_t*)&pc.v;
        if (P.has_depth) depth[gi] = d;
        if (P.has_stencil && P.mode_b) stencil[gi] = (uint8_t)s;
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// ---------------------------------------------------------------- launch
template <int FS, int FMT>
static void launch_opaque_t(const DrawParams& P, const sr_uniforms& U, const float4* setup, const uint32_t* bin_off,
                            const uint32_t* entries, const uint32_t* vidx, const float* vary, const uint32_t* tex,
                            void* color, float* depth, const uint8_t* stencil, uint32_t gate, DeviceFlags* flags,
                            cudaStream_t st) {
    uint32_t nb = P.bins_x * P.bins_y;
    size_t smem = ((size_t)1 << (P.bin_w_log2 + P.bin_h_log2)) * sizeof(unsigned long long);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(raster_opaque_kernel<FS, FMT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        configured = true;
    }
    raster_opaque_kernel<FS, FMT><<<nb, OPQ_THREADS, smem, st>>>(P, U, setup, bin_off, entries, vidx, vary, tex, color,
                                                                   depth, stencil, gate, flags);
}

template <int FS, int FMT, int BLEND>
static void launch_ordered_t(const DrawParams& P, const sr_uniforms& U, const float4* setup, const uint32_t* bin_off,
                             const uint32_t* entries, const uint32_t* vidx, const float* vary, const uint32_t* tex,
                             void* color, float* depth, uint8_t* stencil, uint32_t gate, DeviceFlags* flags,
                             cudaStream_t st) {
    uint32_t nb = P.bins_x * P.bins_y;
    size_t smem = P.mode_b ? 16 : (size_t)SORT_CAP * 4;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(raster_ordered_kernel<FS, FMT, BLEND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SORT_CAP * 4);
        configured = true;
    }
    raster_ordered_kernel<FS, FMT, BLEND><<<nb, ORD_THREADS, smem, st>>>(P, U, setup, bin_off, entries, vidx, vary,
                                                                          tex, color, depth, stencil, gate, flags);
}

template <int FS>
static void dispatch_fmt(bool ordered, const DrawParams& P, const sr_uniforms& U, const float4* setup,
                         const uint32_t* bin_off, const uint32_t* entries, const uint32_t* vidx, const float* vary,
                         const uint32_t* tex, void* color, float* depth, uint8_t* stencil, uint32_t gate,
                         DeviceFlags* flags, cudaStream_t st) {
    if (!ordered) {
        if (P.color_format == SR_COLOR_RGBA32F)
            launch_opaque_t<FS, SR_COLOR_RGBA32F>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        else if (P.color_format == SR_COLOR_RGBA8)
            launch_opaque_t<FS, SR_COLOR_RGBA8>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        else
            launch_opaque_t<FS, SR_COLOR_NONE>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        return;
    }
    if (P.color_format == SR_COLOR_RGBA32F) {
        if (P.blend == BLEND_OVER)
            launch_ordered_t<FS, SR_COLOR_RGBA32F, BLEND_OVER>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        else
            launch_ordered_t<FS, SR_COLOR_RGBA32F, BLEND_REPLACE>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
    } else if (P.color_format == SR_COLOR_RGBA8) {
        if (P.blend == BLEND_OVER)
            launch_ordered_t<FS, SR_COLOR_RGBA8, BLEND_OVER>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        else
            launch_ordered_t<FS, SR_COLOR_RGBA8, BLEND_REPLACE>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
    } else {
        launch_ordered_t<FS, SR_COLOR_NONE, BLEND_REPLACE>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
    }
}

void launch_raster_any(bool ordered, const DrawParams& P, const sr_uniforms& U, const float4* setup,
                       const uint32_t* bin_off, const uint32_t* entries, const uint32_t* vidx, const float* vary,
                       const uint32_t* tex, void* color, float* depth, uint8_t* stencil, uint32_t gate,
                       DeviceFlags* flags, cudaStream_t st) {
    switch (P.fs) {
    case FS_BLINN_PHONG_DIR:
        dispatch_fmt<FS_BLINN_PHONG_DIR>(ordered, P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        break;
    case FS_TEXTURED_BLINN_PHONG:
        dispatch_fmt<FS_TEXTURED_BLINN_PHONG>(ordered, P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        break;
    case FS_VERTEX_COLOR:
        dispatch_fmt<FS_VERTEX_COLOR>(ordered, P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        break;
    case FS_ACES_LIGHTS:
        dispatch_fmt<FS_ACES_LIGHTS>(ordered, P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        break;
    default:
        dispatch_fmt<FS_CONSTANT_COLOR>(ordered, P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, flags, st);
        break;
    }
}

}  // namespace sr
