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
// Opaque draws take the order-independent path of sr_opaque.cu.
//
// raster_ordered_kernel (blending, stencil-gated draws): one thread per pixel
// walks the bin's primitives in submission order (sorted lists, sr_bins.cu),
// once per semantic tile containing the pixel, applying the reference's
// sequence literally.
#include "sr_internal.cuh"
#include "sr_scan.cuh"
#include "sr_shade.cuh"
#include "sr_tma.cuh"

namespace sr {

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

// ---------------------------------------------------------------- ordered
constexpr int ORD_THREADS = 256;      // 16 x 16 bin, one pixel per thread
constexpr int ORD_CHUNK = 128;        // setup records staged per step

template <int FMT>
struct PixelColor;
template <> struct PixelColor<SR_COLOR_RGBA32F> { float4 v; };
template <> struct PixelColor<SR_COLOR_RGBA8> { uint32_t v; };
template <> struct PixelColor<SR_COLOR_NONE> { uint32_t v; };

// Resident blocks per SM asked of the compiler: the light shaders (vertex
// colour, constant) fit 48 registers, so five 256-thread blocks run per SM
// instead of four; the lit shaders keep the default.
template <int FS>
struct OrdOccupancy { static constexpr int BLOCKS = 1; };
template <> struct OrdOccupancy<FS_VERTEX_COLOR> { static constexpr int BLOCKS = 5; };
template <> struct OrdOccupancy<FS_CONSTANT_COLOR> { static constexpr int BLOCKS = 5; };

template <int FS, int FMT, int BLEND>
__global__ void __launch_bounds__(ORD_THREADS, OrdOccupancy<FS>::BLOCKS) raster_ordered_kernel(
    DrawParams P, sr_uniforms U, const float4* __restrict__ setup, const uint32_t* __restrict__ bin_off,
    const uint32_t* __restrict__ entries, const uint32_t* __restrict__ vidx, const float* __restrict__ vary,
    const uint32_t* __restrict__ tex, void* __restrict__ color, float* __restrict__ depth, uint8_t* __restrict__ stencil,
    uint32_t gate_with_stencil, DeviceFlags* flags, uint32_t tma, const __grid_constant__ CUtensorMap tm_color,
    const __grid_constant__ CUtensorMap tm_depth, const __grid_constant__ CUtensorMap tm_stencil) {
    // the bin's framebuffer tile (with `tma`): colour, depth and stencil are
    // loaded by tensor copies, read and written by the bin's pixels in
    // registers, and stored back the same way
    constexpr uint32_t CW = FMT == SR_COLOR_RGBA32F ? 4u : 1u;   // colour words per pixel
    __shared__ alignas(128) uint32_t t_color[ORD_THREADS * CW];
    __shared__ alignas(128) float t_depth[ORD_THREADS];
    __shared__ alignas(128) uint8_t t_stencil[ORD_THREADS];
    __shared__ alignas(8) uint64_t t_bar;
    __shared__ float4 rec[ORD_CHUNK][3];
    __shared__ int4 rbb[ORD_CHUNK];
    __shared__ uint32_t rtri[ORD_CHUNK];
    // per chunk: for each pixel of the bin the chunk entries whose bbox holds
    // it (entries with small bin rectangles), and the entries every pixel
    // tests (larger rectangles, unsafe primitives, exhaustive mode)
    __shared__ uint32_t pmask[ORD_THREADS][ORD_CHUNK / 32];
    // (double-buffered by chunk parity: a warp that finished its pixels of one
    // chunk clears the other buffer while slower warps still read this one)
    __shared__ uint32_t lmask_buf[2][ORD_CHUNK / 32];
    // the chunk entries' vertex varyings, staged once per chunk
    constexpr int NKQ = FsTraits<FS>::NK > 0 ? (FsTraits<FS>::NK + 3) / 4 : 1;
    __shared__ float4 svary[FsTraits<FS>::NK > 0 ? ORD_CHUNK : 1][3][NKQ];
    if (flags->poison) return;
    const uint32_t bin = blockIdx.x;
    const uint32_t N = P.n_raster_host ? P.n_raster_host : (uint32_t)flags->n_gen_tris;
    uint32_t beg = 0, cnt = N;
    if (!P.mode_b) {   // the bin's primitives, sorted in submission order (sr_bins.cu)
        beg = bin_off[2 * (size_t)bin];
        cnt = bin_off[2 * (size_t)bin + 1] - beg;
        if (cnt == 0) return;
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
    // tile coordinates in the tensor maps' elements (colour RGBA32F: 4 words a pixel)
    const int tx = (int)(bx * BW), ty = (int)(by * BH), tcx = (int)(bx * BW * CW);
    if (tma) {
        if (threadIdx.x == 0) {
            mbar_init(&t_bar, 1);
            uint32_t bytes = 0;
            if (FMT != SR_COLOR_NONE) bytes += ORD_THREADS * CW * 4;
            if (P.has_depth) bytes += ORD_THREADS * 4;
            if (P.has_stencil) bytes += ORD_THREADS;
            mbar_arrive_expect_tx(&t_bar, bytes);
            if (FMT != SR_COLOR_NONE) tma_load_2d(t_color, &tm_color, tcx, ty, &t_bar);
            if (P.has_depth) tma_load_2d(t_depth, &tm_depth, tx, ty, &t_bar);
            if (P.has_stencil) tma_load_2d(t_stencil, &tm_stencil, tx, ty, &t_bar);
        }
        __syncthreads();   // the barrier is initialised before it is polled
        bool done = false;
        for (uint32_t polls = 0; !done && polls < TMA_WAIT_POLLS; ++polls) done = mbar_try_wait(&t_bar, 0);
        if (!__syncthreads_and(done)) {
            // the copies did not arrive in time: report, wait (bounded again)
            // until they are no longer writing this CTA's shared memory, skip
            // the tile
            if (threadIdx.x == 0) atomicOr(&flags->copy_timeout, 1u);
            for (uint32_t polls = 0; !done && polls < TMA_WAIT_POLLS; ++polls) done = mbar_try_wait(&t_bar, 0);
            return;
        }
        if (FMT == SR_COLOR_RGBA32F) *(float4*)&pc.v = reinterpret_cast<const float4*>(t_color)[threadIdx.x];
        else if (FMT == SR_COLOR_RGBA8) *(uint32_t*)&pc.v = t_color[threadIdx.x];
        if (P.has_depth) d = t_depth[threadIdx.x];
        if (P.has_stencil) s = t_stencil[threadIdx.x];
    } else if (active) {
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
    uint32_t parity = 0;
    for (int pass = 0; pass < max_kp; ++pass) {
        const bool my_pass = pass < kp;
        const int ri = my_pass ? pass / cs.count : 0, ci = my_pass ? pass % cs.count : 0;
        for (uint32_t cb = 0; cb < cnt; cb += ORD_CHUNK, parity ^= 1u) {
            uint32_t m = min((uint32_t)ORD_CHUNK, cnt - cb);
            uint32_t* lmask = lmask_buf[parity];
#pragma unroll
            for (int w = 0; w < ORD_CHUNK / 32; ++w) pmask[threadIdx.x][w] = 0;   // this pixel's previous chunk is done
            if (threadIdx.x < ORD_CHUNK / 32) lmask[threadIdx.x] = 0;
            __syncthreads();
            if (threadIdx.x < m) {
                uint32_t j = cb + threadIdx.x;
                uint32_t t = P.mode_b ? j : __ldg(entries + beg + j);
                // the extension pass may list a primitive twice in a bin
                bool dup = !P.mode_b && j > 0 && __ldg(entries + beg + j - 1) == t;
                const float4* r = setup + 4 * (size_t)t;
                rec[threadIdx.x][0] = __ldg(r);
                rec[threadIdx.x][1] = __ldg(r + 1);
                float4 r2 = __ldg(r + 2), r3 = __ldg(r + 3);
                if (dup) r2.z = __uint_as_float(0u);
                rec[threadIdx.x][2] = r2;
                rbb[threadIdx.x] = make_int4(__float_as_int(r3.x), __float_as_int(r3.y), __float_as_int(r3.z),
                                             __float_as_int(r3.w));
                rtri[threadIdx.x] = t;
                const uint32_t fl = __float_as_uint(r2.z);
                if (FsTraits<FS>::NK > 0 && (fl & REC_RASTER)) {
#pragma unroll
                    for (int vq = 0; vq < 3; ++vq) {
                        const uint32_t slot = __ldg(vidx + 3 * (size_t)t + vq);
                        const float4* kq = reinterpret_cast<const float4*>(vary + (size_t)slot * VSTRIDE);
#pragma unroll
                        for (int q = 0; q < NKQ; ++q) svary[threadIdx.x][vq][q] = __ldg(kq + q);
                    }
                }
                if (fl & REC_RASTER) {
                    const uint32_t bit = 1u << (threadIdx.x & 31), wi = threadIdx.x >> 5;
                    const int bx0 = (int)(bx * BW), by0 = (int)(by * BH);
                    const int x0 = max(__float_as_int(r3.x), bx0), x1 = min(__float_as_int(r3.z), bx0 + (int)BW - 1);
                    const int y0 = max(__float_as_int(r3.y), by0), y1 = min(__float_as_int(r3.w), by0 + (int)BH - 1);
                    if (P.mode_b || (fl & REC_UNSAFE)) {
                        atomicOr(&lmask[wi], bit);
                    } else if ((x1 - x0 + 1) * (y1 - y0 + 1) > 16) {
                        // a safe primitive touches only covered pixels of its
                        // bbox here (stencil events are counted apart unless in
                        // mode B): one whose sign test clears the bin part of
                        // its bbox is dropped for the whole bin
                        if (!rect_cleared(rec[threadIdx.x][0], rec[threadIdx.x][1], x0, y0, x1, y1))
                            atomicOr(&lmask[wi], bit);
                    } else if (x0 <= x1 && y0 <= y1) {
                        for (int yy = y0; yy <= y1; ++yy)
                            for (int xx = x0; xx <= x1; ++xx)
                                atomicOr(&pmask[((yy - by0) << P.bin_w_log2) + (xx - bx0)][wi], bit);
                    }
                }
            }
            __syncthreads();
            if (!my_pass) continue;
            // the chunk's entries for this pixel, in submission order: one mask
            // word at a time in a register (the unrolled word loop keeps the
            // masks out of local memory)
#pragma unroll
            for (int w = 0; w < ORD_CHUNK / 32; ++w) {
                uint32_t mw = pmask[threadIdx.x][w] | lmask[w];
                while (mw) {
                    const uint32_t e = (uint32_t)w * 32 + (uint32_t)(__ffs(mw) - 1);
                    mw &= mw - 1;
                    float4 r2 = rec[e][2];
                    uint32_t fl = __float_as_uint(r2.z);   // (only raster entries have mask bits)
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
                    constexpr int NK = FsTraits<FS>::NK;
                    float kv[NK > 0 ? ((NK + 3) / 4) * 4 : 4];
                    if (NK > 0) {
                        // (ka*u + kb*v) + kc*w, interpolate.rs:43-52
    #pragma unroll
                        for (int q = 0; q < NKQ; ++q) {
                            const float4 xa = svary[e][0][q], xb = svary[e][1][q], xc = svary[e][2][q];
                            kv[4 * q + 0] = (xa.x * b.u + xb.x * b.v) + xc.x * b.w;
                            kv[4 * q + 1] = (xa.y * b.u + xb.y * b.v) + xc.y * b.w;
                            kv[4 * q + 2] = (xa.z * b.u + xb.z * b.v) + xc.z * b.w;
                            kv[4 * q + 3] = (xa.w * b.u + xb.w * b.v) + xc.w * b.w;
                        }
                    }
                    sr_v4 col = shade_fs<FS>(U, kv, tex, P);
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
    }
    if (tma) {
        // the tile back through the copy engine; its pixels outside the frame
        // are not written
        if (active) {
            if (FMT == SR_COLOR_RGBA32F) reinterpret_cast<float4*>(t_color)[threadIdx.x] = *(float4*)&pc.v;
            else if (FMT == SR_COLOR_RGBA8) t_color[threadIdx.x] = *(uint32_t*)&pc.v;
            if (P.has_depth) t_depth[threadIdx.x] = d;
            if (P.has_stencil && P.mode_b) t_stencil[threadIdx.x] = (uint8_t)s;
        }
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            if (FMT != SR_COLOR_NONE) tma_store_2d(&tm_color, tcx, ty, t_color);
            if (P.has_depth) tma_store_2d(&tm_depth, tx, ty, t_depth);
            if (P.has_stencil && P.mode_b) tma_store_2d(&tm_stencil, tx, ty, t_stencil);
            bulk_commit();
            bulk_wait();
        }
    } else if (active) {
        if (FMT == SR_COLOR_RGBA32F) reinterpret_cast<float4*>(color)[gi] = *(float4*)&pc.v;
        else if (FMT == SR_COLOR_RGBA8) reinterpret_cast<uint32_t*>(color)[gi] = *(uint32_t*)&pc.v;
        if (P.has_depth) depth[gi] = d;
        if (P.has_stencil && P.mode_b) stencil[gi] = (uint8_t)s;
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&flags->fragments, frags);
}

// ---------------------------------------------------------------- launch
// Tensor maps of a draw's framebuffer planes for the ordered kernel's tile
// copies (16 x 16 pixel boxes), when the planes allow them: row strides a
// multiple of 16 bytes (RGBA8 colour and depth: a width that is a multiple
// of 4; stencil: of 16) and 16-byte aligned planes.  Encoded on the host with
// the driver's cuTensorMapEncodeTiled, looked up once through the runtime.
struct FbMaps {
    uint32_t tma = 0;
    CUtensorMap color{}, depth{}, stencil{};
};

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<EncodeTiledFn>(f);
    }();
    return fn;
}

static bool encode_plane(CUtensorMap* m, CUtensorMapDataType type, uint32_t elem_bytes, void* base, uint64_t cols,
                         uint64_t rows, uint32_t box_cols, uint32_t box_rows) {
    const EncodeTiledFn fn = encode_tiled();
    if (!fn || !base || (reinterpret_cast<uintptr_t>(base) & 15) || (cols * elem_bytes) % 16) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * elem_bytes};
    const cuuint32_t box[2] = {box_cols, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, type, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static FbMaps fb_maps(const DrawParams& P, void* color, float* depth, uint8_t* stencil) {
    FbMaps M;
    const uint32_t BW = 1u << P.bin_w_log2, BH = 1u << P.bin_h_log2;
    if (BW * BH != (uint32_t)ORD_THREADS) return M;
    bool ok = true;
    if (P.color_format == SR_COLOR_RGBA8)
        ok = ok && encode_plane(&M.color, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, color, P.W, P.H, BW, BH);
    else if (P.color_format == SR_COLOR_RGBA32F)   // four words a pixel
        ok = ok && encode_plane(&M.color, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, color, 4ull * P.W, P.H, 4 * BW, BH);
    if (P.has_depth) ok = ok && encode_plane(&M.depth, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, depth, P.W, P.H, BW, BH);
    if (P.has_stencil)
        ok = ok && encode_plane(&M.stencil, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, stencil, P.W, P.H, BW, BH);
    M.tma = ok ? 1u : 0u;
    return M;
}

template <int FS, int FMT, int BLEND>
static void launch_ordered_t(const DrawParams& P, const sr_uniforms& U, const float4* setup, const uint32_t* bin_off,
                             const uint32_t* entries, const uint32_t* vidx, const float* vary, const uint32_t* tex,
                             void* color, float* depth, uint8_t* stencil, uint32_t gate, DeviceFlags* flags,
                             const FbMaps& M, cudaStream_t st) {
    uint32_t nb = P.bins_x * P.bins_y;
    raster_ordered_kernel<FS, FMT, BLEND><<<nb, ORD_THREADS, 0, st>>>(P, U, setup, bin_off, entries, vidx, vary, tex,
                                                                      color, depth, stencil, gate, flags, M.tma,
                                                                      M.color, M.depth, M.stencil);
}

template <int FS>
static void dispatch_fmt(const DrawParams& P, const sr_uniforms& U, const float4* setup, const uint32_t* bin_off,
                         const uint32_t* entries, const uint32_t* vidx, const float* vary, const uint32_t* tex,
                         void* color, float* depth, uint8_t* stencil, uint32_t gate, DeviceFlags* flags,
                         const FbMaps& M, cudaStream_t st) {
#define SR_ORD(FMT, BL) launch_ordered_t<FS, FMT, BL>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, \
                                                       stencil, gate, flags, M, st)
    if (P.color_format == SR_COLOR_RGBA32F) {
        if (P.blend == BLEND_OVER) SR_ORD(SR_COLOR_RGBA32F, BLEND_OVER);
        else SR_ORD(SR_COLOR_RGBA32F, BLEND_REPLACE);
    } else if (P.color_format == SR_COLOR_RGBA8) {
        if (P.blend == BLEND_OVER) SR_ORD(SR_COLOR_RGBA8, BLEND_OVER);
        else SR_ORD(SR_COLOR_RGBA8, BLEND_REPLACE);
    } else {
        SR_ORD(SR_COLOR_NONE, BLEND_REPLACE);
    }
#undef SR_ORD
}

void launch_ordered(const DrawParams& P, const sr_uniforms& U, const float4* setup, const uint32_t* bin_off,
                    const uint32_t* entries, const uint32_t* vidx, const float* vary, const uint32_t* tex, void* color,
                    float* depth, uint8_t* stencil, uint32_t gate, DeviceFlags* flags, cudaStream_t st) {
    const FbMaps M = fb_maps(P, color, depth, stencil);
#define SR_DISPATCH(F) dispatch_fmt<F>(P, U, setup, bin_off, entries, vidx, vary, tex, color, depth, stencil, gate, \
                                       flags, M, st)
    switch (P.fs) {
    case FS_BLINN_PHONG_DIR: SR_DISPATCH(FS_BLINN_PHONG_DIR); break;
    case FS_TEXTURED_BLINN_PHONG: SR_DISPATCH(FS_TEXTURED_BLINN_PHONG); break;
    case FS_VERTEX_COLOR: SR_DISPATCH(FS_VERTEX_COLOR); break;
    case FS_ACES_LIGHTS: SR_DISPATCH(FS_ACES_LIGHTS); break;
    default: SR_DISPATCH(FS_CONSTANT_COLOR); break;
    }
#undef SR_DISPATCH
}

}  // namespace sr
