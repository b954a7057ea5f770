// sr_static.cu — sr_render_static: an opaque, indexed triangle draw whose
// scratch lives in a fixed array compiled into this library instead of in
// buffers the library allocates.
//
// Who needs it: code that must not allocate device memory at draw time.  A
// host application that owns all of the GPU's memory through its own
// allocator (an engine's arena, a framework's caching pool) cannot let a
// library call cudaMalloc behind its back; a real-time loop cannot take the
// latency or the implicit device synchronisation of cudaMalloc/cudaFree in
// the middle of a frame; and a plugin that is handed only device pointers for
// its inputs and outputs has no lifetime in which to free what it allocated.
// sr_render_static takes every input and output as a caller-owned device
// pointer and never calls cudaMalloc, cudaFree or any allocating routine.
//
// The scratch is one file-scope __device__ array, sized for the limits
// SR_STATIC_MAX_PIXELS, SR_STATIC_MAX_TRIANGLES and SR_STATIC_MAX_VERTICES of
// include/sr.h (about 17.5 MiB).  Every GPU that loads this library's device
// code holds it until the process exits; with CUDA's lazy module loading that
// happens when the code is first needed on a device, which can be during the
// first call there (include/sr.h says to make that call ahead of any
// latency-critical loop).  The kernels are the ones sr_render runs for the
// same draw (vertex, setup, the opaque raster passes and the resolve), so the
// framebuffer comes out bit-identical; only where their scratch lives differs.
//
// Host code cannot pass the array's name to a kernel (on the host it names a
// host-side shadow, not device memory), so the device address is looked up
// once per device with cudaGetSymbolAddress, with that device current, on
// the first call that runs on it.
#include <cstdint>
#include <cstring>
#include <mutex>

#include "sr_internal.cuh"

using namespace sr;

namespace {

constexpr size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// Sub-buffer offsets inside the array (each 256-byte aligned).
constexpr size_t ST_MAXPX = SR_STATIC_MAX_PIXELS;
constexpr size_t ST_MAXT = SR_STATIC_MAX_TRIANGLES;
constexpr size_t ST_MAXV = SR_STATIC_MAX_VERTICES;
// touched-block bitmap: one bit per 32x32 block.  ceil(W/32) * ceil(H/32) <=
// W*H/1024 + W/32 + H/32 + 1, and W, H <= 32767, so the count is bounded by
// ST_MAXPX/1024 + 2 * 1024 + 1 (checked again per call).
constexpr size_t ST_MAX_BLOCKS = ST_MAXPX / 1024 + 2 * 1024 + 1;
constexpr size_t ST_BITMAP_WORDS = (ST_MAX_BLOCKS + 31) / 32;

constexpr size_t OFF_FLAGS = 0;
constexpr size_t OFF_SCR4 = align256(OFF_FLAGS + sizeof(DeviceFlags));
constexpr size_t OFF_VARY = align256(OFF_SCR4 + ST_MAXV * sizeof(float4));
constexpr size_t OFF_SETUP = align256(OFF_VARY + ST_MAXV * VSTRIDE * sizeof(float));
constexpr size_t OFF_BINRECT = align256(OFF_SETUP + 4 * ST_MAXT * sizeof(float4));
constexpr size_t OFF_AREA = align256(OFF_BINRECT + ST_MAXT * sizeof(uint2));
constexpr size_t OFF_BIG = align256(OFF_AREA + (ST_MAXT + 1) * sizeof(unsigned long long));
constexpr size_t OFF_UNSAFE = align256(OFF_BIG + (ST_MAXT + 1) * sizeof(uint32_t));
constexpr size_t OFF_GKEYS = align256(OFF_UNSAFE + ST_MAXT * sizeof(uint32_t));
constexpr size_t OFF_BITMAP = align256(OFF_GKEYS + ST_MAXPX * sizeof(unsigned long long));
constexpr size_t ST_BYTES = align256(OFF_BITMAP + ST_BITMAP_WORDS * sizeof(uint32_t));
static_assert(ST_BYTES < (18u << 20), "static scratch grew past its stated size");

// The scratch itself.  Shared by every call on a device; see sr_render_static
// in include/sr.h for what that means for concurrent calls.
static __device__ __align__(256) unsigned char g_static_scratch[ST_BYTES];

constexpr int ST_MAX_DEVICES = 64;
std::mutex g_scratch_mu;
unsigned char* g_scratch_ptr[ST_MAX_DEVICES] = {};

// Device address of g_static_scratch on the current device (looked up once).
int scratch_address(unsigned char** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return SR_ECUDA;
    if (dev < 0 || dev >= ST_MAX_DEVICES) return SR_EINVAL;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) return SR_ECUDA;
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return SR_OK;
}

int min_varyings(int fs) {
    switch (fs) {
    case FS_TEXTURED_BLINN_PHONG: return 10;
    case FS_VERTEX_COLOR: return 4;
    case FS_CONSTANT_COLOR: return 0;
    default: return 8;
    }
}

bool aligned(const void* p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) == 0; }

}  // namespace

extern "C" SR_API int sr_render_static(const sr_draw* d, const void* uniforms, size_t uniforms_size,
                                       const float* planes, uint32_t n_planes, uint32_t plane_stride,
                                       uint32_t n_verts, const uint32_t* indices, uint32_t n_triangles,
                                       const uint32_t* texture, uint32_t tex_w, uint32_t tex_h,
                                       const sr_fb_desc* fb, void* color, float* depth, void* stream) {
    // ---- arguments (the checks sr_render makes, plus this variant's limits)
    if (!d || !fb || !uniforms || uniforms_size != sizeof(sr_uniforms)) return SR_EINVAL;
    if (d->mesh || d->texture) return SR_EINVAL;               // handles are for sr_render
    if (d->prim != SR_PRIM_TRIANGLE || d->gs_mode != SR_GS_NONE || d->blend != BLEND_REPLACE) return SR_EINVAL;
    if (d->reuse != SR_REUSE_NONE) return SR_EINVAL;           // no previous draw to refer to
    if (d->vs < 0 || d->vs >= VS_COUNT || d->fs < 0 || d->fs >= FS_COUNT) return SR_EINVAL;
    if (d->tile_w == 0 || d->tile_h == 0 || d->tile_w > 65535 || d->tile_h > 65535) return SR_EINVAL;
    if (d->tex_filter > SR_SAMPLE_BILINEAR || d->tex_edge > SR_SAMPLE_BORDER) return SR_EINVAL;
    if (d->cull > SR_CULL_COUNTER_CLOCKWISE) return SR_EINVAL;
    if (vs_nk(d->vs) < min_varyings(d->fs)) return SR_EINVAL;
    if (fb->width == 0 || fb->height == 0 || fb->width > 32767 || fb->height > 32767) return SR_EINVAL;
    if (fb->color_format > SR_COLOR_RGBA8 || fb->stencil) return SR_EINVAL;
    if (fb->color_format != SR_COLOR_NONE && !color) return SR_EINVAL;
    if (fb->depth && !depth) return SR_EINVAL;
    if (n_planes < (uint32_t)vs_planes(d->vs) || n_planes > (uint32_t)MAX_PLANES) return SR_EINVAL;
    if (n_verts && (!planes || plane_stride < n_verts || (plane_stride & 3u) || !aligned(planes, 16))) return SR_EINVAL;
    if (n_triangles && (!indices || n_verts == 0)) return SR_EINVAL;
    if (d->fs == FS_TEXTURED_BLINN_PHONG && (!texture || tex_w == 0 || tex_h == 0)) return SR_EINVAL;
    if (!aligned(indices, 4) || !aligned(texture, 4) || !aligned(depth, 4) ||
        !aligned(color, fb->color_format == SR_COLOR_RGBA32F ? 16 : 4))
        return SR_EINVAL;
    // sizes beyond the fixed scratch
    if ((uint64_t)fb->width * fb->height > SR_STATIC_MAX_PIXELS || n_triangles > SR_STATIC_MAX_TRIANGLES ||
        n_verts > SR_STATIC_MAX_VERTICES)
        return SR_EOVERFLOW;

    const uint32_t W = fb->width, H = fb->height;
    if (W < 2 || H < 2 || n_triangles == 0 || n_verts == 0) return SR_OK;   // no semantic tiles / nothing to draw
    const size_t nblk = (size_t)((W + 31) / 32) * ((H + 31) / 32);
    if ((nblk + 31) / 32 > ST_BITMAP_WORDS) return SR_EOVERFLOW;

    unsigned char* base = nullptr;
    int rc = scratch_address(&base);
    if (rc != SR_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    DeviceFlags* flags = reinterpret_cast<DeviceFlags*>(base + OFF_FLAGS);
    float4* scr4 = reinterpret_cast<float4*>(base + OFF_SCR4);
    float* vary = reinterpret_cast<float*>(base + OFF_VARY);
    float4* setup = reinterpret_cast<float4*>(base + OFF_SETUP);
    uint32_t* binrect = reinterpret_cast<uint32_t*>(base + OFF_BINRECT);
    unsigned long long* area = reinterpret_cast<unsigned long long*>(base + OFF_AREA);
    uint32_t* big_list = reinterpret_cast<uint32_t*>(base + OFF_BIG);
    uint32_t* unsafe_list = reinterpret_cast<uint32_t*>(base + OFF_UNSAFE);
    unsigned long long* gkeys = reinterpret_cast<unsigned long long*>(base + OFF_GKEYS);
    uint32_t* bitmap = reinterpret_cast<uint32_t*>(base + OFF_BITMAP);

    // ---- draw parameters: the values sr_render derives for this draw
    DrawParams P;
    std::memset(&P, 0, sizeof(P));
    P.W = W; P.H = H;
    P.tile_w = d->tile_w; P.tile_h = d->tile_h;
    P.magic_w = div_magic(d->tile_w); P.magic_h = div_magic(d->tile_h);
    P.ncols = (W - 1 + d->tile_w - 1) / d->tile_w;
    P.nrows = (H - 1 + d->tile_h - 1) / d->tile_h;
    P.n_verts = n_verts;
    P.gen_base = plane_stride;
    P.n_in = n_triangles;
    P.cull = d->cull;
    P.vs = d->vs; P.fs = d->fs; P.blend = BLEND_REPLACE;
    std::memcpy(P.vp, &d->viewport, sizeof(P.vp));
    P.has_depth = fb->depth ? 1u : 0u;
    P.has_stencil = 0;
    P.color_format = fb->color_format;
    P.stencil_test = SR_STENCIL_ALWAYS;
    P.stencil_op = SR_STENCIL_KEEP;
    P.stencil_wrap = 1;
    if (texture) { P.tex_w = tex_w; P.tex_h = tex_h; }
    P.tex_filter = d->tex_filter; P.tex_edge = d->tex_edge;
    P.bin_w_log2 = 5; P.bin_h_log2 = 5;
    P.bins_x = (W + 31) >> 5;
    P.bins_y = (H + 31) >> 5;
    P.n_raster_host = n_triangles;

    sr_uniforms U;
    std::memcpy(&U, uniforms, sizeof(U));
    sr_uniforms_derive(&U);

    // ---- what must start at zero: the counters and error flags, the winner
    // key of every pixel of this frame size, and the touched-block bitmap.
    // The previous call leaves keys and bitmap zero when it completes, but a
    // call that raced with another one may not have.
    if (cudaMemsetAsync(flags, 0, sizeof(DeviceFlags), st) != cudaSuccess ||
        cudaMemsetAsync(gkeys, 0, (size_t)W * H * sizeof(unsigned long long), st) != cudaSuccess ||
        cudaMemsetAsync(bitmap, 0, ((nblk + 31) / 32) * sizeof(uint32_t), st) != cudaSuccess)
        return SR_ECUDA;

    sr_mesh m{};   // a view of the caller's buffers (owns nothing)
    m.planes = const_cast<float*>(planes);
    m.n_planes = n_planes;
    m.n_verts = n_verts;
    m.n_pad = plane_stride;
    m.indices = const_cast<uint32_t*>(indices);
    m.n_indices = 3ull * n_triangles;

    VertexStore vs{nullptr, scr4, vary, (uint32_t)ST_MAXV};
    StencilCountArgs S{nullptr, nullptr, nullptr};
    launch_vertex(P, U, &m, vs, false, st);
    launch_setup_bin(P, indices, vs, setup, binrect, nullptr, nullptr, nullptr, nullptr, nullptr, unsafe_list, nullptr, area,
                     S, flags, st);
    OpaqueArgs A{setup, area, big_list, gkeys, bitmap, unsafe_list, nullptr, indices, vary, texture,
                 fb->color_format != SR_COLOR_NONE ? color : nullptr, fb->depth ? depth : nullptr, nullptr, 0u,
                 flags};
    launch_opaque(P, U, A, st);
    return cudaGetLastError() == cudaSuccess ? SR_OK : SR_ECUDA;
}
