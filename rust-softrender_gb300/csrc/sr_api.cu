// sr_api.cu — the C ABI (include/sr.h): pipeline, framebuffer, resources,
// shader registry and the stream-ordered draw orchestration.
//
// A draw is enqueued without host synchronisation: intermediate buffers have
// grow-only capacities; a stage that would overflow one records the size it
// needed and poisons the pipeline, after which every framebuffer-writing
// kernel of that draw and of later draws skips.  sr_sync() then grows the
// buffers and replays the draws from the first poisoned one, so the
// framebuffer always ends up exactly as if capacities had been large enough.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sr_internal.cuh"
#include "sr_scan.cuh"

using namespace sr;

#include "sr_host.h"

namespace {

uint32_t bytes_per_color(uint32_t f) { return f == SR_COLOR_RGBA32F ? 16 : f == SR_COLOR_RGBA8 ? 4 : 0; }

// Mesh contents versions, unique across meshes (a freed mesh's address can
// come back for a new one), checked by sr_draw.reuse.
uint64_t next_mesh_version() {
    static std::atomic<uint64_t> v{0};
    return ++v;
}

struct ShaderName { const char* name; int stage; int id; };
const ShaderName kShaders[] = {
    {"mvp_pos_nrm", SR_STAGE_VERTEX, VS_MVP_POS_NRM},
    {"mvp_pos_nrm_uv", SR_STAGE_VERTEX, VS_MVP_POS_NRM_UV},
    {"clip_color", SR_STAGE_VERTEX, VS_CLIP_COLOR},
    {"clip_rgba8", SR_STAGE_VERTEX, VS_CLIP_RGBA8},
    {"clip", SR_STAGE_GEOMETRY, GS_CLIP},
    {"vertex_normals", SR_STAGE_GEOMETRY, GS_VERTEX_NORMALS},
    {"face_normals", SR_STAGE_GEOMETRY, GS_FACE_NORMALS},
    {"blinn_phong_dir", SR_STAGE_FRAGMENT, FS_BLINN_PHONG_DIR},
    {"textured_blinn_phong", SR_STAGE_FRAGMENT, FS_TEXTURED_BLINN_PHONG},
    {"vertex_color", SR_STAGE_FRAGMENT, FS_VERTEX_COLOR},
    {"aces_lights", SR_STAGE_FRAGMENT, FS_ACES_LIGHTS},
    {"constant_color", SR_STAGE_FRAGMENT, FS_CONSTANT_COLOR},
    {"replace", SR_STAGE_BLEND, BLEND_REPLACE},
    {"over", SR_STAGE_BLEND, BLEND_OVER},
};

// Clears a colour plane (cn 32-bit words, pattern cv repeating every 4 words),
// a depth plane (dn words of dv) and a stencil plane (sn bytes of 0) with
// 16-byte stores in one launch.  Like every framebuffer write of a draw it
// does nothing once the pipeline is poisoned: sr_sync then replays the draws
// from the first poisoned one with the clears between them in their places,
// and that replay must start from the framebuffer as the poisoned draw found it.
__global__ void clear_planes_kernel(const DeviceFlags* __restrict__ flags, uint32_t* __restrict__ c, size_t cn, uint4 cv,
                                    uint32_t* __restrict__ d, size_t dn, uint32_t dv, uint8_t* __restrict__ s, size_t sn) {
    if (flags->poison) return;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    const size_t c4 = cn / 4, d4 = dn / 4, s16 = sn / 16;
    const uint4 dv4 = make_uint4(dv, dv, dv, dv);
    for (size_t j = i; j < c4; j += stride) reinterpret_cast<uint4*>(c)[j] = cv;
    for (size_t j = i; j < d4; j += stride) reinterpret_cast<uint4*>(d)[j] = dv4;
    for (size_t j = i; j < s16; j += stride) reinterpret_cast<uint4*>(s)[j] = make_uint4(0, 0, 0, 0);
    if (i < cn - 4 * c4) c[4 * c4 + i] = (&cv.x)[i & 3];
    if (i < dn - 4 * d4) d[4 * d4 + i] = dv;
    if (i < sn - 16 * s16) s[16 * s16 + i] = 0;
}

// Copies n 32-bit words of a colour plane into a texture unless the pipeline
// is poisoned: a draw replayed by sr_sync may sample the texture, and must
// find it as it was when the draw was first enqueued.
__global__ void copy_plane_kernel(const DeviceFlags* __restrict__ flags, uint32_t* __restrict__ dst,
                                  const uint32_t* __restrict__ src, size_t n) {
    if (flags->poison) return;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    const size_t n4 = n / 4;
    for (size_t j = i; j < n4; j += stride)
        reinterpret_cast<uint4*>(dst)[j] = reinterpret_cast<const uint4*>(src)[j];
    if (i < n - 4 * n4) dst[4 * n4 + i] = src[4 * n4 + i];
}

// The unit expansion of n RGBA8 texels: each channel c as c / 255
// (sr_u8_unit, the sampler's own conversion).
__global__ void expand_texels_kernel(const uint32_t* __restrict__ src, float4* __restrict__ dst, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const sr_v4 c = sr_from_rgba8(src[i]);
        dst[i] = make_float4(c.x, c.y, c.z, c.w);
    }
}

// Rebuilds an RGBA8 texture's unit expansion from its texels on `st`.
int texture_expand(sr_texture* t, cudaStream_t st) {
    if (!t || t->f32 || t->view || !t->unit) return SR_OK;
    const size_t n = (size_t)t->w * t->h;
    const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
    expand_texels_kernel<<<grid, 256, 0, st>>>(t->data, t->unit, n);
    SR_CK(cudaGetLastError());
    return SR_OK;
}

int fs_min_varyings(int fs) {
    switch (fs) {
    case FS_TEXTURED_BLINN_PHONG: return 10;
    case FS_VERTEX_COLOR: return 4;
    case FS_CONSTANT_COLOR: return 0;
    default: return 8;
    }
}

}  // namespace

// =================================================================== misc
extern "C" SR_API const char* sr_status_string(int s) {
    switch (s) {
    case SR_OK: return "SR_OK";
    case SR_EINVAL: return "SR_EINVAL";
    case SR_ENOMEM: return "SR_ENOMEM";
    case SR_EBUDGET: return "SR_EBUDGET";
    case SR_EOVERFLOW: return "SR_EOVERFLOW";
    case SR_ETIMEOUT: return "SR_ETIMEOUT";
    case SR_ECUDA: return "SR_ECUDA";
    case SR_ENAN: return "SR_ENAN";
    case SR_ENOTFOUND: return "SR_ENOTFOUND";
    case SR_EBUSY: return "SR_EBUSY";
    default: return "SR_UNKNOWN";
    }
}

extern "C" SR_API const char* sr_version(void) { return "softrender-gb300 0.1.0 sm_103a"; }

extern "C" SR_API int sr_shader_lookup(const char* name, int stage, int* id) {
    if (!name || !id) return SR_EINVAL;
    for (const auto& s : kShaders)
        if (s.stage == stage && std::strcmp(s.name, name) == 0) { *id = s.id; return SR_OK; }
    return SR_ENOTFOUND;
}

extern "C" SR_API void sr_draw_init(sr_draw* d) {
    std::memset(d, 0, sizeof(*d));
    d->prim = SR_PRIM_TRIANGLE;
    d->vs = VS_MVP_POS_NRM;
    d->gs_mode = SR_GS_NONE;
    d->gs = GS_CLIP;
    d->cull = SR_CULL_NONE;
    d->fs = FS_BLINN_PHONG_DIR;
    d->blend = BLEND_REPLACE;
    d->tile_w = 128;
    d->tile_h = 128;
    d->tex_filter = SR_SAMPLE_BILINEAR;
    d->tex_edge = SR_SAMPLE_CLAMP;
}

// =============================================================== pipeline
extern "C" SR_API int sr_pipeline_create(const sr_fb_desc* fb, const void* uniforms, size_t usz, sr_pipeline** out) {
    if (!fb || !out) return SR_EINVAL;
    *out = nullptr;
    if (fb->width == 0 || fb->height == 0) return SR_EINVAL;               // mod.rs:129-130
    if (fb->width > 32767 || fb->height > 32767) return SR_EINVAL;
    if (fb->color_format > SR_COLOR_RGBA8) return SR_EINVAL;
    if (uniforms && usz != sizeof(sr_uniforms)) return SR_EINVAL;
    sr_pipeline* p = nullptr;
    const int rc = pipeline_create_cap(fb, (size_t)fb->width * fb->height, &p);
    if (rc != SR_OK) return rc;
    if (uniforms) {
        std::memcpy(&p->U, uniforms, sizeof(sr_uniforms));
        sr_uniforms_derive(&p->U);
    }
    *out = p;
    return SR_OK;
}

int sr::pipeline_create_cap(const sr_fb_desc* fb, size_t cap_px, sr_pipeline** out) {
    sr_pipeline* p = new (std::nothrow) sr_pipeline();
    if (!p) return SR_ENOMEM;
    p->fb = *fb;
    std::memset(&p->U, 0, sizeof(p->U));
    sr_uniforms_derive(&p->U);
    const size_t n = std::max(cap_px, (size_t)fb->width * fb->height);
    p->cap_px = n;
    cudaError_t e = cudaSuccess;
    if (bytes_per_color(fb->color_format)) {
        p->color_plane = new (std::nothrow) sr_color_plane();
        if (!p->color_plane) { sr_pipeline_destroy(p); return SR_ENOMEM; }
        e = cudaMalloc(&p->color_plane->data, n * bytes_per_color(fb->color_format));
        p->color = p->color_plane->data;
    }
    if (e == cudaSuccess && fb->depth) e = cudaMalloc(&p->depth, n * 4);
    if (e == cudaSuccess && fb->stencil) e = cudaMalloc(&p->stencil, n);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&p->flags, sizeof(DeviceFlags));
    if (e == cudaSuccess) e = cudaMallocHost(&p->hflags, sizeof(DeviceFlags));
    if (e != cudaSuccess) {
        last_cuda_error() = e;
        sr_pipeline_destroy(p);
        return e == cudaErrorMemoryAllocation ? SR_ENOMEM : SR_ECUDA;
    }
    p->stream = p->own_stream;
    const char* fu = std::getenv("SR_FORCE_UNSAFE");
    p->force_unsafe = fu && fu[0] == '1';
    const char* ok = std::getenv("SR_OPAQUE_KEYS");
    p->opaque_keys = ok && ok[0] == '1';
    DeviceFlags z;
    std::memset(&z, 0, sizeof(z));
    z.poison_draw = 0xffffffffu;
    cudaMemcpy(p->flags, &z, sizeof(z), cudaMemcpyHostToDevice);
    std::memset(&p->last_stats, 0, sizeof(p->last_stats));
    // Framebuffer starts cleared (colour 0), like RenderBuffer::with_dimensions
    uint8_t zero[16] = {0};
    int st = sr_framebuffer_clear(p, zero);
    if (st != SR_OK) { sr_pipeline_destroy(p); return st; }
    cudaStreamSynchronize(p->stream);
    *out = p;
    return SR_OK;
}

int sr::pipeline_retarget(sr_pipeline* p, uint32_t width, uint32_t height) {
    if (!p || width == 0 || height == 0 || width > 32767 || height > 32767) return SR_EINVAL;
    if ((size_t)width * height > p->cap_px || !p->pending.empty()) return SR_EINVAL;
    p->fb.width = width;
    p->fb.height = height;
    return SR_OK;
}

extern "C" SR_API int sr_pipeline_destroy(sr_pipeline* p) {
    if (!p) return SR_EINVAL;
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (const auto& pd : p->pending) {
        mesh_unref(pd.d.mesh);
        texture_unref(pd.d.texture);
    }
    p->pending.clear();
    color_plane_unref(p->color_plane);   // texture views may still hold the plane
    if (p->depth) cudaFree(p->depth);
    if (p->stencil) cudaFree(p->stencil);
    if (p->flags) cudaFree(p->flags);
    if (p->hflags) cudaFreeHost(p->hflags);
    p->clip4.release(); p->scr4.release(); p->vary.release();
    p->clip_counts.release(); p->clip_offsets.release(); p->clip_tmp.release(); p->refs.release();
    p->setup.release(); p->unsafe_rect.release(); p->binrect.release();
    p->bin_counts.release(); p->bin_off.release(); p->bin_cursor.release(); p->bin_tmp.release(); p->entries.release(); p->unsafe_list.release();
    p->st_diff.release(); p->st_lines.release(); p->st_glob.release();
    p->area.release(); p->big_list.release(); p->gids.release(); p->gkeys.release(); p->bitmap.release();
    p->lpv.release(); p->lpvalid.release();
    p->pcount.release(); p->poff.release(); p->pkeys0.release(); p->pkeys1.release(); p->pvals0.release();
    p->pvals1.release(); p->hist.release(); p->hist_off.release(); p->ranges.release();
    for (auto& e : p->ev) if (e) cudaEventDestroy(e);
    if (p->own_stream) cudaStreamDestroy(p->own_stream);
    delete p;
    return SR_OK;
}

extern "C" SR_API int sr_pipeline_set_uniforms(sr_pipeline* p, const void* uniforms, size_t usz) {
    if (!p || !uniforms || usz != sizeof(sr_uniforms)) return SR_EINVAL;
    std::memcpy(&p->U, uniforms, sizeof(sr_uniforms));
    sr_uniforms_derive(&p->U);
    return SR_OK;
}

extern "C" SR_API int sr_pipeline_set_profiling(sr_pipeline* p, int enable) {
    if (!p) return SR_EINVAL;
    if (enable && !p->ev[0])
        for (auto& e : p->ev) SR_CK(cudaEventCreate(&e));
    p->profiling = enable != 0;
    return SR_OK;
}

extern "C" SR_API int sr_pipeline_set_stencil(sr_pipeline* p, int test, int op, int wrap) {
    if (!p || test < 0 || test > SR_STENCIL_NOT_EQUAL || op < 0 || op > SR_STENCIL_DECREMENT) return SR_EINVAL;
    p->stencil_test = (uint32_t)test;
    p->stencil_op = (uint32_t)op;
    p->stencil_wrap = wrap ? 1u : 0u;
    return SR_OK;
}

extern "C" SR_API int sr_sync(sr_pipeline* p);

extern "C" SR_API int sr_pipeline_set_stream(sr_pipeline* p, void* stream) {
    if (!p) return SR_EINVAL;
    // sr_sync waits on the current stream: settle draws enqueued on the old
    // one first (their status is kept for the next sr_sync)
    if (!p->pending.empty()) {
        const int st = sr_sync(p);
        if (st != SR_OK && p->deferred_status == SR_OK) p->deferred_status = st;
    }
    p->stream = stream ? (cudaStream_t)stream : p->own_stream;
    return SR_OK;
}

// ============================================================ framebuffer
static int enqueue_clear(sr_pipeline* p, const void* color) {
    size_t n = (size_t)p->fb.width * p->fb.height;
    uint4 cv = make_uint4(0, 0, 0, 0);
    size_t cn = 0;
    if (p->fb.color_format == SR_COLOR_RGBA32F) {
        std::memcpy(&cv, color, 16);
        cn = 4 * n;
    } else if (p->fb.color_format == SR_COLOR_RGBA8) {
        uint32_t c;
        std::memcpy(&c, color, 4);
        cv = make_uint4(c, c, c, c);
        cn = n;
    }
    const float far_ = -3.40282347e+38f;  // f32::MIN (attachments/depth.rs:31)
    uint32_t dv;
    std::memcpy(&dv, &far_, 4);
    const size_t dn = p->depth ? n : 0;
    const size_t sn = p->stencil ? n : 0;
    const size_t work = std::max(std::max(cn, dn) / 4, sn / 16) + 16;
    const unsigned grid = (unsigned)std::min<size_t>((work + 255) / 256, 152 * 16);
    if (cn || dn || sn)
        clear_planes_kernel<<<grid, 256, 0, p->stream>>>(p->flags, reinterpret_cast<uint32_t*>(p->color), cn, cv,
                                                         reinterpret_cast<uint32_t*>(p->depth), dn, dv,
                                                         p->stencil, sn);
    SR_CK(cudaGetLastError());
    return SR_OK;
}

// Framebuffer::clear.  A clear between draws that sr_sync has not settled yet
// is recorded with them: a replay after an overflow re-runs it in sequence.
extern "C" SR_API int sr_framebuffer_clear(sr_pipeline* p, const void* color) {
    if (!p || !color) return SR_EINVAL;
    const int rc = enqueue_clear(p, color);
    if (rc == SR_OK && !p->pending.empty()) {
        PendingDraw pc{};
        pc.kind = PENDING_CLEAR;
        const uint32_t f = p->fb.color_format;
        std::memcpy(pc.clear_color, color, f == SR_COLOR_RGBA32F ? 16 : f == SR_COLOR_RGBA8 ? 4 : 0);
        p->pending.push_back(pc);
    }
    return rc;
}

extern "C" SR_API int sr_sync(sr_pipeline* p);

extern "C" SR_API int sr_framebuffer_read(sr_pipeline* p, void* color, float* depth, uint8_t* stencil) {
    if (!p) return SR_EINVAL;
    int st = sr_sync(p);
    size_t n = (size_t)p->fb.width * p->fb.height;
    if (color && p->color) SR_CK(cudaMemcpyAsync(color, p->color, n * bytes_per_color(p->fb.color_format), cudaMemcpyDeviceToHost, p->stream));
    if (depth && p->depth) SR_CK(cudaMemcpyAsync(depth, p->depth, n * 4, cudaMemcpyDeviceToHost, p->stream));
    if (stencil && p->stencil) SR_CK(cudaMemcpyAsync(stencil, p->stencil, n, cudaMemcpyDeviceToHost, p->stream));
    SR_CK(cudaStreamSynchronize(p->stream));
    return st;
}

extern "C" SR_API int sr_framebuffer_write(sr_pipeline* p, const void* color, const float* depth, const uint8_t* stencil) {
    if (!p) return SR_EINVAL;
    // the host planes cannot be replayed later: settle the pending draws
    // first (their status is kept for the next sr_sync)
    if (!p->pending.empty()) {
        const int st = sr_sync(p);
        if (st != SR_OK && p->deferred_status == SR_OK) p->deferred_status = st;
    }
    size_t n = (size_t)p->fb.width * p->fb.height;
    if (color && p->color) SR_CK(cudaMemcpyAsync(p->color, color, n * bytes_per_color(p->fb.color_format), cudaMemcpyHostToDevice, p->stream));
    if (depth && p->depth) SR_CK(cudaMemcpyAsync(p->depth, depth, n * 4, cudaMemcpyHostToDevice, p->stream));
    if (stencil && p->stencil) SR_CK(cudaMemcpyAsync(p->stencil, stencil, n, cudaMemcpyHostToDevice, p->stream));
    SR_CK(cudaStreamSynchronize(p->stream));
    return SR_OK;
}

extern "C" SR_API int sr_framebuffer_device_ptrs(sr_pipeline* p, void** color, float** depth, uint8_t** stencil) {
    if (!p) return SR_EINVAL;
    if (color) *color = p->color;
    if (depth) *depth = p->depth;
    if (stencil) *stencil = p->stencil;
    return SR_OK;
}

// ============================================================== resources
extern "C" SR_API int sr_mesh_upload(const float* const* planes, uint32_t n_planes, uint32_t n_verts,
                                     const uint32_t* indices, uint64_t n_indices, sr_mesh** out) {
    if (!out || (n_planes && !planes) || n_planes > (uint32_t)MAX_PLANES || (n_indices && !indices)) return SR_EINVAL;
    *out = nullptr;
    // vertex references are u32: the padded planes plus the geometry stage's
    // generated vertices (at most 2^30) stay below 2^32
    if (n_verts > (1u << 31)) return SR_EINVAL;
    for (uint64_t i = 0; i < n_indices; ++i)
        if (indices[i] >= n_verts) return SR_EINVAL;
    if (n_indices / 3 > (1ull << 30)) return SR_EINVAL;
    sr_mesh* m = new (std::nothrow) sr_mesh();
    if (!m) return SR_ENOMEM;
    m->n_planes = n_planes;
    m->n_verts = n_verts;
    m->n_pad = (n_verts + 3) & ~3u;
    m->n_indices = n_indices;
    m->planes = nullptr;
    m->indices = nullptr;
    size_t pb = (size_t)m->n_pad * n_planes * 4;
    cudaError_t e = cudaSuccess;
    if (pb) e = cudaMalloc(&m->planes, pb);
    if (e == cudaSuccess && pb) e = cudaMemset(m->planes, 0, pb);
    for (uint32_t j = 0; e == cudaSuccess && j < n_planes; ++j)
        e = cudaMemcpy(m->planes + (size_t)j * m->n_pad, planes[j], (size_t)n_verts * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_indices) e = cudaMalloc(&m->indices, n_indices * 4);
    if (e == cudaSuccess && n_indices) e = cudaMemcpy(m->indices, indices, n_indices * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        last_cuda_error() = e;
        if (m->planes) cudaFree(m->planes);
        if (m->indices) cudaFree(m->indices);
        delete m;
        return e == cudaErrorMemoryAllocation ? SR_ENOMEM : SR_ECUDA;
    }
    m->bytes = pb + n_indices * 4;
    m->version = next_mesh_version();
    *out = m;
    return SR_OK;
}

extern "C" SR_API int sr_mesh_update(sr_mesh* m, const float* const* planes, uint32_t n_planes, uint32_t n_verts,
                                     const uint32_t* indices, uint64_t n_indices, void* stream) {
    if (!m || n_planes != m->n_planes || n_verts != m->n_verts || n_indices != m->n_indices) return SR_EINVAL;
    if ((n_planes && !planes) || (n_indices && !indices)) return SR_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    m->version = next_mesh_version();   // before the copies: a failed update also invalidates
    for (uint32_t j = 0; j < n_planes; ++j)
        SR_CK(cudaMemcpyAsync(m->planes + (size_t)j * m->n_pad, planes[j], (size_t)n_verts * 4, cudaMemcpyHostToDevice, st));
    if (n_indices) SR_CK(cudaMemcpyAsync(m->indices, indices, n_indices * 4, cudaMemcpyHostToDevice, st));
    if (!stream) SR_CK(cudaStreamSynchronize(st));
    return SR_OK;
}

void sr::mesh_unref(const sr_mesh* cm) {
    sr_mesh* m = const_cast<sr_mesh*>(cm);
    if (!m || m->refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
    if (m->planes) cudaFree(m->planes);
    if (m->indices) cudaFree(m->indices);
    delete m;
}

// Releases the caller's reference; draws still pending on a pipeline (until
// its sr_sync) and queued server requests keep the mesh alive.
extern "C" SR_API int sr_mesh_free(sr_mesh* m) {
    if (!m) return SR_EINVAL;
    mesh_unref(m);
    return SR_OK;
}

extern "C" SR_API uint64_t sr_mesh_bytes(const sr_mesh* m) { return m ? m->bytes : 0; }

extern "C" SR_API int sr_texture_upload(const uint32_t* rgba8, uint32_t w, uint32_t h, sr_texture** out) {
    if (!out || !rgba8 || w == 0 || h == 0) return SR_EINVAL;
    *out = nullptr;
    sr_texture* t = new (std::nothrow) sr_texture();
    if (!t) return SR_ENOMEM;
    t->w = w;
    t->h = h;
    cudaError_t e = cudaMalloc(&t->data, (size_t)w * h * 4);
    if (e == cudaSuccess) e = cudaMalloc(&t->unit, (size_t)w * h * 16);
    if (e == cudaSuccess) e = cudaMemcpy(t->data, rgba8, (size_t)w * h * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && texture_expand(t, nullptr) != SR_OK) e = last_cuda_error();
    if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
    if (e != cudaSuccess) {
        last_cuda_error() = e;
        if (t->data) cudaFree(t->data);
        if (t->unit) cudaFree(t->unit);
        delete t;
        return e == cudaErrorMemoryAllocation ? SR_ENOMEM : SR_ECUDA;
    }
    *out = t;
    return SR_OK;
}

extern "C" SR_API int sr_texture_upload_rgba32f(const float* rgba, uint32_t w, uint32_t h, sr_texture** out) {
    if (!out || !rgba || w == 0 || h == 0) return SR_EINVAL;
    *out = nullptr;
    sr_texture* t = new (std::nothrow) sr_texture();
    if (!t) return SR_ENOMEM;
    t->w = w;
    t->h = h;
    t->f32 = 1;
    cudaError_t e = cudaMalloc(&t->data, (size_t)w * h * 16);
    if (e == cudaSuccess) e = cudaMemcpy(t->data, rgba, (size_t)w * h * 16, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        last_cuda_error() = e;
        if (t->data) cudaFree(t->data);
        delete t;
        return e == cudaErrorMemoryAllocation ? SR_ENOMEM : SR_ECUDA;
    }
    *out = t;
    return SR_OK;
}

extern "C" SR_API int sr_texture_view_framebuffer(sr_pipeline* p, sr_texture** out) {
    if (!p || !out) return SR_EINVAL;
    *out = nullptr;
    if (!p->color || (p->fb.color_format != SR_COLOR_RGBA8 && p->fb.color_format != SR_COLOR_RGBA32F))
        return SR_EINVAL;
    sr_texture* t = new (std::nothrow) sr_texture();
    if (!t) return SR_ENOMEM;
    t->data = static_cast<uint32_t*>(p->color);
    t->w = p->fb.width;
    t->h = p->fb.height;
    t->f32 = p->fb.color_format == SR_COLOR_RGBA32F ? 1u : 0u;
    t->view = true;
    t->plane = p->color_plane;
    t->plane->refs.fetch_add(1, std::memory_order_relaxed);
    *out = t;
    return SR_OK;
}

extern "C" SR_API int sr_texture_update(sr_texture* t, const uint32_t* rgba8, uint32_t w, uint32_t h, void* stream) {
    if (!t || !rgba8 || w != t->w || h != t->h || t->f32 || t->view) return SR_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    SR_CK(cudaMemcpyAsync(t->data, rgba8, (size_t)w * h * 4, cudaMemcpyHostToDevice, st));
    const int rc = texture_expand(t, st);
    if (rc != SR_OK) return rc;
    if (!stream) SR_CK(cudaStreamSynchronize(st));
    return SR_OK;
}

static int enqueue_texture_copy(sr_pipeline* p, const sr_texture* t) {
    const size_t n = (size_t)t->w * t->h * (t->f32 ? 4 : 1);
    const unsigned grid = (unsigned)std::min<size_t>((n / 4 + 4 + 255) / 256, 152 * 16);
    copy_plane_kernel<<<grid, 256, 0, p->stream>>>(p->flags, t->data, static_cast<const uint32_t*>(p->color), n);
    SR_CK(cudaGetLastError());
    return texture_expand(const_cast<sr_texture*>(t), p->stream);
}

extern "C" SR_API int sr_texture_from_framebuffer(sr_pipeline* p, sr_texture* t) {
    if (!p || !t || t->view || !p->color) return SR_EINVAL;
    const uint32_t f = p->fb.color_format;
    if ((f != SR_COLOR_RGBA8 && f != SR_COLOR_RGBA32F) || t->f32 != (f == SR_COLOR_RGBA32F ? 1u : 0u)) return SR_EINVAL;
    if (t->w != p->fb.width || t->h != p->fb.height) return SR_EINVAL;
    const int rc = enqueue_texture_copy(p, t);
    if (rc == SR_OK && !p->pending.empty()) {   // repeated in sequence if sync replays the draws
        PendingDraw pt{};
        pt.kind = PENDING_TEXTURE_COPY;
        pt.d.texture = t;
        texture_ref(t);
        p->pending.push_back(pt);
    }
    return rc;
}

void sr::texture_unref(const sr_texture* ct) {
    sr_texture* t = const_cast<sr_texture*>(ct);
    if (!t || t->refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
    if (t->view) color_plane_unref(t->plane);
    else if (t->data) cudaFree(t->data);
    if (t->unit) cudaFree(t->unit);
    delete t;
}

extern "C" SR_API int sr_texture_free(sr_texture* t) {
    if (!t) return SR_EINVAL;
    texture_unref(t);
    return SR_OK;
}

// ================================================================ render
namespace {

// `replay`: re-enqueued by sr_sync after an overflow (stage outputs are then
// always recomputed, from the saved inputs of the draw).
int enqueue_draw(sr_pipeline* p, const PendingDraw& pd, uint32_t draw_id, bool replay) {
    const sr_draw* d = &pd.d;
    const sr_mesh* m = d->mesh;
    cudaStream_t st = p->stream;
    const uint32_t W = p->fb.width, H = p->fb.height;
    DrawParams P;
    std::memset(&P, 0, sizeof(P));
    P.W = W; P.H = H;
    P.tile_w = d->tile_w; P.tile_h = d->tile_h;
    P.magic_w = div_magic(d->tile_w); P.magic_h = div_magic(d->tile_h);
    P.ncols = W >= 2 ? (W - 1 + d->tile_w - 1) / d->tile_w : 0;
    P.nrows = H >= 2 ? (H - 1 + d->tile_h - 1) / d->tile_h : 0;
    P.n_verts = m->n_verts;
    P.gen_base = m->n_pad;
    P.n_in = (uint32_t)(m->n_indices / std::max(1u, d->prim));
    P.cull = d->cull;
    P.vs = d->vs; P.fs = d->fs; P.blend = d->blend;
    std::memcpy(P.vp, &d->viewport, sizeof(P.vp));
    P.has_depth = p->depth != nullptr;
    P.has_stencil = p->stencil != nullptr;
    P.color_format = p->fb.color_format;
    P.draw_id = draw_id;
    P.force_unsafe = p->force_unsafe ? 1u : 0u;
    uint32_t tex_f32 = 0;
    const uint32_t* tex_data = sampled_texels(d->texture, &tex_f32);
    if (d->texture) { P.tex_w = d->texture->w; P.tex_h = d->texture->h; P.tex_f32 = tex_f32; }
    P.tex_filter = d->tex_filter; P.tex_edge = d->tex_edge;
    // stencil mode (src/stencil.rs; a missing attachment behaves as `()`)
    uint32_t test = pd.stencil_test, op = pd.stencil_op;
    P.stencil_test = test; P.stencil_op = op; P.stencil_wrap = pd.stencil_wrap;
    P.sref = P.has_stencil ? (d->stencil_ref & 0xffu) : 0u;
    bool nothing = false;
    uint32_t gate = 0;
    if (!P.has_stencil) {
        nothing = !stencil_test(test, 0, 0);
    } else if (test == SR_STENCIL_NEVER) {
        nothing = true;
    } else if (op == SR_STENCIL_KEEP) {
        gate = test != SR_STENCIL_ALWAYS;
    } else if (test == SR_STENCIL_ALWAYS) {
        P.stencil_active = 1;
    } else {
        P.mode_b = 1;
        P.stencil_active = 1;
    }
    if (W < 2 || H < 2 || P.n_in == 0) nothing = true;   // no semantic tiles / no primitives
    const bool ordered = P.mode_b || d->blend != BLEND_REPLACE;
    const bool indexed = d->gs_mode == SR_GS_NONE;
    P.keep_degenerate = P.stencil_active ? 1u : 0u;
    if (ordered) { P.bin_w_log2 = 4; P.bin_h_log2 = 4; }
    else { P.bin_w_log2 = 5; P.bin_h_log2 = 5; }
    P.bins_x = (W + (1u << P.bin_w_log2) - 1) >> P.bin_w_log2;
    P.bins_y = (H + (1u << P.bin_h_log2) - 1) >> P.bin_h_log2;
    const uint32_t n_bins = P.bins_x * P.bins_y;

    // per-draw statistics start from zero; a draw that rasterises the
    // previous draw's geometry again keeps its geometry counters
    auto reset_stats = [&](bool keep_geometry) -> int {
        char* f = reinterpret_cast<char*>(p->flags);
        if (!keep_geometry) {
            SR_CK(cudaMemsetAsync(f + FLAGS_STATS_OFFSET, 0, sizeof(DeviceFlags) - FLAGS_STATS_OFFSET, st));
            return SR_OK;
        }
        const size_t a = offsetof(DeviceFlags, triangles_raster), b = offsetof(DeviceFlags, n_gen_tris);
        const size_t c = offsetof(DeviceFlags, n_unsafe_list);
        SR_CK(cudaMemsetAsync(f + a, 0, b - a, st));
        SR_CK(cudaMemsetAsync(f + c, 0, sizeof(DeviceFlags) - c, st));
        return SR_OK;
    };
    // the stage-output buffers before this draw's capacity checks (vertex
    // store first, then the geometry stage's): a reuse draw skips its
    // producer stages only if the buffers it reads did not move
    const void* const out0[6] = {p->scr4.p, p->vary.p, p->clip4.p, p->refs.p, p->lpv.p, p->lpvalid.p};
    auto outputs_kept = [&]() {
        const void* const out1[6] = {p->scr4.p, p->vary.p, p->clip4.p, p->refs.p, p->lpv.p, p->lpvalid.p};
        const size_t n = d->reuse == SR_REUSE_GEOMETRY ? 6 : 3;
        return d->reuse != SR_REUSE_NONE && p->outputs_intact && !replay &&
               std::memcmp(out0, out1, n * sizeof(void*)) == 0;
    };
    p->last_launches = 0;
    p->last_profiled = false;
    if (nothing) {
        p->outputs_intact = false;
        return reset_stats(false);
    }

    // ---- lines and points (and triangles turned into lines by a named GS)
    const bool named = d->gs_mode == SR_GS_NAMED && d->gs != GS_CLIP;
    if (d->prim != SR_PRIM_TRIANGLE || named) {
        const uint32_t prim_n = d->prim;
        const uint32_t n_in = (uint32_t)(m->n_indices / prim_n);
        const uint32_t prim_out = (named && prim_n == 3) ? 2u : prim_n;
        const uint32_t n_out = (named && prim_n == 3) ? (d->gs == GS_VERTEX_NORMALS ? 3u : 1u) * n_in : n_in;
        const bool gs = d->gs_mode != SR_GS_NONE;
        P.aa_lines = d->aa_lines ? 1u : 0u;
        int rc2;
        if ((rc2 = p->scr4.ensure(m->n_pad + 4)) || (rc2 = p->vary.ensure(((size_t)m->n_pad + 4) * VSTRIDE)) ||
            (gs && (rc2 = p->clip4.ensure(m->n_pad + 4))) ||
            (rc2 = p->lpv.ensure(4 * ((size_t)n_out * prim_out + 1))) || (rc2 = p->lpvalid.ensure((size_t)n_out + 1)))
            return rc2;
        VertexStore vs{p->clip4.p, p->scr4.p, p->vary.p, (uint32_t)p->scr4.cap};
        const bool skip_v = outputs_kept();
        const bool skip_g = skip_v && d->reuse == SR_REUSE_GEOMETRY;
        if ((rc2 = reset_stats(skip_g))) return rc2;
        p->outputs_intact = false;
        cudaEvent_t* ev = p->profiling ? p->ev : nullptr;
        if (ev) cudaEventRecord(ev[0], st);
        if (!skip_v) launch_vertex(P, pd.vU, m, vs, gs, st);
        if (ev) { cudaEventRecord(ev[1], st); }
        LPV* lv = reinterpret_cast<LPV*>(p->lpv.p);
        if (!skip_g)
            launch_lp_geometry(P, pd.gU, m, vs, prim_n, d->gs_mode, (uint32_t)d->gs, lv, p->lpvalid.p, p->flags, st);
        if (ev) { cudaEventRecord(ev[2], st); cudaEventRecord(ev[3], st); }
        const uint32_t tex_launches = 0;
        const uint32_t* tex = tex_data;
        const uint32_t ph = launch_lp_raster(P, pd.U, lv, p->lpvalid.p, n_out, prim_out, tex, p->color, p->depth,
                                             p->stencil, p->flags, st);
        if (ev) { cudaEventRecord(ev[4], st); cudaEventRecord(ev[5], st); }
        p->last_launches = (skip_v ? 0 : 1) + (skip_g ? 0 : 1) + ph + tex_launches;
        p->last_profiled = ev != nullptr;
        SR_CK(cudaGetLastError());
        p->outputs_intact = true;
        return SR_OK;
    }

    // ---- capacities
    if (!indexed) {
        if (p->gen_tri_cap < 2ull * P.n_in + 4096) p->gen_tri_cap = 2ull * P.n_in + 4096;
        if (p->gen_vert_cap < 2ull * P.n_in + 4096) p->gen_vert_cap = 2ull * P.n_in + 4096;
        if (p->gen_tri_cap > (1ull << 30)) p->gen_tri_cap = 1ull << 30;
        if (p->gen_vert_cap > (1ull << 30)) p->gen_vert_cap = 1ull << 30;
    }
    uint64_t n_raster_cap = indexed ? P.n_in : p->gen_tri_cap;
    // (bin, primitive) pairs: about two per small primitive, plus the bins of
    // large ones -- 16 per bin covers a frame overlapped a dozen times by
    // large triangles without the overflow replay (a few KB per bin)
    if (p->entry_cap < 2 * n_raster_cap + 16ull * n_bins) p->entry_cap = 2 * n_raster_cap + 16ull * n_bins;
    if (p->entry_cap > 0xffffffffull) p->entry_cap = 0xffffffffull;
    P.gen_tri_cap = (uint32_t)p->gen_tri_cap;
    P.gen_vert_cap = (uint32_t)p->gen_vert_cap;
    P.entry_cap = p->entry_cap;
    P.n_raster_host = indexed ? P.n_in : 0;
    int rc;
    uint64_t vslots = (uint64_t)m->n_pad + (indexed ? 0 : p->gen_vert_cap);
    if ((rc = p->scr4.ensure(vslots)) || (rc = p->vary.ensure(vslots * VSTRIDE))) return rc;
    if (!indexed) {
        if ((rc = p->clip4.ensure(m->n_pad)) || (rc = p->clip_counts.ensure(P.n_in)) ||
            (rc = p->clip_offsets.ensure((size_t)P.n_in + 1)) || (rc = p->clip_tmp.ensure(scan_blocks(P.n_in) + 2)) ||
            (rc = p->refs.ensure(3 * p->gen_tri_cap)))
            return rc;
    }
    if ((rc = p->setup.ensure(4 * n_raster_cap)) || (rc = p->binrect.ensure(n_raster_cap)) ||
        (rc = p->unsafe_list.ensure(n_raster_cap)) || (rc = p->unsafe_rect.ensure(n_raster_cap)))
        return rc;
    BinBuffers B{};
    if (ordered && !P.mode_b) {
        const size_t nblk = radix_blocks(p->entry_cap);
        const size_t tmp = std::max(scan_blocks(n_raster_cap + 1), scan_blocks(256 * nblk)) + 2;
        if ((rc = p->pcount.ensure(n_raster_cap + 1)) || (rc = p->poff.ensure(n_raster_cap + 1)) ||
            (rc = p->pkeys0.ensure(p->entry_cap)) || (rc = p->pkeys1.ensure(p->entry_cap)) ||
            (rc = p->pvals0.ensure(p->entry_cap)) || (rc = p->pvals1.ensure(p->entry_cap)) ||
            (rc = p->hist.ensure(256 * nblk)) || (rc = p->hist_off.ensure(256 * nblk + 1)) ||   // + the scan's total
            (rc = p->ranges.ensure(2 * (size_t)n_bins)) || (rc = p->bin_tmp.ensure(tmp)))
            return rc;
        B = BinBuffers{p->pcount.p, p->poff.p, p->bin_tmp.p, {p->pkeys0.p, p->pkeys1.p}, {p->pvals0.p, p->pvals1.p},
                       p->hist.p, p->hist_off.p, p->ranges.p, p->entry_cap};
    }
    // opaque draws: binned (sr_tiled.cu) unless SR_OPAQUE_KEYS selects the
    // global key buffer path (sr_opaque.cu)
    const bool tiled = !ordered && !p->opaque_keys;
    if (!ordered) {
        const size_t npx = (size_t)W * H;
        const size_t nblk = (size_t)((W + 31) / 32) * ((H + 31) / 32);
        const bool fresh = p->gkeys.cap < npx || p->bitmap.cap < (nblk + 31) / 32;
        if (tiled) {
            if ((rc = p->bin_counts.ensure(2 * (size_t)n_bins)) || (rc = p->bin_off.ensure(2 * (size_t)n_bins + 2)) ||
                (rc = p->entries.ensure(p->entry_cap)) || (rc = p->gkeys.ensure(npx)) ||
                (rc = p->bitmap.ensure((nblk + 31) / 32)) || (rc = p->gids.ensure((size_t)n_bins << 10)))
                return rc;
        } else if ((rc = p->area.ensure(n_raster_cap + 1)) || (rc = p->big_list.ensure(n_raster_cap + 1)) ||
                   (rc = p->gkeys.ensure(npx)) || (rc = p->bitmap.ensure((nblk + 31) / 32))) {
            return rc;
        }
        if (fresh) {   // zero once; the raster passes leave them zero
            SR_CK(cudaMemsetAsync(p->gkeys.p, 0, p->gkeys.cap * 8, st));
            SR_CK(cudaMemsetAsync(p->bitmap.p, 0, p->bitmap.cap * 4, st));
        }
        // the bin counts and slot cursors start at zero in every draw
        if (tiled) SR_CK(cudaMemsetAsync(p->bin_counts.p, 0, 2 * (size_t)n_bins * 4, st));
    }
    StencilCountArgs S{nullptr, nullptr, nullptr};
    if (P.stencil_active && !P.mode_b) {
        size_t nd = (size_t)(W + 1) * (H + 1);
        size_t nseg = (size_t)stencil_colseg_rows(H) * (W + 1);   // column-scan scratch after the array
        size_t nl = 3 * (size_t)(W + 1) + 3 * (size_t)(H + 1);
        if ((rc = p->st_diff.ensure(nd + nseg)) || (rc = p->st_lines.ensure(nl)) || (rc = p->st_glob.ensure(16)))
            return rc;
        SR_CK(cudaMemsetAsync(p->st_diff.p, 0, nd * 4, st));
        SR_CK(cudaMemsetAsync(p->st_lines.p, 0, nl * 4, st));
        SR_CK(cudaMemsetAsync(p->st_glob.p, 0, 16 * 8, st));
        S = StencilCountArgs{p->st_diff.p, p->st_lines.p, p->st_glob.p, p->st_diff.p + nd};
    }
    VertexStore vs{p->clip4.p, p->scr4.p, p->vary.p, (uint32_t)vslots};
    const bool skip_v = outputs_kept();
    const bool skip_g = skip_v && d->reuse == SR_REUSE_GEOMETRY;
    if ((rc = reset_stats(skip_g))) return rc;
    p->outputs_intact = false;

    // ---- stages, with optional events between them
    cudaEvent_t* ev = p->profiling ? p->ev : nullptr;
    if (ev) cudaEventRecord(ev[0], st);
    uint32_t launches = 0;
    if (!skip_v) {
        launch_vertex(P, pd.vU, m, vs, !indexed, st);
        launches += 1;
    }
    if (ev) cudaEventRecord(ev[1], st);
    const uint32_t* vidx = m->indices;
    if (!indexed) {
        if (!skip_g) {
            launch_clip(P, m, vs, p->clip_counts.p, p->clip_offsets.p, p->clip_tmp.p, p->refs.p, p->flags, st);
            launches += 5;
        }
        vidx = p->refs.p;
    }
    if (ev) cudaEventRecord(ev[2], st);
    launch_setup_bin(P, vidx, vs, p->setup.p, reinterpret_cast<uint32_t*>(p->binrect.p),
                     tiled ? p->bin_counts.p : nullptr, nullptr, nullptr, nullptr, nullptr, p->unsafe_list.p,
                     p->unsafe_rect.p, (ordered || tiled) ? nullptr : p->area.p, S, p->flags, st);
    launches += 1;
    const uint32_t* bin_list = nullptr;
    if (ordered && !P.mode_b) {
        bin_list = launch_bins(P, p->binrect.p, p->setup.p, p->unsafe_list.p, B, p->flags, st);
        uint32_t bits = 1;
        while ((1ull << bits) < n_bins) ++bits;
        launches += 7 + 2 * ((bits + 7) / 8) + 3;   // counts, scan, check, emits, radix passes, ranges
    }
    if (ev) cudaEventRecord(ev[3], st);
    const uint32_t* tex = tex_data;
    if (ordered) {
        launch_ordered(P, pd.U, p->setup.p, P.mode_b ? nullptr : p->ranges.p, bin_list, vidx, p->vary.p, tex, p->color,
                       p->depth, p->stencil, gate, p->flags, st);
        launches += 1;
    } else if (tiled) {
        TiledArgs T{p->setup.p, p->binrect.p, p->bin_counts.p, p->bin_counts.p + n_bins, p->bin_off.p,
                    p->bin_off.p + n_bins + 1, p->entries.p,
                    p->entry_cap, p->gkeys.p, p->bitmap.p, p->gids.p, p->unsafe_list.p, p->unsafe_rect.p, vidx,
                    p->vary.p, tex, p->color, p->depth, p->stencil, gate, p->flags};
        launches += (uint32_t)launch_tiled(P, pd.U, T, st);
    } else {
        OpaqueArgs A{p->setup.p, p->area.p, p->big_list.p, p->gkeys.p, p->bitmap.p, p->unsafe_list.p,
                     p->unsafe_rect.p, vidx, p->vary.p, tex, p->color, p->depth, p->stencil, gate, p->flags};
        launches += (uint32_t)launch_opaque(P, pd.U, A, st);
    }
    if (ev) cudaEventRecord(ev[4], st);
    if (P.stencil_active && !P.mode_b) {
        launch_stencil_apply(P, S, p->stencil, p->flags, st);
        launches += 6;
    }
    if (ev) cudaEventRecord(ev[5], st);
    p->last_launches = launches;
    p->last_profiled = ev != nullptr;
    SR_CK(cudaGetLastError());
    p->outputs_intact = true;
    return SR_OK;
}

}  // namespace

extern "C" SR_API int sr_render(sr_pipeline* p, const sr_draw* d) {
    if (!p || !d || !d->mesh) return SR_EINVAL;
    const sr_mesh* m = d->mesh;
    if (d->prim != SR_PRIM_TRIANGLE && d->prim != SR_PRIM_LINE && d->prim != SR_PRIM_POINT) return SR_EINVAL;
    if (m->n_indices % d->prim != 0) return SR_EINVAL;                     // mod.rs:148
    if (d->vs < 0 || d->vs >= VS_COUNT || d->fs < 0 || d->fs >= FS_COUNT || d->blend < 0 || d->blend >= BLEND_COUNT)
        return SR_EINVAL;
    if (d->gs_mode != SR_GS_NONE && d->gs_mode != SR_GS_CLIP && d->gs_mode != SR_GS_NAMED) return SR_EINVAL;
    if (d->gs_mode == SR_GS_NAMED && (d->gs < 0 || d->gs >= GS_COUNT)) return SR_EINVAL;
    // the normal shaders read world position and normal from varyings 0..7
    if (d->gs_mode == SR_GS_NAMED && d->gs != GS_CLIP && vs_nk(d->vs) < 8) return SR_EINVAL;
    if (d->tile_w == 0 || d->tile_h == 0 || d->tile_w > 65535 || d->tile_h > 65535) return SR_EINVAL;
    if (d->tex_filter > SR_SAMPLE_BILINEAR || d->tex_edge > SR_SAMPLE_BORDER) return SR_EINVAL;
    if (d->cull > SR_CULL_COUNTER_CLOCKWISE) return SR_EINVAL;
    if (m->n_planes < (uint32_t)vs_planes(d->vs)) return SR_EINVAL;
    if (vs_nk(d->vs) < fs_min_varyings(d->fs)) return SR_EINVAL;
    if (d->fs == FS_TEXTURED_BLINN_PHONG && !d->texture) return SR_EINVAL;
    // a texture view may not read the colour plane this draw writes
    if (d->texture && d->texture->view && d->texture->data == p->color) return SR_EINVAL;
    if (p->stencil && d->stencil_ref > 255) return SR_EINVAL;
    // duplicate(): the producing draw must be the previous one, over the same
    // mesh contents, vertex shader and viewport (and geometry stage)
    if (d->reuse > SR_REUSE_GEOMETRY) return SR_EINVAL;
    if (d->reuse != SR_REUSE_NONE) {
        const sr_draw& q = p->prev.d;
        if (!p->have_prev || q.mesh != d->mesh || p->prev.mesh_version != m->version || q.vs != d->vs ||
            std::memcmp(&q.viewport, &d->viewport, sizeof(sr_viewport)) != 0)
            return SR_EINVAL;
        if (d->reuse == SR_REUSE_VERTICES && (q.gs_mode == SR_GS_NONE || d->gs_mode == SR_GS_NONE)) return SR_EINVAL;
        if (d->reuse == SR_REUSE_GEOMETRY &&
            (q.prim != d->prim || q.gs_mode != d->gs_mode || (d->gs_mode == SR_GS_NAMED && q.gs != d->gs)))
            return SR_EINVAL;
    }
    PendingDraw pd;
    pd.d = *d;
    pd.U = p->U;
    pd.vU = d->reuse != SR_REUSE_NONE ? p->prev.vU : p->U;
    pd.gU = d->reuse == SR_REUSE_GEOMETRY ? p->prev.gU : p->U;
    pd.mesh_version = m->version;
    pd.stencil_test = p->stencil_test;
    pd.stencil_op = p->stencil_op;
    pd.stencil_wrap = p->stencil_wrap;
    uint32_t id = (uint32_t)p->pending.size();
    p->pending.push_back(pd);
    int rc = enqueue_draw(p, pd, id, false);
    if (rc != SR_OK) {
        p->pending.pop_back();
        p->outputs_intact = false;
        return rc;
    }
    // the draw may be replayed from its descriptor until the next sr_sync
    mesh_ref(pd.d.mesh);
    texture_ref(pd.d.texture);
    p->prev = pd;
    p->have_prev = true;
    return SR_OK;
}

namespace {
int enqueue_read(sr_pipeline* p, void* color, float* depth, uint8_t* stencil) {
    size_t n = (size_t)p->fb.width * p->fb.height;
    if (color && p->color) SR_CK(cudaMemcpyAsync(color, p->color, n * bytes_per_color(p->fb.color_format), cudaMemcpyDeviceToHost, p->stream));
    if (depth && p->depth) SR_CK(cudaMemcpyAsync(depth, p->depth, n * 4, cudaMemcpyDeviceToHost, p->stream));
    if (stencil && p->stencil) SR_CK(cudaMemcpyAsync(stencil, p->stencil, n, cudaMemcpyDeviceToHost, p->stream));
    return SR_OK;
}
}  // namespace

extern "C" SR_API int sr_framebuffer_read_async(sr_pipeline* p, void* color, float* depth, uint8_t* stencil) {
    if (!p) return SR_EINVAL;
    const int rc = enqueue_read(p, color, depth, stencil);
    if (rc == SR_OK && !p->pending.empty()) {   // repeated in sequence if sync replays the draws
        PendingDraw pr{};
        pr.kind = PENDING_READ;
        pr.read_color = color;
        pr.read_depth = depth;
        pr.read_stencil = stencil;
        p->pending.push_back(pr);
    }
    return rc;
}

extern "C" SR_API int sr_sync(sr_pipeline* p) {
    if (!p) return SR_EINVAL;
    int status = SR_OK;
    bool settled = false;   // the flags read clean after the last enqueue or replay
    for (int attempt = 0; attempt < 8; ++attempt) {
        SR_CK(cudaMemcpyAsync(p->hflags, p->flags, sizeof(DeviceFlags), cudaMemcpyDeviceToHost, p->stream));
        cudaError_t e = cudaStreamSynchronize(p->stream);
        if (e != cudaSuccess) { last_cuda_error() = e; return SR_ECUDA; }
        DeviceFlags f = *p->hflags;
        if (!f.poison) {
            settled = true;
            if (p->pending.empty()) break;
            std::memset(&p->last_stats, 0, sizeof(p->last_stats));
            p->last_stats.triangles_generated = f.triangles_generated;
            p->last_stats.triangles_raster = f.triangles_raster;
            p->last_stats.unsafe_triangles = f.unsafe;
            p->last_stats.bin_entries = f.entries;
            p->last_stats.fragments = f.fragments;
            p->last_stats.nan_bbox = f.nan_bbox;
            p->last_stats.overflow = f.overflow_bits;
            const PendingDraw* last = nullptr;   // the last draw (clears may follow it)
            for (auto it = p->pending.rbegin(); it != p->pending.rend() && !last; ++it)
                if (it->kind == PENDING_DRAW) last = &*it;
            const sr_mesh* m = last ? last->d.mesh : nullptr;
            p->last_stats.triangles_in = m ? m->n_indices / std::max(1u, last->d.prim) : 0;
            p->last_stats.kernel_launches = p->last_launches;
            if (p->last_profiled) {
                p->last_stats.profiled = 1;
                for (int k = 0; k < 5; ++k) cudaEventElapsedTime(&p->last_stats.stage_ms[k], p->ev[k], p->ev[k + 1]);
                cudaEventElapsedTime(&p->last_stats.stage_ms[5], p->ev[0], p->ev[5]);
            }
            if (f.nan_total) status = SR_ENAN;
            if (f.bad_index) status = SR_EINVAL;
            if (f.copy_timeout) status = SR_ECUDA;
            break;
        }
        // grow what overflowed and replay from the first poisoned draw
        if (f.overflow_bits & OVF_GEN_TRIS) p->gen_tri_cap = f.need_gen_tris + f.need_gen_tris / 4 + 1024;
        if (f.overflow_bits & OVF_GEN_VERTS) p->gen_vert_cap = f.need_gen_verts + f.need_gen_verts / 4 + 1024;
        if (f.overflow_bits & OVF_ENTRIES) p->entry_cap = f.need_entries + f.need_entries / 4 + 1024;
        if (f.overflow_bits & OVF_SORT) { status = SR_EOVERFLOW; }
        // the capacities are clamped when a draw is enqueued (2^30 generated
        // triangles and vertices, 2^32 - 1 bin entries): a draw needing more
        // overflows again on every replay
        if (f.need_gen_tris > (1ull << 30) || f.need_gen_verts > (1ull << 30) || f.need_entries > 0xffffffffull)
            status = SR_EOVERFLOW;
        uint32_t from = f.poison_draw;
        DeviceFlags z;
        std::memset(&z, 0, sizeof(z));
        z.poison_draw = 0xffffffffu;
        z.nan_total = f.nan_total;
        SR_CK(cudaMemcpyAsync(p->flags, &z, sizeof(z), cudaMemcpyHostToDevice, p->stream));
        SR_CK(cudaStreamSynchronize(p->stream));
        if (status == SR_EOVERFLOW || from >= p->pending.size()) break;
        for (uint32_t i = from; i < p->pending.size(); ++i) {
            const PendingDraw& e = p->pending[i];
            int rc = SR_OK;
            switch (e.kind) {
            case PENDING_CLEAR: rc = enqueue_clear(p, e.clear_color); break;
            case PENDING_READ: rc = enqueue_read(p, e.read_color, e.read_depth, e.read_stencil); break;
            case PENDING_TEXTURE_COPY: rc = enqueue_texture_copy(p, e.d.texture); break;
            default: rc = enqueue_draw(p, e, i, true); break;
            }
            if (rc != SR_OK) { status = rc; break; }
        }
        if (status != SR_OK) break;
    }
    // out of attempts with the last replay unchecked, or poisoned without a draw
    // to replay: the frame is incomplete
    if (!settled && status == SR_OK) status = SR_EOVERFLOW;
    for (const auto& pd : p->pending) {
        mesh_unref(pd.d.mesh);
        texture_unref(pd.d.texture);
    }
    p->pending.clear();
    if (status == SR_OK) status = p->deferred_status;
    p->deferred_status = SR_OK;
    DeviceFlags z;
    std::memset(&z, 0, sizeof(z));
    z.poison_draw = 0xffffffffu;
    SR_CK(cudaMemcpyAsync(p->flags, &z, sizeof(z), cudaMemcpyHostToDevice, p->stream));
    SR_CK(cudaStreamSynchronize(p->stream));
    return status;
}

extern "C" SR_API int sr_get_stats(sr_pipeline* p, sr_stats* out) {
    if (!p || !out) return SR_EINVAL;
    *out = p->last_stats;
    return SR_OK;
}
