// sr_host.h — host-side internals shared by the C ABI translation units:
// the pipeline object, grow-only device buffers and CUDA error plumbing.
#pragma once
#include <cstring>
#include <vector>

#include "sr_internal.cuh"

namespace sr {

// Last CUDA runtime error seen by this thread (kept for diagnostics).
inline cudaError_t& last_cuda_error() {
    static thread_local cudaError_t e = cudaSuccess;
    return e;
}

// Grow-only device buffer (capacity in elements).
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    int ensure(size_t n) {
        if (n <= cap) return SR_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = n + n / 4 + 64;
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e != cudaSuccess) { last_cuda_error() = e; p = nullptr; return SR_ENOMEM; }
        cap = want;
        return SR_OK;
    }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
};

// What a pending entry is: a draw, or an operation on the framebuffer ordered
// between draws, which a replay (sr_sync after an overflow) repeats in
// sequence.
enum PendingKind : uint32_t { PENDING_DRAW = 0, PENDING_CLEAR = 1, PENDING_READ = 2, PENDING_TEXTURE_COPY = 3 };

struct PendingDraw {
    sr_draw d;
    sr_uniforms U;              // the fragment stage's uniforms
    sr_uniforms vU, gU;         // the vertex and geometry stages' (earlier ones under sr_draw.reuse)
    uint64_t mesh_version;      // of the mesh the vertex outputs derive from
    uint32_t stencil_test, stencil_op, stencil_wrap;
    uint32_t kind = PENDING_DRAW;
    uint8_t clear_color[16] = {};       // PENDING_CLEAR
    void* read_color = nullptr;         // PENDING_READ: host destinations
    float* read_depth = nullptr;
    uint8_t* read_stencil = nullptr;    // (PENDING_TEXTURE_COPY: the texture is d.texture)
};

}  // namespace sr

#define SR_CK(x)                                                        \
    do {                                                                \
        cudaError_t e_ = (x);                                           \
        if (e_ != cudaSuccess) {                                        \
            sr::last_cuda_error() = e_;                                 \
            return e_ == cudaErrorMemoryAllocation ? SR_ENOMEM : SR_ECUDA; \
        }                                                               \
    } while (0)

// The pipeline object behind the opaque sr_pipeline handle.
struct sr_pipeline {
    sr_fb_desc fb;
    size_t cap_px = 0;          // pixels the colour/depth/stencil planes were allocated for
    void* color = nullptr;                  // color_plane->data
    sr_color_plane* color_plane = nullptr;  // referenced by the pipeline and its texture views
    float* depth = nullptr;
    uint8_t* stencil = nullptr;
    sr_uniforms U;
    uint32_t stencil_test = SR_STENCIL_ALWAYS, stencil_op = SR_STENCIL_KEEP, stencil_wrap = 1;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    sr::DeviceFlags* flags = nullptr;     // device
    sr::DeviceFlags* hflags = nullptr;    // pinned host mirror
    // workspace
    sr::DevBuf<float4> clip4, scr4;
    sr::DevBuf<float> vary;
    sr::DevBuf<unsigned long long> clip_counts, clip_offsets, clip_tmp;
    sr::DevBuf<uint32_t> refs;
    sr::DevBuf<float4> setup, unsafe_rect;
    sr::DevBuf<uint2> binrect;
    sr::DevBuf<uint32_t> bin_counts, bin_off, bin_cursor, bin_tmp, entries, unsafe_list;
    sr::DevBuf<unsigned long long> area, gkeys;
    sr::DevBuf<uint32_t> big_list, gids;
    sr::DevBuf<uint32_t> bitmap;
    sr::DevBuf<int> st_diff, st_lines;
    sr::DevBuf<uint32_t> pcount, poff, pkeys0, pkeys1, pvals0, pvals1, hist, hist_off, ranges;   // ordered bins
    sr::DevBuf<float4> lpv;           // line / point vertices (4 x float4 each)
    sr::DevBuf<uint8_t> lpvalid;      // per line / point: kept by the geometry stage
    sr::DevBuf<unsigned long long> st_glob;
    // capacities (elements) requested for the generated geometry
    uint64_t gen_tri_cap = 0, gen_vert_cap = 0, entry_cap = 0;
    std::vector<sr::PendingDraw> pending;     // draws (and clears between them) since the last sync
    int deferred_status = SR_OK;              // a status of draws synced early, for the next sr_sync
    // the previous sr_render (what sr_draw.reuse refers to), and whether the
    // stage-output buffers (vertex store, generated geometry, line/point
    // vertices) still hold its outputs
    sr::PendingDraw prev;
    bool have_prev = false;
    bool outputs_intact = false;
    sr_stats last_stats;
    bool stats_valid = false;
    bool force_unsafe = false;   // SR_FORCE_UNSAFE=1: every primitive takes the exact unsafe path
    bool opaque_keys = false;    // SR_OPAQUE_KEYS=1: opaque draws through the global key buffer (sr_opaque.cu)
    bool profiling = false;
    cudaEvent_t ev[6] = {};
    uint32_t last_launches = 0;
    bool last_profiled = false;
};

namespace sr {
// References to meshes and textures held by work that may still read them;
// the release of the last one frees the object (see sr_mesh).
inline void mesh_ref(const sr_mesh* m) {
    if (m) const_cast<sr_mesh*>(m)->refs.fetch_add(1, std::memory_order_relaxed);
}
inline void texture_ref(const sr_texture* t) {
    if (t) const_cast<sr_texture*>(t)->refs.fetch_add(1, std::memory_order_relaxed);
}
void mesh_unref(const sr_mesh* m);
void texture_unref(const sr_texture* t);
// Releases one reference on a colour plane; the last frees its memory.
inline void color_plane_unref(sr_color_plane* c) {
    if (!c || c->refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
    if (c->data) cudaFree(c->data);
    delete c;
}
// Target-independent eligibility of a draw for sr_batch_render (SR_OK or
// SR_EINVAL), shared with the server's submission checks.
int batch_draw_check(const sr_draw* d);
// Creates a pipeline whose planes hold cap_px pixels (>= width * height), so
// that pipeline_retarget can later give it any frame of at most cap_px pixels.
int pipeline_create_cap(const sr_fb_desc* fb, size_t cap_px, sr_pipeline** out);
// Changes the frame size of an idle pipeline within its capacity (the planes'
// contents become undefined: clear before drawing).
int pipeline_retarget(sr_pipeline* p, uint32_t width, uint32_t height);
}  // namespace sr
