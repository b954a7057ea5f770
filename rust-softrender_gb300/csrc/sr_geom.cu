// sr_geom.cu — vertex stage and the clipping geometry shader.
//
//   vertex_kernel  VertexShader::run / run_to_fragment (stages/vertex.rs:87-160):
//                  out[v] = vs(vertex v); screen = ClipVertex::normalize
//                  (geometry/clipvertex.rs:89-127).  One thread per vertex:
//                  a warp reads 32 consecutive floats of each attribute plane
//                  (one 128-byte transaction per plane), and writes its
//                  vertices' screen positions and varyings contiguously.
//   clip_*_kernel  GeometryShader::clip_primitives, triangle arm
//                  (stages/geometry.rs:264-299) + finish (geometry.rs:60-129):
//                  a counting pass, an exclusive scan (order-preserving
//                  compaction), and an emit pass writing the generated
//                  vertices (normalised) and the output triangles in input
//                  order, exactly as the single-threaded reference orders them.
#include "sr_internal.cuh"
#include "sr_scan.cuh"
#include "sr_vertex.cuh"

namespace sr {

// ------------------------------------------------------------ vertex stage
template <int VS>
__global__ void __launch_bounds__(128) vertex_kernel(uint32_t n_verts, uint32_t n_pad, sr_uniforms U, VpMatrix vpm,
                                                     const float* __restrict__ planes, float4* __restrict__ clip4,
                                                     float4* __restrict__ scr4, float* __restrict__ vary) {
    vertex_one<VS>(blockIdx.x * blockDim.x + threadIdx.x, n_verts, n_pad, U, vpm, planes, clip4, scr4, vary);
}

void launch_vertex(const DrawParams& P, const sr_uniforms& U, const sr_mesh* m, VertexStore vs,
                   bool write_clip, cudaStream_t st) {
    if (m->n_verts == 0) return;
    dim3 grid((m->n_verts + 127) / 128), block(128);
    VpMatrix vpm = viewport_matrix(P.vp);
    float4* c4 = write_clip ? vs.clip4 : nullptr;
    switch (P.vs) {
    case VS_MVP_POS_NRM:
        vertex_kernel<VS_MVP_POS_NRM><<<grid, block, 0, st>>>(m->n_verts, m->n_pad, U, vpm, m->planes, c4, vs.scr4, vs.vary);
        break;
    case VS_MVP_POS_NRM_UV:
        vertex_kernel<VS_MVP_POS_NRM_UV><<<grid, block, 0, st>>>(m->n_verts, m->n_pad, U, vpm, m->planes, c4, vs.scr4, vs.vary);
        break;
    case VS_CLIP_COLOR:
        vertex_kernel<VS_CLIP_COLOR><<<grid, block, 0, st>>>(m->n_verts, m->n_pad, U, vpm, m->planes, c4, vs.scr4, vs.vary);
        break;
    default:
        vertex_kernel<VS_CLIP_RGBA8><<<grid, block, 0, st>>>(m->n_verts, m->n_pad, U, vpm, m->planes, c4, vs.scr4, vs.vary);
        break;
    }
}

// ------------------------------------------------------- clipping (GS)
// Polygon entries: a vertex of the input triangle (0, 1, 2) or an
// intersection 0x80 | edge << 3 | plane.
struct Poly {
    uint8_t e[36];
    int n;
};

// ClippingPlane::has_inside (geometry/clip.rs:33-44), Left..Far
__device__ __forceinline__ uint32_t inside_mask(float4 c) {
    uint32_t m = 0;
    m |= (c.x >= -c.w) ? 1u : 0u;
    m |= (c.x <= c.w) ? 2u : 0u;
    m |= (c.y >= -c.w) ? 4u : 0u;
    m |= (c.y <= c.w) ? 8u : 0u;
    m |= (c.z >= 0.0f) ? 16u : 0u;
    m |= (c.z <= c.w) ? 32u : 0u;
    return m;
}

// The push loop of clip_primitives (geometry.rs:270-284).
__device__ __forceinline__ void build_poly(const uint32_t mk[3], Poly& P) {
    int n = 0;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        int s = e, p = e == 2 ? 0 : e + 1;
#pragma unroll
        for (int plane = 0; plane < 6; ++plane) {
            bool s_in = (mk[s] >> plane) & 1u;
            bool p_in = (mk[p] >> plane) & 1u;
            if (s_in != p_in) P.e[n++] = (uint8_t)(0x80 | (e << 3) | plane);
            if (p_in) P.e[n++] = (uint8_t)p;
        }
    }
    P.n = n;
}

__device__ __forceinline__ bool same_vertex(const Poly& P, int i, int j) {
    if (i == j) return true;
    uint8_t a = P.e[i], b = P.e[j];
    return !(a & 0x80) && a == b;
}

// Output triangle k of the polygon (geometry.rs:286-297): len == 3 keeps
// (p0, p1, p2); len > 3 fans (last, p_i, p_i+1).
__device__ __forceinline__ void out_tri(const Poly& P, int k, int& i0, int& i1, int& i2) {
    if (P.n == 3) { i0 = 0; i1 = 1; i2 = 2; }
    else { i0 = P.n - 1; i1 = k; i2 = k + 1; }
}

__device__ __forceinline__ int n_out_tris(const Poly& P) { return P.n == 3 ? 1 : (P.n > 3 ? P.n - 2 : 0); }

// A triangle inside every plane (all inside masks 0x3f): the push loop yields
// the polygon b x6, c x6, a x6 and its fan from the last entry (a) the 16
// triangles (a, P[k], P[k+1]); only k = 5, (a, b, c), is not degenerate.
constexpr uint32_t ALL_INSIDE = 0x3fu;
constexpr int INSIDE_OUT_TRIS = 16;
__device__ __forceinline__ int inside_poly_vertex(int j) { return j < 6 ? 1 : (j < 12 ? 2 : 0); }

__device__ __forceinline__ bool out_tri_degenerate(const Poly& P, int k) {
    int i0, i1, i2;
    out_tri(P, k, i0, i1, i2);
    return same_vertex(P, i0, i1) || same_vertex(P, i1, i2) || same_vertex(P, i0, i2);
}

__global__ void __launch_bounds__(256) clip_count_kernel(uint32_t n_in, uint32_t n_verts, uint32_t keep_degenerate,
                                                         const uint32_t* __restrict__ idx,
                                                         const float4* __restrict__ clip4,
                                                         unsigned long long* __restrict__ counts,
                                                         DeviceFlags* flags) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long gen = 0;
    if (t < n_in) {
        uint32_t i0 = __ldg(idx + 3 * t), i1 = __ldg(idx + 3 * t + 1), i2 = __ldg(idx + 3 * t + 2);
        if (i0 >= n_verts || i1 >= n_verts || i2 >= n_verts) {
            counts[t] = 0;
            atomicOr(&flags->bad_index, 1u);
            t = n_in;   // contributes nothing
        }
    }
    if (t < n_in) {
        uint32_t mk[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) mk[j] = inside_mask(__ldg(clip4 + __ldg(idx + 3 * t + j)));
        if ((mk[0] & mk[1] & mk[2]) == ALL_INSIDE) {
            counts[t] = keep_degenerate ? (unsigned long long)INSIDE_OUT_TRIS : 1ull;
            gen = INSIDE_OUT_TRIS;
        } else {
            Poly P;
            build_poly(mk, P);
            int nv = 0;
            for (int i = 0; i < P.n; ++i) nv += (P.e[i] & 0x80) ? 1 : 0;
            int no = n_out_tris(P);
            int kept = 0;
            for (int k = 0; k < no; ++k) kept += (keep_degenerate || !out_tri_degenerate(P, k)) ? 1 : 0;
            counts[t] = ((unsigned long long)nv << 32) | (unsigned long long)kept;
            gen = (unsigned long long)no;
        }
    }
    // block-reduce the number of generated primitives for the statistics
    __shared__ unsigned long long s_gen;
    if (threadIdx.x == 0) s_gen = 0;
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) gen += __shfl_down_sync(0xffffffffu, gen, o);
    if ((threadIdx.x & 31) == 0 && gen) atomicAdd(&s_gen, gen);
    __syncthreads();
    if (threadIdx.x == 0 && s_gen) atomicAdd(&flags->triangles_generated, s_gen);
}

// ClippingPlane::intersect (geometry/clip.rs:46-63) on position and varyings,
// then ClipVertex::normalize of finish().
__device__ __forceinline__ float lerp1(float t, float x1, float x2) { return (1.0f - t) * x1 + t * x2; }

__global__ void __launch_bounds__(256) clip_emit_kernel(uint32_t n_in, uint32_t n_verts, uint32_t keep_degenerate,
                                                        uint32_t draw_id, int nkq,
                                                        VpMatrix vpm,
                                                        uint32_t gen_base, uint32_t gen_tri_cap,
                                                        uint32_t gen_vert_cap,
                                                        const uint32_t* __restrict__ idx,
                                                        const float4* __restrict__ clip4,
                                                        float4* __restrict__ scr4, float* __restrict__ vary,
                                                        const unsigned long long* __restrict__ offsets,
                                                        uint32_t* __restrict__ refs, DeviceFlags* flags) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        unsigned long long tot = offsets[n_in];
        unsigned long long tv = tot >> 32, tt = tot & 0xffffffffull;
        flags->n_gen_tris = tt;
        flags->n_gen_verts = tv;
        if (tt > gen_tri_cap) { atomicOr(&flags->overflow_bits, (unsigned)OVF_GEN_TRIS); atomicOr(&flags->poison, 1u); atomicMin(&flags->poison_draw, draw_id); }
        if (tv > gen_vert_cap) { atomicOr(&flags->overflow_bits, (unsigned)OVF_GEN_VERTS); atomicOr(&flags->poison, 1u); atomicMin(&flags->poison_draw, draw_id); }
        if (tt > flags->need_gen_tris) flags->need_gen_tris = tt;
        if (tv > flags->need_gen_verts) flags->need_gen_verts = tv;
    }
    if (t >= n_in) return;
    unsigned long long off = offsets[t];
    uint32_t voff = (uint32_t)(off >> 32), toff = (uint32_t)(off & 0xffffffffull);
    uint32_t vi[3];
    float4 c[3];
    uint32_t mk[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) vi[j] = __ldg(idx + 3 * t + j);
    if (vi[0] >= n_verts || vi[1] >= n_verts || vi[2] >= n_verts) return;   // flagged in the count pass
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        c[j] = __ldg(clip4 + vi[j]);
        mk[j] = inside_mask(c[j]);
    }
    if ((mk[0] & mk[1] & mk[2]) == ALL_INSIDE) {   // no intersections; see inside_poly_vertex
        if (!keep_degenerate) {
            if (toff < gen_tri_cap) {
                refs[3 * (size_t)toff + 0] = vi[0];
                refs[3 * (size_t)toff + 1] = vi[1];
                refs[3 * (size_t)toff + 2] = vi[2];
            }
            return;
        }
        for (int k = 0; k < INSIDE_OUT_TRIS; ++k) {
            const uint32_t o = toff + (uint32_t)k;
            if (o >= gen_tri_cap) break;
            refs[3 * (size_t)o + 0] = vi[0];
            refs[3 * (size_t)o + 1] = vi[inside_poly_vertex(k)];
            refs[3 * (size_t)o + 2] = vi[inside_poly_vertex(k + 1)];
        }
        return;
    }
    Poly P;
    build_poly(mk, P);
    int no = n_out_tris(P);
    if (no == 0) return;
    // slots of the polygon entries: input vertices keep their mesh slot,
    // intersections become generated vertices in push order
    uint32_t slot[36];
    uint32_t j = 0;
    for (int i = 0; i < P.n; ++i) {
        uint8_t e = P.e[i];
        if (!(e & 0x80)) { slot[i] = vi[e]; continue; }
        uint32_t g = voff + j++;
        slot[i] = gen_base + g;
        if (g >= gen_vert_cap) continue;
        int edge = (e >> 3) & 3, plane = e & 7;
        int si = edge, pi = edge == 2 ? 0 : edge + 1;
        float4 a4 = c[si], b4 = c[pi];
        float a, b;
        switch (plane) {
        case 0: a = a4.w + a4.x; b = b4.w + b4.x; break;
        case 1: a = a4.w - a4.x; b = b4.w - b4.x; break;
        case 2: a = a4.w + a4.y; b = b4.w + b4.y; break;
        case 3: a = a4.w - a4.y; b = b4.w - b4.y; break;
        case 4: a = a4.z; b = b4.z; break;
        default: a = a4.w - a4.z; b = b4.w - b4.z; break;
        }
        float tt = a / (a - b);
        sr_v4 pc = sr_make_v4(lerp1(tt, a4.x, b4.x), lerp1(tt, a4.y, b4.y), lerp1(tt, a4.z, b4.z), lerp1(tt, a4.w, b4.w));
        sr_v4 s = normalize_pos(pc, vpm.m);
        scr4[gen_base + g] = make_float4(s.x, s.y, s.z, s.w);
        const float4* ka = reinterpret_cast<const float4*>(vary + (size_t)vi[si] * VSTRIDE);
        const float4* kb = reinterpret_cast<const float4*>(vary + (size_t)vi[pi] * VSTRIDE);
        float4* ko = reinterpret_cast<float4*>(vary + (size_t)(gen_base + g) * VSTRIDE);
#pragma unroll
        for (int q = 0; q < nkq; ++q) {   // the vertex shader's varyings
            float4 x = ka[q], y = kb[q];
            ko[q] = make_float4(lerp1(tt, x.x, y.x), lerp1(tt, x.y, y.y), lerp1(tt, x.z, y.z), lerp1(tt, x.w, y.w));
        }
    }
    uint32_t o = toff;
    for (int k = 0; k < no; ++k) {
        if (!keep_degenerate && out_tri_degenerate(P, k)) continue;
        if (o < gen_tri_cap) {
            int i0, i1, i2;
            out_tri(P, k, i0, i1, i2);
            refs[3 * (size_t)o + 0] = slot[i0];
            refs[3 * (size_t)o + 1] = slot[i1];
            refs[3 * (size_t)o + 2] = slot[i2];
        }
        ++o;
    }
}

void launch_clip(const DrawParams& P, const sr_mesh* m, VertexStore vs, unsigned long long* counts,
                 unsigned long long* offsets, unsigned long long* scan_tmp, uint32_t* refs,
                 DeviceFlags* flags, cudaStream_t st) {
    uint32_t n = P.n_in;
    dim3 block(256), grid((n + 255) / 256 ? (n + 255) / 256 : 1);
    clip_count_kernel<<<grid, block, 0, st>>>(n, P.n_verts, P.keep_degenerate, m->indices, vs.clip4, counts, flags);
    exclusive_scan<unsigned long long>(counts, n, offsets, scan_tmp, st);
    VpMatrix vpm = viewport_matrix(P.vp);
    clip_emit_kernel<<<grid, block, 0, st>>>(n, P.n_verts, P.keep_degenerate, P.draw_id, (vs_nk(P.vs) + 3) / 4, vpm,
                                             P.gen_base, P.gen_tri_cap, P.gen_vert_cap,
                                             m->indices, vs.clip4, vs.scr4, vs.vary, offsets, refs, flags);
}

}  // namespace sr
