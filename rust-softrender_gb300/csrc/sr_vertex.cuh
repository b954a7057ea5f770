// sr_vertex.cuh — vertex-stage device code shared by the per-draw and the
// batched kernels: VertexShader::run / run_to_fragment (stages/vertex.rs:87-160)
// and ClipVertex::normalize (geometry/clipvertex.rs:89-127).
#pragma once
#include "sr_internal.cuh"

namespace sr {

struct VpMatrix { float m[16]; };

__device__ __forceinline__ sr_v4 normalize_pos(sr_v4 c, const float* vpm) {
    sr_v4 s = sr_m4_mul_v4(vpm, sr_make_v4(c.x / c.w, c.y / c.w, c.z / c.w, 1.0f));
    s.w = 1.0f / c.w;
    return s;
}

template <int VS>
__device__ __forceinline__ sr_v4 run_vs(const sr_uniforms* U, const float* a, float* k) {
    if (VS == VS_MVP_POS_NRM) return sr_vs_mvp_pos_nrm(U, a, k);
    if (VS == VS_MVP_POS_NRM_UV) return sr_vs_mvp_pos_nrm_uv(U, a, k);
    if (VS == VS_CLIP_COLOR) return sr_vs_clip_color(U, a, k);
    return sr_vs_clip_rgba8(U, a, k);
}

// One thread's work of the vertex stage: vertex v, shaded, normalised and
// written to the store.  Consecutive threads take consecutive vertices, so
// the plane loads and the position / varying stores are contiguous per warp.
template <int VS>
__device__ __forceinline__ void vertex_one(uint32_t v, uint32_t n_verts, uint32_t n_pad, const sr_uniforms& U,
                                           const VpMatrix& vpm, const float* __restrict__ planes,
                                           float4* __restrict__ clip4, float4* __restrict__ scr4,
                                           float* __restrict__ vary) {
    constexpr int NP = VS == VS_MVP_POS_NRM ? 6 : VS == VS_CLIP_RGBA8 ? 4 : 8;
    if (v >= n_verts) return;
    float a[8];
#pragma unroll
    for (int j = 0; j < NP; ++j) a[j] = __ldg(planes + (size_t)j * n_pad + v);
    float k[VSTRIDE];
#pragma unroll
    for (int i = 0; i < VSTRIDE; ++i) k[i] = 0.0f;
    sr_v4 c = run_vs<VS>(&U, a, k);
    if (clip4) clip4[v] = make_float4(c.x, c.y, c.z, c.w);
    sr_v4 s = normalize_pos(c, vpm.m);
    scr4[v] = make_float4(s.x, s.y, s.z, s.w);
    // only the shader's varyings are written (readers never go beyond them:
    // each fragment shader's are validated against the vertex shader's)
    constexpr int NKQ = (vs_nk(VS) + 3) / 4;
    float4* vo = reinterpret_cast<float4*>(vary + (size_t)v * VSTRIDE);
    vo[0] = make_float4(k[0], k[1], k[2], k[3]);
    if (NKQ > 1) vo[1] = make_float4(k[4], k[5], k[6], k[7]);
    if (NKQ > 2) vo[2] = make_float4(k[8], k[9], k[10], k[11]);
}

inline VpMatrix viewport_matrix(const float* vp) {
    // the matrix of ClipVertex::normalize, built with the same f32 operations
    float left = vp[0], bottom = vp[1], width = vp[2], height = vp[3], nr = vp[4], fr = vp[5];
    float right = left + width;
    float top = bottom + height;
    VpMatrix M = {{(right - left) / 2.0f, 0.0f, 0.0f, (right + left) / 2.0f,
                   0.0f, (top - bottom) / -2.0f, 0.0f, (top + bottom) / 2.0f,
                   0.0f, 0.0f, (fr - nr) / -2.0f, (fr + nr) / -2.0f,
                   0.0f, 0.0f, 0.0f, 1.0f}};
    return M;
}


}  // namespace sr
