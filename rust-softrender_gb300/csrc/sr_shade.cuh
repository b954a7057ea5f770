// sr_shade.cuh — the fragment closures compiled into the library and the
// barycentric interpolation of their varyings (interpolate.rs:43-52).
#pragma once
#include "sr_internal.cuh"

namespace sr {

template <int FS>
struct FsTraits { static constexpr int NK = 8; };
template <> struct FsTraits<FS_TEXTURED_BLINN_PHONG> { static constexpr int NK = 10; };
template <> struct FsTraits<FS_VERTEX_COLOR> { static constexpr int NK = 4; };
template <> struct FsTraits<FS_CONSTANT_COLOR> { static constexpr int NK = 0; };

// The fragment closures compiled into the library (RGBA f32 result).
template <int FS>
__device__ __forceinline__ sr_v4 shade_fs(const sr_uniforms& U, const float* k, const uint32_t* tex, const DrawParams& P) {
    if (FS == FS_BLINN_PHONG_DIR)
        return sr_blinn_phong(&U, sr_make_v4(k[0], k[1], k[2], k[3]), sr_make_v4(k[4], k[5], k[6], k[7]),
                              sr_make_v4(U.color[0], U.color[1], U.color[2], U.color[3]));
    if (FS == FS_TEXTURED_BLINN_PHONG) {
        sr_v4 t = sr_sample(tex, P.tex_f32, P.tex_w, P.tex_h, k[8], k[9], (int)P.tex_filter, (int)P.tex_edge);
        t = sr_decode_gamma(t, U.gamma);
        return sr_blinn_phong(&U, sr_make_v4(k[0], k[1], k[2], k[3]), sr_make_v4(k[4], k[5], k[6], k[7]), t);
    }
    if (FS == FS_VERTEX_COLOR) return sr_make_v4(k[0], k[1], k[2], k[3]);
    if (FS == FS_ACES_LIGHTS)
        return sr_aces_lights(&U, sr_make_v4(k[0], k[1], k[2], k[3]), sr_make_v4(k[4], k[5], k[6], k[7]));
    return sr_make_v4(U.color[0], U.color[1], U.color[2], U.color[3]);
}

// The RGBA8 word of the fragment closure's colour, equal to
// sr_to_rgba8(shade_fs<FS>(...)) for every input: the Blinn-Phong shaders
// take the bounded-error fast path of sr_shaders.h, which repeats the exact
// computation for the pixels its bound does not decide.
template <int FS>
__device__ __forceinline__ uint32_t shade_fs_rgba8(const sr_uniforms& U, const float* k, const uint32_t* tex,
                                                   const DrawParams& P) {
    if (FS == FS_BLINN_PHONG_DIR)
        return sr_blinn_phong_rgba8(&U, sr_make_v4(k[0], k[1], k[2], k[3]), sr_make_v4(k[4], k[5], k[6], k[7]),
                                    sr_make_v4(U.color[0], U.color[1], U.color[2], U.color[3]));
    if (FS == FS_TEXTURED_BLINN_PHONG) {
        const sr_v4 t = sr_sample(tex, P.tex_f32, P.tex_w, P.tex_h, k[8], k[9], (int)P.tex_filter, (int)P.tex_edge);
        return sr_textured_blinn_phong_rgba8(&U, sr_make_v4(k[0], k[1], k[2], k[3]),
                                             sr_make_v4(k[4], k[5], k[6], k[7]), t);
    }
    return sr_to_rgba8(shade_fs<FS>(U, k, tex, P));
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


}  // namespace sr
