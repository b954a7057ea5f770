// sr_setup.cuh — per-primitive setup helpers shared by the per-draw and the
// batched setup kernels (stages/rasterization/triangle.rs:48-78).
#pragma once
#include "sr_internal.cuh"

namespace sr {

__device__ __forceinline__ void tri_slots(uint32_t t, const uint32_t* __restrict__ vidx, uint32_t& a, uint32_t& b,
                                          uint32_t& c) {
    a = __ldg(vidx + 3 * (size_t)t);
    b = __ldg(vidx + 3 * (size_t)t + 1);
    c = __ldg(vidx + 3 * (size_t)t + 2);
}

// Conservative bound of the pixel centres whose computed coverage
// !(u<0 || v<0 || w<0) can hold (the inflated triangle of sr_setup.cu): true when no pixel centre
// outside the integer bbox [ix0, ix1] x [iy0, iy1] can be covered.
__device__ __forceinline__ bool inflated_region(float x1, float y1, float x2, float y2, float x3, float y3, float det,
                                uint32_t W, uint32_t H, int ix0, int iy0, int ix1, int iy1) {
    const float BIG = 1.0e6f;
    if (!(fabsf(x1) < BIG && fabsf(x2) < BIG && fabsf(x3) < BIG && fabsf(y1) < BIG && fabsf(y2) < BIG &&
          fabsf(y3) < BIG))
        return false;
    float a = y2 - y3, b = x3 - x2, c = y3 - y1, d = x1 - x3;
    float Rx = fmaxf(fabsf(0.5f - x3), fabsf((float)W - x3));
    float Ry = fmaxf(fabsf(0.5f - y3), fabsf((float)H - y3));
    // g >= 2 * gamma_4 (gamma_4 = 4u/(1-4u), u = 2^-24): absolute rounding of
    // the two-product numerators and the determinant, with slack for the
    // float evaluation of these bounds themselves
    const float g = 5.0e-7f;
    const float eps = 6.0e-8f;
    float Su = fabsf(a) * Rx + fabsf(b) * Ry;
    float Sv = fabsf(c) * Rx + fabsf(d) * Ry;
    float SD = fabsf(a * d) + fabsf(b * c);
    float absD = fabsf(det);
    float Dlo = absD - g * SD * 2.0f;
    if (!(Dlo > 1.0e-20f) || !(absD > 4.0f * g * SD)) return false;
    float tu = (g * Su + 1.0e-30f) / Dlo;
    float tv = (g * Sv + 1.0e-30f) / Dlo;
    float tw = 2.0f * (g * SD / Dlo + (g * (Su + Sv)) / Dlo + 16.0f * eps);
    if (!(tu < 1.0f && tv < 1.0f && tw < 1.0f)) return false;
    // vertices of {l_u >= -tu, l_v >= -tv, l_w >= -tw}
    float v1x = x1 + tv * (x1 - x2) + tw * (x1 - x3), v1y = y1 + tv * (y1 - y2) + tw * (y1 - y3);
    float v2x = x2 + tu * (x2 - x1) + tw * (x2 - x3), v2y = y2 + tu * (y2 - y1) + tw * (y2 - y3);
    float v3x = x3 + tu * (x3 - x1) + tv * (x3 - x2), v3y = y3 + tu * (y3 - y1) + tv * (y3 - y2);
    float slack = 1.0e-3f + 4.0e-6f * (fabsf(x1) + fabsf(x2) + fabsf(x3) + fabsf(y1) + fabsf(y2) + fabsf(y3));
    float fx0 = fminf(fminf(v1x, v2x), v3x) - slack, fx1 = fmaxf(fmaxf(v1x, v2x), v3x) + slack;
    float fy0 = fminf(fminf(v1y, v2y), v3y) - slack, fy1 = fmaxf(fmaxf(v1y, v2y), v3y) + slack;
    // a side only constrains where the frame has pixel centres beyond it
    // (ix0 etc. are clamped to [-1, W] / [-1, H])
    bool ok_l = ix0 <= 0 || fx0 > (float)ix0 - 0.5f;
    bool ok_r = ix1 >= (int)W - 1 || fx1 < (float)ix1 + 1.5f;
    bool ok_t = iy0 <= 0 || fy0 > (float)iy0 - 0.5f;
    bool ok_b = iy1 >= (int)H - 1 || fy1 < (float)iy1 + 1.5f;
    return ok_l && ok_r && ok_t && ok_b;
}

}  // namespace sr
