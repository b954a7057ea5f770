// Host check of the RGBA8 fast shading path of include/sr_shaders.h against
// the exact computation it must reproduce byte for byte.  Built and run by
// tests/test_fast_shading.py (g++, -ffp-contract=off, the oracle's flags).
//
//   pow      sr_exp2_fast(sr_ylog2_fast(x, y)) against sr_powf(x, y): the
//            observed relative error stays under half of sr_fast_pow_err;
//            sr_pow_bounded by squaring (y = 2^k) within its stated bound
//   bytes    sr_encode_byte_fast(u, 0, g) next to every byte boundary
//            (u = (k/255)^(1/g) and its 512 float neighbours each side):
//            a decided byte equals trunc(sr_powf(u, g) * 255)
//   shade    sr_blinn_phong_rgba8 / sr_textured_blinn_phong_rgba8 against
//            sr_to_rgba8(sr_blinn_phong(...)) on random scenes
//
//   near     the same with the intensity steered so that the red channel's
//            255 c lies within 2^-14 of an integer (most of these fall back)
//
// Prints one line "pow_max_ratio=... byte_cases=... ... mismatches=..." and
// exits 1 on any mismatch or bound violation.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "../include/sr_shaders.h"

namespace {

uint64_t g_state = 0x9e3779b97f4a7c15ull;
uint64_t next_u64() {   // splitmix64
    uint64_t z = (g_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
float uni(float lo, float hi) { return lo + (hi - lo) * (float)((next_u64() >> 40) * (1.0 / 16777216.0)); }

sr_v4 unit3(float w) {
    for (;;) {
        float x = uni(-1, 1), y = uni(-1, 1), z = uni(-1, 1);
        float n = std::sqrt(x * x + y * y + z * z);
        if (n > 0.1f && n <= 1.0f) return sr_make_v4(x / n, y / n, z / n, w);
    }
}

uint32_t exact_rgba8(const sr_uniforms* U, sr_v4 p, sr_v4 n, sr_v4 c) {
    return sr_to_rgba8(sr_blinn_phong(U, p, n, c));
}

}  // namespace

int main(int argc, char** argv) {
    const long n_pow = argc > 1 ? atol(argv[1]) : 400000;
    const long n_shade = argc > 2 ? atol(argv[2]) : 400000;
    g_state = argc > 3 ? strtoull(argv[3], nullptr, 10) : 1;
    long mismatches = 0;

    // ---- pow: the stated error bound
    double worst = 0.0;
    const float ys[] = {1.0f / 2.2f, 2.2f, 1.0f / 1.8f, 1.8f, 64.0f, 10.0f, 255.0f, 0.5f};
    for (long k = 0; k < n_pow; ++k) {
        const float y = (k % 4 == 3) ? uni(0.01f, 256.0f) : ys[k % 8];
        const float x = (k & 1) ? uni(0.0f, 1.0f) : std::exp2(uni(-100.0f, 0.0f));
        if (!(x >= 0x1p-100f && x <= 1.0f)) continue;
        const float t = sr_ylog2_fast(x, y);
        if (!(std::fabs(t) <= 120.0f)) continue;
        const float fast = sr_exp2_fast(t);
        const float ex = sr_powf(x, y);
        if (ex < 0x1p-125f) continue;   // the bound is relative for normal results
        const double rel = std::fabs((double)fast - (double)ex) / (double)fast;
        const double ratio = rel / (double)sr_fast_pow_err(y, t);
        if (ratio > worst) worst = ratio;
    }
    if (!(worst < 0.5)) ++mismatches;

    // ---- pow by squaring (exponents 2^k): within the stated absolute bound
    double worst_sq = 0.0;
    for (long k = 0; k < n_pow; ++k) {
        const float y = (float)(1 << (1 + (int)(k % 7)));
        const float x = (k & 1) ? uni(0.0f, 1.0f) : std::exp2(uni(-100.0f, 0.0f));
        float val = 0.0f, err = 0.0f;
        if (!sr_pow_bounded(x, y, &val, &err)) continue;
        const double d = std::fabs((double)val - (double)sr_powf(x, y));
        if (err > 0.0f && d / (double)err > worst_sq) worst_sq = d / (double)err;
        if (d > (double)err) ++mismatches;
    }

    // ---- bytes at every boundary
    long byte_cases = 0, byte_fallbacks = 0;
    const float gs[] = {1.0f / 2.2f, 1.0f / 1.8f, 0.5f, 1.0f, 2.2f};
    for (float g : gs)
        for (int k = 1; k <= 255; ++k) {
            const float u0 = (float)std::pow((double)k / 255.0, 1.0 / (double)g);
            uint32_t bits = sr_f2u(u0) - 512u;
            for (int j = 0; j <= 1024; ++j, ++bits) {
                const float u = sr_u2f(bits);
                const uint32_t b = sr_encode_byte_fast(u, 0.0f, g);
                ++byte_cases;
                if (b > 255u) { ++byte_fallbacks; continue; }
                if (b != sr_f32_to_u8(sr_powf(u, g) * 255.0f)) ++mismatches;
            }
        }

    // ---- whole shaders on random scenes
    long shade_cases = 0, shade_fallbacks = 0;
    for (long k = 0; k < n_shade; ++k) {
        sr_uniforms U;
        memset(&U, 0, sizeof(U));
        const sr_v4 cam = sr_make_v4(uni(-4, 4), uni(-4, 4), uni(-4, 4), 1.0f);
        const sr_v4 ld = unit3(0.0f);
        U.camera[0] = cam.x; U.camera[1] = cam.y; U.camera[2] = cam.z; U.camera[3] = cam.w;
        U.light_dir[0] = ld.x; U.light_dir[1] = ld.y; U.light_dir[2] = ld.z; U.light_dir[3] = ld.w;
        U.ior = uni(1.0f, 3.0f);
        U.shininess = (k & 1) ? 32.0f : uni(1.0f, 128.0f);
        U.gamma = (k & 2) ? 2.2f : uni(1.6f, 2.6f);
        U.intensity = uni(0.2f, 3.0f);
        U.color[0] = uni(0, 1); U.color[1] = uni(0, 1); U.color[2] = uni(0, 1); U.color[3] = 1.0f;
        const sr_v4 pos = sr_make_v4(uni(-1.5f, 1.5f), uni(-1.5f, 1.5f), uni(-1.5f, 1.5f), 1.0f);
        const sr_v4 nrm = unit3(0.0f);
        uint32_t w, fast;
        const bool textured = (k % 3) == 0;
        if (textured) {
            // bytes / 255 (nearest) or bilinear mixes of them
            sr_v4 t;
            float* tc[3] = {&t.x, &t.y, &t.z};
            for (float* c : tc) {
                const float a = sr_u8_unit((uint32_t)(next_u64() & 255)), b = sr_u8_unit((uint32_t)(next_u64() & 255));
                const float f = uni(0, 1);
                *c = (k & 4) ? a : a * (1.0f - f) + b * f;
            }
            t.w = 1.0f;
            w = sr_textured_blinn_phong_rgba8(&U, pos, nrm, t);
            const float g = U.gamma;
            sr_v4 col, dcol;
            bool ok = sr_pow_bounded(t.x, g, &col.x, &dcol.x) && sr_pow_bounded(t.y, g, &col.y, &dcol.y) &&
                      sr_pow_bounded(t.z, g, &col.z, &dcol.z);
            col.w = t.w; dcol.w = 0.0f;
            ok = ok && sr_blinn_phong_rgba8_fast(&U, pos, nrm, col, dcol, &fast);
            if (!ok) ++shade_fallbacks;
            if (w != exact_rgba8(&U, pos, nrm, sr_decode_gamma(t, g))) ++mismatches;
        } else {
            const sr_v4 c = sr_make_v4(U.color[0], U.color[1], U.color[2], U.color[3]);
            w = sr_blinn_phong_rgba8(&U, pos, nrm, c);
            if (!sr_blinn_phong_rgba8_fast(&U, pos, nrm, c, sr_make_v4(0, 0, 0, 0), &fast)) ++shade_fallbacks;
            if (w != exact_rgba8(&U, pos, nrm, c)) ++mismatches;
        }
        ++shade_cases;
    }
    // ---- whole shader with the red channel steered next to a byte boundary:
    // the intensity is chosen so that (I t)^(1/gamma) * 255 = k + e, |e| < 2^-14
    long near_cases = 0, near_fallbacks = 0;
    for (long k = 0; k < n_shade; ++k) {
        sr_uniforms U;
        memset(&U, 0, sizeof(U));
        const sr_v4 ld = unit3(0.0f);
        const sr_v4 nrm = ld;                        // lit: N . L = 1
        const sr_v4 pos = sr_make_v4(uni(-1, 1), uni(-1, 1), uni(-1, 1), 1.0f);
        U.camera[0] = pos.x + 3 * ld.x + uni(-1, 1); U.camera[1] = pos.y + 3 * ld.y + uni(-1, 1);
        U.camera[2] = pos.z + 3 * ld.z + uni(-1, 1); U.camera[3] = 1.0f;
        U.light_dir[0] = ld.x; U.light_dir[1] = ld.y; U.light_dir[2] = ld.z;
        U.ior = uni(1.0f, 3.0f);
        U.shininess = uni(1.0f, 128.0f);
        U.gamma = 2.2f;
        U.color[0] = uni(0.05f, 1); U.color[1] = uni(0, 1); U.color[2] = uni(0, 1); U.color[3] = 1.0f;
        U.intensity = 1.0f;
        // t of the red channel at intensity 1, from the exact shader's inputs
        const sr_v4 c = sr_make_v4(U.color[0], U.color[1], U.color[2], U.color[3]);
        const sr_v4 cam = sr_make_v4(U.camera[0], U.camera[1], U.camera[2], U.camera[3]);
        const sr_v4 vd = sr_normalize4(sr_sub4(cam, pos));
        const sr_v4 hw = sr_normalize4(sr_add4(ld, vd));
        const float NdotH = sr_max(sr_min(sr_dot4(nrm, hw), 1.0f), 0.0f);
        const float VdotH = sr_max(sr_min(sr_dot4(vd, hw), 1.0f), 0.0f);
        const float f = sr_fresnel_schlick(VdotH, U.ior);
        const float NdotL = sr_max(sr_min(sr_dot4(ld, nrm), 1.0f), 0.0f);
        const double t = (double)(f * sr_powf(NdotH, U.shininess * 2.0f)) + (double)(NdotL * (1.0f - f)) * c.x;
        if (!(t > 1e-6)) continue;
        const int kb = 1 + (int)(next_u64() % 254);
        const double target = (kb + (double)uni(-1.0f, 1.0f) * 0x1p-14) / 255.0;
        U.intensity = (float)(std::pow(target, 2.2) / t);
        uint32_t w, fast;
        w = sr_blinn_phong_rgba8(&U, pos, nrm, c);
        if (!sr_blinn_phong_rgba8_fast(&U, pos, nrm, c, sr_make_v4(0, 0, 0, 0), &fast)) ++near_fallbacks;
        if (w != exact_rgba8(&U, pos, nrm, c)) ++mismatches;
        ++near_cases;
    }
    printf("sq_max_ratio=%.4f pow_max_ratio=%.4f byte_cases=%ld byte_fallbacks=%ld shade_cases=%ld shade_fallbacks=%ld "
           "near_cases=%ld near_fallbacks=%ld mismatches=%ld\n",
           worst_sq, worst, byte_cases, byte_fallbacks, shade_cases, shade_fallbacks, near_cases, near_fallbacks,
           mismatches);
    return mismatches ? 1 : 0;
}
