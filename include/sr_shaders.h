/*
 * sr_shaders.h — shader arithmetic shared by the CUDA device code and host code.
 *
 * In softrender the vertex, fragment and blend stages are user closures written
 * against nalgebra (examples/suzanne.rs:123-183, full_example/src/shaders.rs,
 * full_example/src/texture.rs, full_example/src/color.rs).  This header restates
 * the arithmetic of those closures once, as __host__ __device__ functions, so
 * that the GPU kernels and any host-side caller execute the same IEEE-754 FP32
 * operation sequence.  It must be compiled without FMA contraction
 * (nvcc -fmad=false; gcc/clang -ffp-contract=off) and without fast-math.
 *
 * Operation-order conventions (nalgebra 0.12, num-traits 0.1 semantics):
 *   - dot / norm_squared: left-to-right sum  ((a0*b0 + a1*b1) + a2*b2) + a3*b3
 *   - Matrix4 * Vector4 and Matrix4 * Matrix4: each output element summed k=0..3
 *   - Vector / scalar: component-wise IEEE division
 *   - f32::min / f32::max: NaN-ignoring (fminf / fmaxf)
 *   - f32::powi: square-and-multiply, the algorithm of LLVM's __powisf2
 *   - `as u8`: truncate toward zero, saturate to [0,255], NaN -> 0
 * f32::powf is libm's in the reference; here it is sr_powf below (own
 * implementation: table-driven double-float log2 and exp2, tables generated by
 * rust-softrender_gb300/gen_pow_tables.py; measured within 0.51 ULP of the
 * exact power).
 * Explicit fused multiply-adds (sr_fma) appear only inside these library
 * functions (pow, the byte -> unit conversion), which are defined here, not
 * restated from the reference.
 *
 * Matrices are 16 floats, row-major: m[row*4 + col].
 */
#ifndef SR_SHADERS_H
#define SR_SHADERS_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SR_HD __host__ __device__ __forceinline__
#else
#define SR_HD static inline
#endif

#if !defined(__CUDACC__)
#include <math.h>
#endif

#ifdef __cplusplus
extern "C++" {
#endif

struct sr_v4 { float x, y, z, w; };

/* Paired single-precision operations of sm_100 and later (mul and fma on
 * .f32x2): one instruction gives two IEEE round-to-nearest results, each
 * equal to the scalar operation's.  The device uses them for two colour
 * channels of the RGBA8 conversions and of the over operator's quotients;
 * the host and every other target compute the same values one at a time. */
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
#define SR_PAIRED 1
/* Written as PTX.  The code generator was seen to fuse a paired product
 * with a paired sum consuming it although fused multiply-adds are disabled
 * (the GPU parity tests caught 1-ulp differences), so a paired product is
 * used only where no addition consumes it (a clamp, a multiplicand, the
 * addend of a fused multiply-add); sums of products stay scalar, two
 * roundings as the reference computes them. */
__device__ __forceinline__ float2 sr_mul2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 sr_fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mov.b64 pc, {%6, %7};\n\tfma.rn.f32x2 pd, pa, pb, pc;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
#endif

SR_HD sr_v4 sr_make_v4(float x, float y, float z, float w) { sr_v4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }

SR_HD uint32_t sr_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
SR_HD float sr_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f; memcpy(&f, &u, 4); return f;
#endif
}

SR_HD bool sr_isnan(float x) { return x != x; }
SR_HD bool sr_isinf(float x) { return (sr_f2u(x) & 0x7fffffffu) == 0x7f800000u; }
SR_HD float sr_fabs(float x) { return sr_u2f(sr_f2u(x) & 0x7fffffffu); }

/* f32::min / f32::max: if one argument is NaN the other is returned. */
SR_HD float sr_min(float a, float b) {
    if (sr_isnan(a)) return b;
    if (sr_isnan(b)) return a;
    return a < b ? a : b;
}
SR_HD float sr_max(float a, float b) {
    if (sr_isnan(a)) return b;
    if (sr_isnan(b)) return a;
    return a > b ? a : b;
}

SR_HD float sr_floor(float x) {
#if defined(__CUDA_ARCH__)
    return floorf(x);
#else
    return floorf(x);
#endif
}
SR_HD float sr_rint(float x) {  /* round half to even */
#if defined(__CUDA_ARCH__)
    return rintf(x);
#else
    return rintf(x);
#endif
}
SR_HD float sr_sqrt(float x) {  /* IEEE correctly rounded on both sides */
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return sqrtf(x);
#endif
}

/* Rust `f as u8` (saturating cast): NaN -> 0, truncation toward zero.  On
 * the device the same function as a clamp and one truncating conversion:
 * fmaxf returns its other operand for a quiet NaN (IEEE maxNum), so NaN and
 * everything <= 0 clamp to 0 and everything >= 255 to 255, and the clamped
 * value truncates as the cast does.  Equal for every input but a signalling
 * NaN, which no arithmetic result is (every caller passes a product or a
 * sum); checked over all 2^32 bit patterns by the tests. */
SR_HD uint8_t sr_f32_to_u8_clamp(float x) { return (uint8_t)(uint32_t)fminf(fmaxf(x, 0.0f), 255.0f); }
SR_HD uint8_t sr_f32_to_u8(float x) {
#if defined(__CUDA_ARCH__)
    return sr_f32_to_u8_clamp(x);
#else
    if (!(x > 0.0f)) return 0;
    if (x >= 255.0f) return 255;
    return (uint8_t)(int)x;
#endif
}

/* ---------------------------------------------------------------- vectors */
SR_HD sr_v4 sr_add4(sr_v4 a, sr_v4 b) { return sr_make_v4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
SR_HD sr_v4 sr_sub4(sr_v4 a, sr_v4 b) { return sr_make_v4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
SR_HD sr_v4 sr_scale4(sr_v4 a, float s) { return sr_make_v4(a.x * s, a.y * s, a.z * s, a.w * s); }
SR_HD float sr_dot4(sr_v4 a, sr_v4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
/* nalgebra normalize(): self / self.norm(), norm = sqrt(norm_squared) */
SR_HD sr_v4 sr_normalize4(sr_v4 a) {
    float n = sr_sqrt(sr_dot4(a, a));
    return sr_make_v4(a.x / n, a.y / n, a.z / n, a.w / n);
}

/* Matrix4 * Vector4 (row-major storage) */
SR_HD sr_v4 sr_m4_mul_v4(const float* m, sr_v4 v) {
    sr_v4 r;
    r.x = ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3] * v.w;
    r.y = ((m[4] * v.x + m[5] * v.y) + m[6] * v.z) + m[7] * v.w;
    r.z = ((m[8] * v.x + m[9] * v.y) + m[10] * v.z) + m[11] * v.w;
    r.w = ((m[12] * v.x + m[13] * v.y) + m[14] * v.z) + m[15] * v.w;
    return r;
}
/* Matrix4 * Matrix4 (row-major storage), out may not alias a or b */
SR_HD void sr_m4_mul_m4(const float* a, const float* b, float* out) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            out[i * 4 + j] = ((a[i * 4 + 0] * b[0 * 4 + j] + a[i * 4 + 1] * b[1 * 4 + j])
                              + a[i * 4 + 2] * b[2 * 4 + j]) + a[i * 4 + 3] * b[3 * 4 + j];
}

/* ------------------------------------------------------ powi (square-and-multiply) */
SR_HD float sr_powi(float x, int n) {
    int recip = n < 0;
    unsigned b = recip ? (unsigned)(-(long long)n) : (unsigned)n;
    float r = 1.0f;
    for (;;) {
        if (b & 1u) r = r * x;
        b >>= 1;
        if (b == 0) break;
        x = x * x;
    }
    return recip ? 1.0f / r : r;
}

/* ---------------------------------------------- double-float building blocks
 * Error-free transformations: Knuth's TwoSum, Dekker's FastTwoSum, and the
 * exact product error e = fma(a, b, -a*b).  Explicit fused multiply-adds are
 * single correctly rounded operations on every IEEE-754 target (CUDA fma.rn,
 * C99 fmaf), so host and device results are identical; they are used only
 * inside these library functions, never in the restated shader expressions. */
SR_HD float sr_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
SR_HD void sr_two_sum(float a, float b, float* s, float* e) {
    float ss = a + b;
    float bb = ss - a;
    *e = (a - (ss - bb)) + (b - bb);
    *s = ss;
}
SR_HD void sr_fast_two_sum(float a, float b, float* s, float* e) {  /* |a| >= |b| */
    float ss = a + b;
    *e = b - (ss - a);
    *s = ss;
}
SR_HD void sr_two_prod(float a, float b, float* p, float* e) {
    float pp = a * b;
    *e = sr_fma(a, b, -pp);
    *p = pp;
}

/* 2^n for integer n in [-126, 127] */
SR_HD float sr_exp2i(int n) { return sr_u2f((uint32_t)(n + 127) << 23); }

#include "sr_pow_tables.h"

/*
 * log2(x) for finite x > 0, returned as a double-float hi + lo (table-driven).
 * x = m * 2^e with m in [1, 2); i = the top 6 fraction bits of m selects
 * INV[i] ~ 1/c_i (c_i the centre of m's 1/64-wide interval) and
 * L[i] = -log2(INV[i]) (a float pair); r = m * INV[i] - 1 is formed exactly as
 * a double-float (|r| < 2^-7) and ln(1 + r) = r + r^2 q(r) with
 * q = -1/2 + r/3 - r^2/4 + r^3/5 - r^4/6 (truncation < 2^-52).
 * log2(x) = e + L[i] + ln(1 + r) * log2(e).
 */
SR_HD void sr_log2_df(float x, float* lhi, float* llo) {
    uint32_t bits = sr_f2u(x);
    int e = (int)((bits >> 23) & 0xffu);
    if (e == 0) {                     /* subnormal: rescale by 2^23 */
        x = x * 8388608.0f;
        bits = sr_f2u(x);
        e = (int)((bits >> 23) & 0xffu) - 23;
    }
    e -= 127;
    const float m = sr_u2f((bits & 0x007fffffu) | 0x3f800000u);  /* [1,2) */
    const int i = (int)((bits >> 17) & 63u);
    const float inv = SR_TAB(SR_LOG2_INV, i);
    float ph, pl;
    sr_two_prod(m, inv, &ph, &pl);    /* m * inv exactly */
    float rh, rl;
    sr_two_sum(ph - 1.0f, pl, &rh, &rl);   /* ph - 1 is exact (|ph - 1| < 2^-6) */
    float q = -0.16666666666666666f;                  /* -1/6 */
    q = sr_fma(rh, q, 0.2f);                          /*  1/5 */
    q = sr_fma(rh, q, -0.25f);                        /* -1/4 */
    q = sr_fma(rh, q, 0.33333333333333333f);          /*  1/3 */
    q = sr_fma(rh, q, -0.5f);                         /* -1/2 */
    const float tail = sr_fma(rh * rh, q, rl);
    float lnh, lnl;
    sr_fast_two_sum(rh, tail, &lnh, &lnl);
    /* ln -> log2: multiply by log2(e) = LOG2E_HI + LOG2E_LO */
    const float LOG2E_HI = 0x1.715476p+0f;
    const float LOG2E_LO = 0x1.4ae0cp-26f;
    float qh, ql;
    sr_two_prod(lnh, LOG2E_HI, &qh, &ql);
    ql = ql + (lnh * LOG2E_LO + lnl * LOG2E_HI);
    /* + e + L[i] */
    float sh, sl;
    sr_two_sum((float)e, SR_TAB(SR_LOG2_HI, i), &sh, &sl);
    sl = sl + SR_TAB(SR_LOG2_LO, i);
    float th, tl;
    sr_two_sum(sh, qh, &th, &tl);
    tl = tl + (sl + ql);
    sr_fast_two_sum(th, tl, lhi, llo);
}

/*
 * 2^(th + tl) for a double-float exponent (table-driven).  n = rint(th),
 * f = (th - n) + tl kept as a double-float, j = rint(64 f),
 * g = f - j/64 (|g| <= 1/128, exact); 2^f = T[j] * e^(g ln 2) with T[j] =
 * 2^(j/64) (a float pair) and e^x = 1 + x + x^2 (1/2 + x/6 + x^2/24 +
 * x^3/120) (truncation < 2^-52); then an exact scale by 2^n.
 */
SR_HD float sr_exp2_df(float th, float tl) {
    if (sr_isnan(th)) return th;
    if (th >= 128.0f) return sr_u2f(0x7f800000u);
    if (th < -151.0f) return 0.0f;
    const float n = sr_rint(th);
    float fh, fl;
    sr_two_sum(th - n, tl, &fh, &fl);                 /* th - n is exact */
    const float jf = sr_rint(fh * 64.0f);
    const int j = (int)jf;
    const float gh = fh - jf * 0.015625f;             /* exact: |gh| <= 1/128 + ulp */
    const float LN2_HI = 0x1.62e43p-1f;
    const float LN2_LO = -0x1.05c61p-29f;
    float xh, xl;
    sr_two_prod(gh, LN2_HI, &xh, &xl);
    xl = xl + (gh * LN2_LO + fl * LN2_HI);
    float p = 8.3333333333333332e-03f;                /* 1/5! */
    p = sr_fma(xh, p, 4.1666666666666664e-02f);       /* 1/4! */
    p = sr_fma(xh, p, 1.6666666666666666e-01f);       /* 1/3! */
    p = sr_fma(xh, p, 0.5f);                          /* 1/2! */
    const float ex = xh + sr_fma(xh * xh, p, xl);     /* e^x - 1 */
    const float t_hi = SR_TAB(SR_EXP2_HI, j + 32), t_lo = SR_TAB(SR_EXP2_LO, j + 32);
    const float res = t_hi + sr_fma(t_hi, ex, t_lo);
    const int ni = (int)n;
    if (ni >= -126 && ni <= 127) return res * sr_exp2i(ni);
    const int n1 = ni / 2;
    const int n2 = ni - n1;
    return (res * sr_exp2i(n1)) * sr_exp2i(n2);
}

SR_HD bool sr_is_integer(float y) { return sr_floor(y) == y && !sr_isinf(y); }
SR_HD bool sr_is_odd_integer(float y) {
    if (!sr_is_integer(y)) return false;
    float a = sr_fabs(y);
    if (a >= 16777216.0f) return false;
    return ((long long)a & 1LL) != 0;
}

/* f32::powf replacement with C99 Annex F special cases. */
SR_HD float sr_powf(float x, float y) {
    const float INF = sr_u2f(0x7f800000u);
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (sr_isnan(x) || sr_isnan(y)) return x + y;
    float ax = sr_fabs(x);
    if (sr_isinf(y)) {
        if (ax == 1.0f) return 1.0f;
        bool big = ax > 1.0f;
        return (big == (y > 0.0f)) ? INF : 0.0f;
    }
    bool odd = sr_is_odd_integer(y);
    if (x == 0.0f) {
        if (y < 0.0f) return odd ? (sr_f2u(x) >> 31 ? -INF : INF) : INF;
        return odd ? x : 0.0f;
    }
    if (sr_isinf(x)) {
        bool neg = x < 0.0f;
        if (y < 0.0f) return (neg && odd) ? -0.0f : 0.0f;
        return (neg && odd) ? -INF : INF;
    }
    float sign = 1.0f;
    if (x < 0.0f) {
        if (!sr_is_integer(y)) return (x - x) / (x - x);  /* NaN */
        if (odd) sign = -1.0f;
    }
    float lh, ll;
    sr_log2_df(ax, &lh, &ll);
    float th, tl;
    sr_two_prod(y, lh, &th, &tl);
    tl = tl + y * ll;
    float t2h, t2l;
    sr_fast_two_sum(th, tl, &t2h, &t2l);
    return sign * sr_exp2_df(t2h, t2l);
}

/* ------------------------------------------------------------------ colour */
/* full_example/src/color.rs:5-17, the alpha "over" operator on f32 RGBA. */
SR_HD float sr_over_component(float x, float y, float a, float b) {
    float a1 = 1.0f - a;
    return (x * a + (y * b) * a1) / (a + b * a1);
}
SR_HD sr_v4 sr_blend_over_f32(sr_v4 src, sr_v4 dst) {
    return sr_make_v4(sr_over_component(src.x, dst.x, src.w, dst.w),
                      sr_over_component(src.y, dst.y, src.w, dst.w),
                      sr_over_component(src.z, dst.z, src.w, dst.w),
                      src.w + dst.w * (1.0f - src.w));
}
SR_HD uint32_t sr_pack_rgba8(uint8_t r, uint8_t g, uint8_t b, uint8_t a) {
    return (uint32_t)r | ((uint32_t)g << 8) | ((uint32_t)b << 16) | ((uint32_t)a << 24);
}
/* RGBA f32 in [0,1] -> RGBA8 via (c * 255.0) as u8 per channel. */
SR_HD uint32_t sr_to_rgba8(sr_v4 c) {
#if defined(SR_PAIRED)
    const float2 k = make_float2(255.0f, 255.0f);
    const float2 rg = sr_mul2(make_float2(c.x, c.y), k), ba = sr_mul2(make_float2(c.z, c.w), k);
    return sr_pack_rgba8(sr_f32_to_u8(rg.x), sr_f32_to_u8(rg.y), sr_f32_to_u8(ba.x), sr_f32_to_u8(ba.y));
#else
    return sr_pack_rgba8(sr_f32_to_u8(c.x * 255.0f), sr_f32_to_u8(c.y * 255.0f),
                         sr_f32_to_u8(c.z * 255.0f), sr_f32_to_u8(c.w * 255.0f));
#endif
}
/* c as f32 / 255.0 for a byte c: the correctly rounded quotient, computed as
 * one fused c * r_hi + (c * r_lo) with r_hi + r_lo = 1/255 to 2^-57.  The sum
 * is within 2^-24 ulp of c/255 and c/255 is at least 2^-9 ulp from every
 * rounding midpoint (2 c 2^k - 255 (2 m + 1) is odd, so never 0), so the one
 * rounding gives the quotient's; equal to the IEEE division for all 256
 * values (checked exhaustively by the tests). */
#define SR_R255_HI 0x1.010102p-8f     /* 1/255 rounded */
#define SR_R255_LO (-0x1.fdfdfep-33f) /* 1/255 - SR_R255_HI rounded */
SR_HD float sr_u8_unit(uint32_t c) {
    const float x = (float)c;
    return sr_fma(x, SR_R255_HI, x * SR_R255_LO);
}
/* RGBA8 -> f32 as in from_image_texel (full_example/src/texture.rs:38-45): c as f32 / 255.0 */
SR_HD sr_v4 sr_from_rgba8(uint32_t p) {
#if defined(SR_PAIRED)
    const float2 hi = make_float2(SR_R255_HI, SR_R255_HI), lo = make_float2(SR_R255_LO, SR_R255_LO);
    const float2 rg = make_float2((float)(p & 0xffu), (float)((p >> 8) & 0xffu));
    const float2 ba = make_float2((float)((p >> 16) & 0xffu), (float)(p >> 24));
    const float2 urg = sr_fma2(rg, hi, sr_mul2(rg, lo)), uba = sr_fma2(ba, hi, sr_mul2(ba, lo));
    return sr_make_v4(urg.x, urg.y, uba.x, uba.y);
#else
    return sr_make_v4(sr_u8_unit(p & 0xffu), sr_u8_unit((p >> 8) & 0xffu),
                      sr_u8_unit((p >> 16) & 0xffu), sr_u8_unit(p >> 24));
#endif
}
/* n / d correctly rounded given r = 1/d correctly rounded, for the operands
 * of the RGBA8 over operator below: the quotient q0 = n r and one correction
 * by the exact residual n - d q0 (Markstein's division step).  Equal to the
 * IEEE quotient for every (colour, alpha) byte combination the operator can
 * see, checked exhaustively by the tests; not a general division. */
SR_HD float sr_over_div(float n, float d, float r) {
    const float q0 = n * r;
    const float e = sr_fma(-q0, d, n);
    return sr_fma(e, r, q0);
}
/* Over operator on RGBA8: channels to f32 (c/255), over, back with `as u8`
 * (sr_blend_over_f32 on the unit values).  The three colour quotients share
 * one denominator, which is also the result's alpha; its reciprocal is taken
 * once. */
SR_HD uint32_t sr_blend_over_rgba8(uint32_t src, uint32_t dst) {
    const sr_v4 s = sr_from_rgba8(src), t = sr_from_rgba8(dst);
    const float a = s.w, b = t.w;
    const float a1 = 1.0f - a;
    const float den = a + b * a1;
    const float r = 1.0f / den;
    sr_v4 c;
#if defined(SR_PAIRED)
    /* red and green quotients as one pair (the numerators are scalar sums);
     * fma(q0, -d, n) is fma(-q0, d, n) exactly */
    const float2 n = make_float2(s.x * a + (t.x * b) * a1, s.y * a + (t.y * b) * a1);
    const float2 R = make_float2(r, r), ND = make_float2(-den, -den);
    const float2 q0 = sr_mul2(n, R);
    const float2 q = sr_fma2(sr_fma2(q0, ND, n), R, q0);
    c.x = q.x;
    c.y = q.y;
#else
    c.x = sr_over_div(s.x * a + (t.x * b) * a1, den, r);
    c.y = sr_over_div(s.y * a + (t.y * b) * a1, den, r);
#endif
    c.z = sr_over_div(s.z * a + (t.z * b) * a1, den, r);
    c.w = den;
    return sr_to_rgba8(c);
}

/* decode_gamma / encode_gamma (full_example/src/color.rs:41-57) */
SR_HD sr_v4 sr_decode_gamma(sr_v4 c, float gamma) {
    return sr_make_v4(sr_powf(c.x, gamma), sr_powf(c.y, gamma), sr_powf(c.z, gamma), c.w);
}
SR_HD sr_v4 sr_encode_gamma(sr_v4 c, float gamma) {
    float inv = 1.0f / gamma;
    return sr_make_v4(sr_powf(c.x, inv), sr_powf(c.y, inv), sr_powf(c.z, inv), c.w);
}
/* ACES filmic tonemap (full_example/src/color.rs:19-35) */
SR_HD float sr_aces_component(float x) {
    return (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
}

/* ----------------------------------------------------------------- texture
 * Bilinear / nearest sampling of an RGBA8 or RGBA f32 texture, restating
 * full_example/src/texture.rs:47-84 (clamp: u.min(1).max(0); wrap: u.fract()).
 * Divergence, documented: the reference reads texel x+1 == width when
 * u*(W-1)+0.5 >= W-1 (an out-of-bounds panic at u == 1); here x+1 and y+1 are
 * clamped to the last texel, and x, y to [0, W-1] / [0, H-1].
 */
enum { SR_FILTER_NEAREST = 0, SR_FILTER_BILINEAR = 1 };
enum { SR_EDGE_CLAMP = 0, SR_EDGE_WRAP = 1, SR_EDGE_BORDER = 2 };

SR_HD float sr_fract(float v) {  /* Rust f32::fract: v - trunc(v) */
    return v - truncf(v);
}
SR_HD uint32_t sr_clamp_index(float f, uint32_t n) {
    if (!(f > 0.0f)) return 0;                 /* NaN and negatives -> 0 */
    if (f >= (float)(n - 1)) return n - 1;
    return (uint32_t)f;
}
/* One texel as RGBA f32: an RGBA8 texel as c/255 per channel
 * (from_image_texel), an RGBA f32 texel (the colour attachment of an RGBA f32
 * texture buffer, src/framebuffer/texturebuffer.rs:211-221) as stored. */
SR_HD sr_v4 sr_texel(const void* tex, uint32_t f32, uint32_t w, uint32_t x, uint32_t y) {
    const size_t i = (size_t)y * w + x;
    if (f32) {
#if defined(__CUDA_ARCH__)
        const float4 t = __ldg(reinterpret_cast<const float4*>(tex) + i);
        return sr_make_v4(t.x, t.y, t.z, t.w);
#else
        const float* t = (const float*)tex + 4 * i;
        return sr_make_v4(t[0], t[1], t[2], t[3]);
#endif
    }
#if defined(__CUDA_ARCH__)
    return sr_from_rgba8(__ldg((const uint32_t*)tex + i));
#else
    return sr_from_rgba8(((const uint32_t*)tex)[i]);
#endif
}
/* `f32`: the texture holds RGBA f32 texels, else RGBA8 */
SR_HD sr_v4 sr_sample(const void* tex, uint32_t f32, uint32_t w, uint32_t h, float u, float v,
                      int filter, int edge) {
    /* Border: coordinates outside [0, 1] (or NaN) read the border colour,
     * transparent black; inside, sampling is as with clamp. */
    if (edge == SR_EDGE_BORDER) {
        if (!(u >= 0.0f && u <= 1.0f && v >= 0.0f && v <= 1.0f)) return sr_make_v4(0.0f, 0.0f, 0.0f, 0.0f);
        edge = SR_EDGE_CLAMP;
    }
    if (edge == SR_EDGE_CLAMP) {
        u = sr_max(sr_min(u, 1.0f), 0.0f);
        v = sr_max(sr_min(v, 1.0f), 0.0f);
    } else {
        u = sr_fract(u);
        v = sr_fract(v);
    }
    if (filter == SR_FILTER_NEAREST) {
        uint32_t x = sr_clamp_index(roundf(u * (float)(w - 1)), w);
        uint32_t y = sr_clamp_index(roundf(v * (float)(h - 1)), h);
        return sr_texel(tex, f32, w, x, y);
    }
    float uu = (u * (float)(w - 1)) + 0.5f;
    float vv = (v * (float)(h - 1)) + 0.5f;
    uint32_t x = sr_clamp_index(sr_floor(uu), w);
    uint32_t y = sr_clamp_index(sr_floor(vv), h);
    float u_ratio = uu - (float)x;
    float v_ratio = vv - (float)y;
    float u_opp = 1.0f - u_ratio;
    float v_opp = 1.0f - v_ratio;
    uint32_t x1 = x + 1 < w ? x + 1 : w - 1;
    uint32_t y1 = y + 1 < h ? y + 1 : h - 1;
    sr_v4 a = sr_texel(tex, f32, w, x, y);
    sr_v4 b = sr_texel(tex, f32, w, x1, y);
    sr_v4 c = sr_texel(tex, f32, w, x, y1);
    sr_v4 d = sr_texel(tex, f32, w, x1, y1);
    sr_v4 r;
    r.x = (a.x * u_opp + b.x * u_ratio) * v_opp + (c.x * u_opp + d.x * u_ratio) * v_ratio;
    r.y = (a.y * u_opp + b.y * u_ratio) * v_opp + (c.y * u_opp + d.y * u_ratio) * v_ratio;
    r.z = (a.z * u_opp + b.z * u_ratio) * v_opp + (c.z * u_opp + d.z * u_ratio) * v_ratio;
    r.w = (a.w * u_opp + b.w * u_ratio) * v_opp + (c.w * u_opp + d.w * u_ratio) * v_ratio;
    return r;
}

/* ------------------------------------------------------------------ uniforms
 * Global uniforms for the shaders compiled into this library; the layout
 * follows GlobalUniforms of full_example/src/uniforms.rs with the light set
 * reduced to what each shader reads.  Set through sr_pipeline_set_uniforms.
 */
typedef struct sr_uniforms {
    float model[16];        /* object -> world                         */
    float mit[16];          /* inverse transpose of model (normals)    */
    float view[16];         /* world -> camera                         */
    float projection[16];   /* camera -> clip                          */
    float camera[4];        /* camera position (w = 1)                 */
    float light_dir[4];     /* directional light, normalised, w = 0    */
    float light_pos[4];     /* point light position (w = 1)            */
    float color[4];         /* linear surface colour                   */
    float intensity;        /* light intensity                         */
    float shininess;        /* Blinn-Phong shininess (suzanne: 32)     */
    float ior;              /* Fresnel index of refraction (1.45)      */
    float gamma;            /* display gamma (2.2)                     */
    float light_color[4][4];/* 4-light ACES shader: colours            */
    float light_pos4[4][4]; /* 4-light ACES shader: positions (w = 1)  */
    float light_int4[4];    /* 4-light ACES shader: intensities        */
    /* derived, filled by the library from the matrices above */
    float pv[16];           /* projection * view                        */
    float mvp[16];          /* (projection * view) * model              */
} sr_uniforms;

SR_HD void sr_uniforms_derive(sr_uniforms* u) {
    sr_m4_mul_m4(u->projection, u->view, u->pv);
    sr_m4_mul_m4(u->pv, u->model, u->mvp);
}

/* ----------------------------------------------------------- vertex shaders
 * Each returns the clip-space position and writes the varyings (the
 * declare_uniforms! structure, flattened field by field, component by
 * component).  Attribute planes are addressed by the caller.
 */

/* examples/suzanne.rs:123-141: world = model*pos; n = normalize(mit*n4);
 * clip = (projection*view)*world.  Varyings: world position (4), normal (4). */
SR_HD sr_v4 sr_vs_mvp_pos_nrm(const sr_uniforms* U, const float* a, float* k) {
    sr_v4 pos = sr_make_v4(a[0], a[1], a[2], 1.0f);
    sr_v4 n4 = sr_make_v4(a[3], a[4], a[5], 0.0f);
    sr_v4 world = sr_m4_mul_v4(U->model, pos);
    sr_v4 nrm = sr_normalize4(sr_m4_mul_v4(U->mit, n4));
    sr_v4 clip = sr_m4_mul_v4(U->pv, world);
    k[0] = world.x; k[1] = world.y; k[2] = world.z; k[3] = world.w;
    k[4] = nrm.x; k[5] = nrm.y; k[6] = nrm.z; k[7] = nrm.w;
    return clip;
}

/* full_example/src/shaders.rs:8-31: world = model*pos; n = normalize(mit*n4);
 * clip = ((projection*view)*model)*pos.  Varyings: position (4), normal (4), uv (2). */
SR_HD sr_v4 sr_vs_mvp_pos_nrm_uv(const sr_uniforms* U, const float* a, float* k) {
    sr_v4 pos = sr_make_v4(a[0], a[1], a[2], 1.0f);
    sr_v4 n4 = sr_make_v4(a[3], a[4], a[5], 0.0f);
    sr_v4 world = sr_m4_mul_v4(U->model, pos);
    sr_v4 nrm = sr_normalize4(sr_m4_mul_v4(U->mit, n4));
    sr_v4 clip = sr_m4_mul_v4(U->mvp, pos);
    k[0] = world.x; k[1] = world.y; k[2] = world.z; k[3] = world.w;
    k[4] = nrm.x; k[5] = nrm.y; k[6] = nrm.z; k[7] = nrm.w;
    k[8] = a[6]; k[9] = a[7];
    return clip;
}

/* Positions already in clip space (x, y, z, w) plus an RGBA colour given as
 * four floats in [0,1]; the colour is passed through as varyings. */
SR_HD sr_v4 sr_vs_clip_color(const sr_uniforms* U, const float* a, float* k) {
    (void)U;
    k[0] = a[4]; k[1] = a[5]; k[2] = a[6]; k[3] = a[7];
    return sr_make_v4(a[0], a[1], a[2], a[3]);
}

/* Positions in clip space with w = 1 (x, y, z planes) plus a packed RGBA8
 * colour plane (the u32 bit pattern stored in a float plane); the colour is
 * passed through as four varyings c/255. */
SR_HD sr_v4 sr_vs_clip_rgba8(const sr_uniforms* U, const float* a, float* k) {
    (void)U;
    sr_v4 c = sr_from_rgba8(sr_f2u(a[3]));
    k[0] = c.x; k[1] = c.y; k[2] = c.z; k[3] = c.w;
    return sr_make_v4(a[0], a[1], a[2], 1.0f);
}

/* --------------------------------------------------------- fragment shaders */

/* Fresnel-Schlick (examples/suzanne.rs:163-168) */
SR_HD float sr_fresnel_schlick(float cos_theta, float ior) {
    float f0 = sr_powi((1.0f - ior) / (1.0f + ior), 2);
    return f0 + (1.0f - f0) * sr_powi(1.0f - cos_theta, 5);
}

/* Blinn-Phong + Fresnel of examples/suzanne.rs:147-183 with one directional
 * light: L is the constant U->light_dir instead of normalize(light - position).
 * Returns the gamma-encoded RGBA f32 colour (alpha 1). */
SR_HD sr_v4 sr_blinn_phong(const sr_uniforms* U, sr_v4 position, sr_v4 normal, sr_v4 color) {
    sr_v4 camera = sr_make_v4(U->camera[0], U->camera[1], U->camera[2], U->camera[3]);
    sr_v4 light_dir = sr_make_v4(U->light_dir[0], U->light_dir[1], U->light_dir[2], U->light_dir[3]);
    sr_v4 view_dir = sr_normalize4(sr_sub4(camera, position));
    sr_v4 halfway = sr_normalize4(sr_add4(light_dir, view_dir));
    float NdotL = sr_max(sr_min(sr_dot4(light_dir, normal), 1.0f), 0.0f);
    float NdotH = sr_max(sr_min(sr_dot4(normal, halfway), 1.0f), 0.0f);
    float VdotH = sr_max(sr_min(sr_dot4(view_dir, halfway), 1.0f), 0.0f);
    float f = sr_fresnel_schlick(VdotH, U->ior);
    float diffuse = NdotL * (1.0f - f);
    float specular = f * sr_powf(NdotH, U->shininess * 2.0f);
    float inv_gamma = 1.0f / U->gamma;
    float I = U->intensity;
    return sr_make_v4(sr_powf(I * (specular + (diffuse * color.x)), inv_gamma),
                      sr_powf(I * (specular + (diffuse * color.y)), inv_gamma),
                      sr_powf(I * (specular + (diffuse * color.z)), inv_gamma),
                      1.0f);
}

/* ------------------------------------------------ RGBA8 shading, fast path
 * An RGBA8 target stores trunc(c * 255) of each gamma-encoded channel, so a
 * power known to within a stated relative error decides the stored byte
 * whenever c * 255 lies farther than that error from an integer.  The
 * functions below compute the Blinn-Phong channels with single-precision
 * powers on the tables of sr_log2_df / sr_exp2_df, carry a rigorous bound on
 * the distance to the exactly computed value (sr_powf and the same f32 ops)
 * through every step, and fall back to the exact computation for any pixel
 * whose byte the bound does not decide or whose values leave the ranges the
 * bound covers.  The returned word therefore equals
 * sr_to_rgba8(sr_blinn_phong(...)) for every input.
 *
 * Error budget of the two primitives (each term over-estimated 4x or more in
 * SR_FAST_POW_ERR; the CPU tests check the stated bounds on random and
 * boundary inputs):
 *   sr_ylog2_fast:  |t - y log2 x| <= |y| 2^-28 + |t| 2^-23
 *                   (ln(1+r) to 2^-29 absolute, the table pair exact to 2^-48,
 *                    y*e split exactly, two final roundings)
 *   sr_exp2_fast:   relative error <= 2^-22.9 (table value and final fma
 *                   rounding 2^-24 each, e^a - 1 to 2^-29 absolute)
 *   so 2^t / x^y - 1 is within ln 2 (|y| 2^-28 + |t| 2^-23) + 2^-22.9.
 */

/* y log2(x) for a normal x > 0 */
SR_HD float sr_ylog2_fast(float x, float y) {
    const uint32_t bits = sr_f2u(x);
    const float e = (float)((int)((bits >> 23) & 0xffu) - 127);
    const float m = sr_u2f((bits & 0x007fffffu) | 0x3f800000u);
    const int i = (int)((bits >> 17) & 63u);
    const float r = sr_fma(m, SR_TAB(SR_LOG2_INV, i), -1.0f);     /* |r| < 2^-7, one rounding */
    /* ln(1 + r) = r - r^2/2 + r^3/3 - r^4/4, truncation < 2^-37 */
    const float lnr = r * sr_fma(r, sr_fma(r, sr_fma(r, -0.25f, 0.33333334f), -0.5f), 1.0f);
    float sh, sl;
    sr_two_sum(SR_TAB(SR_LOG2_HI, i), lnr * 0x1.715476p+0f, &sh, &sl);
    sl = sl + SR_TAB(SR_LOG2_LO, i);
    const float p = y * e;
    const float pe = sr_fma(y, e, -p);                             /* y e = p + pe exactly */
    return sr_fma(y, sh, p) + (pe + y * sl);
}

/* 2^t for |t| <= 120 (a normal result) */
SR_HD float sr_exp2_fast(float t) {
    const float n = sr_rint(t);
    const float f = t - n;                                         /* exact, |f| <= 1/2 */
    const float jf = sr_rint(f * 64.0f);
    const float g = f - jf * 0.015625f;                            /* exact, |g| <= 1/128 */
    const float a = g * 0x1.62e430p-1f;                            /* g ln 2 */
    /* e^a - 1 = a + a^2/2 + a^3/6, truncation < 2^-34 */
    const float em1 = a * sr_fma(a, sr_fma(a, 0.16666667f, 0.5f), 1.0f);
    const float th = SR_TAB(SR_EXP2_HI, (int)jf + 32);
    return sr_fma(th, em1, th) * sr_exp2i((int)n);
}

/* Relative error bound of sr_exp2_fast(sr_ylog2_fast(x, y)) against x^y,
 * plus sr_powf's own (0.51 ulp <= 2^-23): a bound on |fast - sr_powf| / fast
 * up to a factor 1 + 2^-20. */
SR_HD float sr_fast_pow_err(float y, float t) {
    return sr_fabs(y) * 0x1p-26f + sr_fabs(t) * 0x1p-21f + 0x1p-20f;
}

/* `as u8` of a value known to be non-NaN */
SR_HD uint32_t sr_u8_of(float v) { return (uint32_t)sr_f32_to_u8(v); }

/*
 * The stored byte of one gamma-encoded channel, trunc(u^g * 255) with
 * u^g = sr_powf(u, g), where the u given is within du of the exactly
 * computed u.  Returns 256 when the bound does not decide the byte.
 */
SR_HD uint32_t sr_encode_byte_fast(float u, float du, float g) {
    /* unlit: |u_exact| <= 2^-63, so |u_exact^g| * 255 < 1 for g >= 1/4 (a
     * negative u_exact gives NaN or a value of the same tiny size): byte 0 */
    if (sr_fabs(u) + du <= 0x1p-64f && g >= 0.25f && g <= 256.0f) return 0u;
    if (!(u >= 0x1p-100f && u <= 0x1p100f && du <= u * 0x1p-10f && sr_fabs(g) <= 256.0f)) return 256u;
    const float t = sr_ylog2_fast(u, g);
    if (!(sr_fabs(t) <= 120.0f)) return 256u;
    const float G = sr_exp2_fast(t);
    /* |G - sr_powf(u_exact, g)| <= R G: the fast power's error and the
     * input's, |(1 +- d)^g - 1| <= 1.25 |g| d with d = du / u, which holds
     * because R <= 2^-8 below keeps |g| d under 2^-8.  On the device d is
     * bounded from above without a division: the hardware reciprocal of the
     * normal u (PTX rcp.approx.f32, within 1 ulp, 2^-23, of 1/u) and two
     * roundings (2^-24 each) stay under the 2^-20 added. */
#if defined(__CUDA_ARCH__)
    float ru;
    asm("rcp.approx.f32 %0, %1;" : "=f"(ru) : "f"(u));
    const float d = (du * ru) * (1.0f + 0x1p-20f);
#else
    const float d = du / u;
#endif
    const float R = sr_fast_pow_err(g, t) + 1.25f * sr_fabs(g) * d;
    if (!(R <= 0x1p-8f)) return 256u;
    const float v = G * 255.0f;
    /* both sides round G * 255 (2^-24 each); 2 ulp(v) more keep the rounded
     * ends v -+ B outside the exact interval */
    const float B = v * (R * 1.0625f + 0x1p-20f) + 0x1p-30f;
    const uint32_t lo = sr_u8_of(v - B), hi = sr_u8_of(v + B);
    return lo == hi ? lo : 256u;
}

/*
 * x^y for the decoded texel channel or the specular term: the value and a
 * bound on its distance to sr_powf(x, y), for x in [0, 1] and y in (0, 256].
 * Returns false when the case is outside the bound's domain.
 */
SR_HD bool sr_pow_bounded(float x, float y, float* val, float* err) {
    if (!(y > 0.0f && y <= 256.0f)) return false;
    if (x == 0.0f) { *val = sr_powf(x, y); *err = 0.0f; return true; }   /* exact zero (+0 or -0) */
    if (!(x >= 0x1p-100f && x <= 1.0f)) return false;
    /* y = 2^k, k = 1..7 (the Blinn-Phong shininess of the examples gives
     * 64): k squarings.  Each rounds once, so the relative error is at most
     * (2^k - 1) 2^-24 while the squares are normal; subnormal squares add at
     * most 2^-150 each, at most doubled by each later squaring (x <= 1), so
     * under 2^-143 in all.  sr_powf is within 0.51 ulp of x^y. */
    const uint32_t yb = sr_f2u(y);
    if ((yb & 0x007fffffu) == 0u && y >= 2.0f && y <= 128.0f) {
        const int k = (int)((yb >> 23) & 0xffu) - 127;
        float p = x;
        for (int i = 0; i < k; ++i) p = p * p;
        *val = p;
        *err = p * ((float)(1 << k) * 0x1p-23f + 0x1p-22f) + 0x1p-138f;   /* twice the bound */
        return true;
    }
    const float t = sr_ylog2_fast(x, y);
    if (t < -120.0f) { *val = 0.0f; *err = 0x1p-119f; return true; }  /* exact value < 2^-119.9 */
    if (!(t <= 120.0f)) return false;
    const float p = sr_exp2_fast(t);
    *val = p;
    *err = p * (sr_fast_pow_err(y, t) * 1.0625f) + 0x1p-140f;
    return true;
}

/*
 * sr_to_rgba8(sr_blinn_phong(U, position, normal, color)) where `color` is
 * within dcol (per channel, absolute) of the colour the exact computation
 * uses; returns false when the fast path cannot decide a byte.
 */
SR_HD bool sr_blinn_phong_rgba8_fast(const sr_uniforms* U, sr_v4 position, sr_v4 normal, sr_v4 color,
                                     sr_v4 dcol, uint32_t* out) {
    /* the same operations as sr_blinn_phong up to the powers */
    sr_v4 camera = sr_make_v4(U->camera[0], U->camera[1], U->camera[2], U->camera[3]);
    sr_v4 light_dir = sr_make_v4(U->light_dir[0], U->light_dir[1], U->light_dir[2], U->light_dir[3]);
    sr_v4 view_dir = sr_normalize4(sr_sub4(camera, position));
    sr_v4 halfway = sr_normalize4(sr_add4(light_dir, view_dir));
    float NdotL = sr_max(sr_min(sr_dot4(light_dir, normal), 1.0f), 0.0f);
    float NdotH = sr_max(sr_min(sr_dot4(normal, halfway), 1.0f), 0.0f);
    float VdotH = sr_max(sr_min(sr_dot4(view_dir, halfway), 1.0f), 0.0f);
    float f = sr_fresnel_schlick(VdotH, U->ior);
    float diffuse = NdotL * (1.0f - f);
    float P, dP;
    if (!sr_pow_bounded(NdotH, U->shininess * 2.0f, &P, &dP)) return false;
    const float specular = f * P;
    if (!(sr_fabs(specular) <= 0x1p100f && sr_fabs(diffuse) <= 0x1p100f)) return false;
    /* |f P - f P_exact| plus the rounding of both products */
    const float dspec = sr_fabs(f) * dP * 1.0625f + sr_fabs(specular) * 0x1p-22f + 0x1p-140f;
    const float inv_gamma = 1.0f / U->gamma;
    const float I = U->intensity;
    const float cc[3] = {color.x, color.y, color.z};
    const float dc[3] = {dcol.x, dcol.y, dcol.z};
    uint32_t bytes[3];
    for (int ch = 0; ch < 3; ++ch) {
        const float dcl = diffuse * cc[ch];
        const float t = specular + dcl;
        /* the two sums and products round on both sides (2^-23 of each) */
        const float dt = dspec + (sr_fabs(diffuse) * dc[ch] * 1.0625f + sr_fabs(dcl) * 0x1p-22f) +
                         sr_fabs(t) * 0x1p-22f;
        const float u = I * t;
        const float du = sr_fabs(I) * dt * 1.0625f + sr_fabs(u) * 0x1p-22f;
        const uint32_t b = sr_encode_byte_fast(u, du, inv_gamma);
        if (b > 255u) return false;
        bytes[ch] = b;
    }
    *out = bytes[0] | (bytes[1] << 8) | (bytes[2] << 16) | (255u << 24);   /* alpha 1.0 */
    return true;
}

/* The RGBA8 word of the Blinn-Phong fragment shader (uniform colour). */
SR_HD uint32_t sr_blinn_phong_rgba8(const sr_uniforms* U, sr_v4 position, sr_v4 normal, sr_v4 color) {
    uint32_t w;
    if (sr_blinn_phong_rgba8_fast(U, position, normal, color, sr_make_v4(0.0f, 0.0f, 0.0f, 0.0f), &w)) return w;
    return sr_to_rgba8(sr_blinn_phong(U, position, normal, color));
}

/* The RGBA8 word of the textured Blinn-Phong fragment shader: `texel` is the
 * sampled colour before decode_gamma. */
SR_HD uint32_t sr_textured_blinn_phong_rgba8(const sr_uniforms* U, sr_v4 position, sr_v4 normal, sr_v4 texel) {
    const float g = U->gamma;
    sr_v4 col, dcol;
    uint32_t w;
    if (sr_pow_bounded(texel.x, g, &col.x, &dcol.x) && sr_pow_bounded(texel.y, g, &col.y, &dcol.y) &&
        sr_pow_bounded(texel.z, g, &col.z, &dcol.z)) {
        col.w = texel.w;
        dcol.w = 0.0f;
        if (sr_blinn_phong_rgba8_fast(U, position, normal, col, dcol, &w)) return w;
    }
    return sr_to_rgba8(sr_blinn_phong(U, position, normal, sr_decode_gamma(texel, g)));
}

/* 4-point-light Blinn-Phong with ACES tonemap (full_example/src/shaders.rs:108-163). */
SR_HD sr_v4 sr_aces_lights(const sr_uniforms* U, sr_v4 position, sr_v4 normal) {
    sr_v4 camera = sr_make_v4(U->camera[0], U->camera[1], U->camera[2], U->camera[3]);
    sr_v4 view_dir = sr_normalize4(sr_sub4(camera, position));
    float g = U->gamma;
    sr_v4 material = sr_decode_gamma(sr_make_v4(0.25f, 0.25f, 0.25f, 1.0f), g);
    float albedo = 0.7f;
    sr_v4 col = sr_make_v4(0.0f, 0.0f, 0.0f, 1.0f);
    for (int i = 0; i < 4; ++i) {
        sr_v4 lp = sr_make_v4(U->light_pos4[i][0], U->light_pos4[i][1], U->light_pos4[i][2], U->light_pos4[i][3]);
        sr_v4 d = sr_sub4(lp, position);
        float light_distance = sr_sqrt(sr_dot4(d, d));
        sr_v4 light_dir = sr_normalize4(d);
        sr_v4 halfway = sr_normalize4(sr_add4(light_dir, view_dir));
        float intensity = U->light_int4[i] / sr_powi(light_distance, 2);
        float NdotL = sr_max(sr_min(sr_dot4(light_dir, normal), 1.0f), 0.0f);
        float NdotH = sr_max(sr_min(sr_dot4(normal, halfway), 1.0f), 0.0f);
        float VdotH = sr_max(sr_min(sr_dot4(view_dir, halfway), 1.0f), 0.0f);
        float f = sr_fresnel_schlick(VdotH, U->ior);
        float diffuse = (1.0f - f) * NdotL;
        float specular = f * sr_powi(NdotH, 32 * 2);
        col.x = col.x + intensity * U->light_color[i][0] * (specular + (diffuse * albedo * material.x));
        col.y = col.y + intensity * U->light_color[i][1] * (specular + (diffuse * albedo * material.y));
        col.z = col.z + intensity * U->light_color[i][2] * (specular + (diffuse * albedo * material.z));
    }
    sr_v4 t = sr_make_v4(sr_aces_component(col.x), sr_aces_component(col.y), sr_aces_component(col.z), col.w);
    return sr_encode_gamma(t, g);
}

#ifdef __cplusplus
}
#endif

#endif /* SR_SHADERS_H */
