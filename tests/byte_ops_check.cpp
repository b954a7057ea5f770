// Exhaustive host check of the RGBA8 byte arithmetic of include/sr_shaders.h
// that the kernels compute in a cheaper form than the reference's.  Built and
// run by tests/test_byte_ops.py (g++, -ffp-contract=off, the oracle's flags).
//
//   cast     sr_f32_to_u8_clamp (the device form of `as u8`: clamp with
//            fminf/fmaxf, then truncate) equals sr_f32_to_u8 (the reference's
//            saturating cast, NaN -> 0) for all 2^32 float bit patterns but
//            the 2^23 - 2 signalling NaNs, which no arithmetic result is
//   unit     sr_u8_unit(c) equals the IEEE quotient c / 255 for all 256 bytes
//   over     for every (colour x, colour y, alpha a, alpha b) byte quadruple
//            (2^32 of them): the numerator and denominator of the over
//            operator on the unit values, and sr_over_div(n, d, 1/d) equal to
//            the IEEE quotient n / d bit for bit (NaN where it is NaN)
//   words    sr_blend_over_rgba8 against sr_to_rgba8(sr_blend_over_f32(...))
//            on random source and destination words
//
// Prints "cast_mismatches=... unit_mismatches=... over_mismatches=...
// word_mismatches=..." and exits 1 on any mismatch.
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/sr_shaders.h"

namespace {

bool same_bits(float p, float q) {
    if (p != p && q != q) return true;
    uint32_t a, b;
    std::memcpy(&a, &p, 4);
    std::memcpy(&b, &q, 4);
    return a == b;
}

template <class F>
uint64_t parallel_count(uint32_t n_parts, F part) {
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 4;
    if (nt > 64) nt = 64;
    std::atomic<uint32_t> next{0};
    std::atomic<uint64_t> bad{0};
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&] {
            uint64_t local = 0;
            for (uint32_t i; (i = next.fetch_add(1)) < n_parts;) local += part(i);
            bad += local;
        });
    for (auto& t : th) t.join();
    return bad.load();
}

}  // namespace

int main() {
    // cast: 2^32 bit patterns in 65536 parts of 65536
    const uint64_t cast_bad = parallel_count(65536u, [](uint32_t hi) {
        uint64_t bad = 0;
        for (uint32_t lo = 0; lo < 65536u; ++lo) {
            const uint32_t bits = (hi << 16) | lo;
            if ((bits & 0x7fc00000u) == 0x7f800000u && (bits & 0x003fffffu) != 0u) continue;   // signalling NaN
            float x;
            std::memcpy(&x, &bits, 4);
            bad += sr_f32_to_u8_clamp(x) != sr_f32_to_u8(x);
        }
        return bad;
    });

    uint64_t unit_bad = 0;
    for (uint32_t c = 0; c < 256; ++c) unit_bad += !same_bits(sr_u8_unit(c), (float)c / 255.0f);

    // over: one part per (a, b) alpha pair, all (x, y) colour pairs in it
    const uint64_t over_bad = parallel_count(65536u, [](uint32_t ab) {
        uint64_t bad = 0;
        const float a = sr_u8_unit(ab & 255u), b = sr_u8_unit(ab >> 8);
        const float a1 = 1.0f - a;
        const float den = a + b * a1;
        const float r = 1.0f / den;
        for (uint32_t x = 0; x < 256; ++x) {
            const float xa = sr_u8_unit(x) * a;
            for (uint32_t y = 0; y < 256; ++y) {
                const float n = xa + (sr_u8_unit(y) * b) * a1;
                bad += !same_bits(sr_over_div(n, den, r), n / den);
            }
        }
        return bad;
    });

    uint64_t word_bad = 0;
    uint64_t st = 0x243f6a8885a308d3ull;
    for (int i = 0; i < 4000000; ++i) {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        const uint32_t s = (uint32_t)(st >> 32), d = (uint32_t)st;
        word_bad += sr_blend_over_rgba8(s, d) != sr_to_rgba8(sr_blend_over_f32(sr_from_rgba8(s), sr_from_rgba8(d)));
    }

    std::printf("cast_mismatches=%llu unit_mismatches=%llu over_mismatches=%llu word_mismatches=%llu\n",
                (unsigned long long)cast_bad, (unsigned long long)unit_bad, (unsigned long long)over_bad,
                (unsigned long long)word_bad);
    return (cast_bad | unit_bad | over_bad | word_bad) ? 1 : 0;
}
