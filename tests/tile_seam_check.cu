// Host check of the semantic-tile arithmetic the raster kernels use for pass
// ranks: seam_count with its division magic (sr_opaque.cuh, per-pixel keys of
// the opaque path) and tiles_of (sr_internal.cuh, the extension pass and the
// ordered path), against the reference's tile walk along one axis
// (fragment.rs:188-216: x = 0; while x < last { nx = min(x + t, last);
// tile [x, nx]; x = nx }), for every tile size 1..65535.
// Built by tests/test_tile_seams.py with nvcc as host code; runs on the CPU.
//
// Prints "checked=... magic=... bad=..." and exits 1 on a mismatch.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "sr_opaque.cuh"

namespace {

uint64_t g_state = 7;
uint32_t next_u32() {   // xorshift64*
    g_state ^= g_state >> 12;
    g_state ^= g_state << 25;
    g_state ^= g_state >> 27;
    return (uint32_t)((g_state * 0x2545F4914F6CDD1Dull) >> 32);
}

long g_bad = 0;
void report(const char* what, uint32_t t, uint32_t E, uint32_t p, long got, long want) {
    if (g_bad < 8) std::printf("mismatch %s: tile %u extent %u p %u: got %ld want %ld\n", what, t, E, p, got, want);
    ++g_bad;
}

// Tiles of the walk containing each coordinate (count, first index), and the
// number of tiles, for extent E (frame width or height) and tile size t.
uint32_t walk(uint32_t E, uint32_t t, std::vector<uint8_t>& count, std::vector<uint32_t>& first) {
    const uint32_t last = E - 1;
    count.assign(E, 0);
    first.assign(E, 0);
    uint32_t n = 0;
    for (uint32_t x = 0; x < last;) {
        const uint32_t nx = std::min(x + t, last);
        for (uint32_t p = x; p <= nx; ++p) {
            if (!count[p]) first[p] = n;
            ++count[p];
        }
        ++n;
        x = nx;
    }
    return n;
}

}  // namespace

int main() {
    long checked = 0, magic = 0;
    std::vector<uint8_t> count;
    std::vector<uint32_t> first;
    // every coordinate of frames up to 4097 pixels, for every tile size
    const uint32_t small_extents[] = {2, 3, 5, 17, 128, 1000, 2160, 4097};
    // the largest frame (32767) for a sample of tile sizes
    std::vector<uint32_t> big_tiles;
    for (uint32_t t = 1; t <= 300; ++t) big_tiles.push_back(t);
    for (uint32_t k = 9; k < 16; ++k) big_tiles.push_back(1u << k);
    for (uint32_t t : {32765u, 32766u, 32767u, 32768u, 65535u}) big_tiles.push_back(t);
    for (int i = 0; i < 300; ++i) big_tiles.push_back(1 + next_u32() % 65535);

    auto check_axis = [&](uint32_t E, uint32_t t) {
        const uint32_t n = walk(E, t, count, first);
        const uint32_t last = E - 1, m = sr::div_magic(t);
        for (uint32_t p = 0; p <= last; ++p) {
            const int seams = sr::seam_count(p, t, m, last);
            const sr::TileSpan s = sr::tiles_of(p, t, n, last);
            if (seams != count[p]) report("seam_count", t, E, p, seams, count[p]);
            if (s.count != count[p]) report("tiles_of.count", t, E, p, s.count, count[p]);
            if ((uint32_t)s.first != first[p]) report("tiles_of.first", t, E, p, s.first, first[p]);
            ++checked;
        }
    };
    for (uint32_t t = 1; t <= 65535; ++t)
        for (uint32_t E : small_extents) check_axis(E, t);
    for (uint32_t t : big_tiles) check_axis(32767, t);

    // the division magic itself: floor(p / t) for p < 2^15, 2 <= t < 2^16,
    // at every multiple of t, its neighbours and random points
    for (uint32_t t = 2; t <= 65535; ++t) {
        const uint32_t m = sr::div_magic(t);
        auto one = [&](uint32_t p) {
            if (p >= 32768u) return;
            const uint32_t got = sr::umulhi32(p, m);
            if (got != p / t) report("div_magic", t, 32768, p, got, p / t);
            ++magic;
        };
        for (uint32_t k = t; k < 32768u; k += t) { one(k - 1); one(k); one(k + 1); }
        for (int i = 0; i < 16; ++i) one(next_u32() & 32767u);
        one(0);
        one(32767);
    }
    std::printf("checked=%ld magic=%ld bad=%ld\n", checked, magic, g_bad);
    return g_bad ? 1 : 0;
}
