// Host check of the sign tests that skip pixels without evaluating them
// (segment_cleared / rect_cleared in rust-softrender_gb300/csrc/sr_internal.cuh):
// whenever a test declares a pixel rectangle cleared, no pixel in it may be
// covered under the reference's coverage evaluation (triangle.rs:104-113,
// f32, no contraction) of the setup record the setup kernels build.
// Built by tests/test_rect_clear.py with nvcc as host code; runs on the CPU.
//
// Prints "cleared=... pixels=... violations=..." and exits 1 on a violation.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "sr_internal.cuh"

namespace {

uint64_t g_state = 1;
uint64_t next_u64() {   // splitmix64
    uint64_t z = (g_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
double uni(double lo, double hi) { return lo + (hi - lo) * ((next_u64() >> 11) * (1.0 / 9007199254740992.0)); }

// the coverage test of frag_emit / the reference, per pixel
bool covered(const float4& r0, const float4& r1, int px, int py) {
    const float x = (float)px + 0.5f, y = (float)py + 0.5f;
    const float dx = x - r1.x, dy = y - r1.y;
    const float u = (r0.x * dx + r0.y * dy) / r1.z;
    const float v = (r0.z * dx + r0.w * dy) / r1.z;
    const float w = 1.0f - u - v;
    return !(u < 0.0f || v < 0.0f || w < 0.0f);
}

}  // namespace

int main(int argc, char** argv) {
    const long n = argc > 1 ? atol(argv[1]) : 200000;
    g_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
    long cleared = 0, pixels = 0, violations = 0, seg_cleared = 0;
    for (long k = 0; k < n; ++k) {
        // screen-space triangles: generic, slivers, tiny, far from the origin
        const int kind = (int)(k % 4);
        const double ox = kind == 3 ? uni(1e3, 3e4) : 0.0, oy = kind == 3 ? uni(1e3, 3e4) : 0.0;
        double X[3], Y[3];
        for (int j = 0; j < 3; ++j) { X[j] = ox + uni(0, 200); Y[j] = oy + uni(0, 200); }
        if (kind == 1) {   // third vertex within 1e-2 .. 1e-6 of the line through the first two
            const double t = uni(-0.5, 1.5), off = std::pow(10.0, -uni(2, 6)) * (next_u64() & 1 ? 1 : -1);
            const double ex = X[1] - X[0], ey = Y[1] - Y[0], len = std::sqrt(ex * ex + ey * ey) + 1e-30;
            X[2] = X[0] + t * ex - ey / len * off;
            Y[2] = Y[0] + t * ey + ex / len * off;
        } else if (kind == 2) {   // area below a pixel
            for (int j = 1; j < 3; ++j) { X[j] = X[0] + uni(-1.5, 1.5); Y[j] = Y[0] + uni(-1.5, 1.5); }
        }
        const float x1 = (float)X[0], y1 = (float)Y[0], x2 = (float)X[1], y2 = (float)Y[1];
        const float x3 = (float)X[2], y3 = (float)Y[2];
        // the setup record (sr_setup.cu): edge terms, anchor, det
        const float det = (y2 - y3) * (x1 - x3) + (x3 - x2) * (y1 - y3);
        if (!(det != 0.0f) || std::isnan(det)) continue;   // such primitives get no record
        const float4 r0 = make_float4(y2 - y3, x3 - x2, y3 - y1, x1 - x3);
        const float4 r1 = make_float4(x3, y3, det, 0.0f);
        // rectangles around and near the triangle (non-negative pixel coordinates)
        const double mnx = std::fmin(std::fmin(X[0], X[1]), X[2]), mxx = std::fmax(std::fmax(X[0], X[1]), X[2]);
        const double mny = std::fmin(std::fmin(Y[0], Y[1]), Y[2]), mxy = std::fmax(std::fmax(Y[0], Y[1]), Y[2]);
        for (int rr = 0; rr < 4; ++rr) {
            int rx0 = (int)std::floor(uni(mnx - 8, mxx + 8)), ry0 = (int)std::floor(uni(mny - 8, mxy + 8));
            if (rx0 < 0) rx0 = 0;
            if (ry0 < 0) ry0 = 0;
            const int rw = (int)uni(0, 24), rh = rr == 3 ? 0 : (int)uni(0, 24);
            const int rx1 = rx0 + rw, ry1 = ry0 + rh;
            const bool seg = rr == 3;   // a one-row segment through segment_cleared as well
            const bool c = sr::rect_cleared(r0, r1, rx0, ry0, rx1, ry1);
            const bool cs = seg && sr::segment_cleared(r0, r1, (uint32_t)rx0, (uint32_t)ry0, (uint32_t)rx1, (uint32_t)ry1);
            if (!c && !cs) continue;
            cleared += c ? 1 : 0;
            seg_cleared += cs ? 1 : 0;
            for (int py = ry0; py <= ry1; ++py)
                for (int px = rx0; px <= rx1; ++px) {
                    ++pixels;
                    if (covered(r0, r1, px, py)) {
                        if (violations < 5)
                            printf("violation: tri (%.9g,%.9g) (%.9g,%.9g) (%.9g,%.9g) rect [%d,%d]x[%d,%d] px %d %d\n",
                                   x1, y1, x2, y2, x3, y3, rx0, rx1, ry0, ry1, px, py);
                        ++violations;
                    }
                }
        }
    }
    printf("cleared=%ld seg_cleared=%ld pixels=%ld violations=%ld\n", cleared, seg_cleared, pixels, violations);
    return violations ? 1 : 0;
}
