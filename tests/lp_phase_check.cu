// Host check of the line / point raster schedule (lp_phase_step and
// lp_phase_first_row in rust-softrender_gb300/csrc/sr_internal.cuh): for
// frames and semantic tile sizes from 1 pixel up, with and without Xiaolin Wu
// lines (which plot one pixel beyond their tile),
//   - the phases enumerate every tile of the reference's walk
//     (fragment.rs:188-216) exactly once, within the launch's nrows blocks;
//   - any two tiles that can write a common pixel run in distinct phases, the
//     earlier phase holding the tile the reference visits first (row-major).
// Built by tests/test_lp_schedule.py with nvcc as host code; runs on the CPU.
//
// Prints "configs=... pairs=... bad=..." and exits 1 on a violation.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "sr_internal.cuh"

namespace {

// tile spans along one axis: [x, min(x + t, last)] while x < last
std::vector<std::pair<int, int>> spans(int E, int t) {
    std::vector<std::pair<int, int>> out;
    const int last = E - 1;
    for (int x = 0; x < last;) {
        const int nx = std::min(x + t, last);
        out.push_back({x, nx});
        x = nx;
    }
    return out;
}

long g_bad = 0;

}  // namespace

int main() {
    long configs = 0, pairs = 0;
    const int extents[] = {2, 3, 4, 5, 7, 8, 13, 17, 24};
    for (int wu = 0; wu < 2; ++wu)
        for (int W : extents)
            for (int H : extents)
                for (int tw = 1; tw <= 6; ++tw)
                    for (int th = 1; th <= 6; ++th) {
                        const auto cx = spans(W, tw), cy = spans(H, th);
                        const uint32_t ncols = (uint32_t)cx.size(), nrows = (uint32_t)cy.size();
                        const uint32_t K = sr::lp_phase_step(wu != 0, (uint32_t)tw);
                        const uint32_t phases = (ncols - 1) + K * (nrows - 1) + 1;
                        // the kernel's enumeration: block b of phase p is row r_lo + b
                        std::vector<int> seen(ncols * nrows, 0), phase_of(ncols * nrows, -1);
                        for (uint32_t p = 0; p < phases; ++p) {
                            const uint32_t r_lo = sr::lp_phase_first_row(p, ncols, K);
                            for (uint32_t b = 0; b < nrows; ++b) {
                                const int r = (int)(r_lo + b), c = (int)p - (int)K * r;
                                if (r >= (int)nrows || c < 0 || c >= (int)ncols) continue;
                                ++seen[r * ncols + c];
                                phase_of[r * ncols + c] = (int)p;
                            }
                        }
                        for (uint32_t i = 0; i < ncols * nrows; ++i)
                            if (seen[i] != 1) {
                                if (g_bad < 8) std::printf("tile %u seen %d times (W %d H %d tile %dx%d wu %d)\n", i,
                                                           seen[i], W, H, tw, th, wu);
                                ++g_bad;
                            }
                        // pixels a tile's pass can write: its span, one more each side for Wu lines
                        const int s = wu;
                        for (uint32_t a = 0; a < ncols * nrows; ++a)
                            for (uint32_t b = a + 1; b < ncols * nrows; ++b) {   // a before b, row-major
                                const auto& ax = cx[a % ncols]; const auto& ay = cy[a / ncols];
                                const auto& bx = cx[b % ncols]; const auto& by = cy[b / ncols];
                                const bool meet = std::max(ax.first - s, bx.first - s) <= std::min(ax.second + s, bx.second + s) &&
                                                  std::max(ay.first - s, by.first - s) <= std::min(ay.second + s, by.second + s);
                                if (!meet) continue;
                                ++pairs;
                                if (!(phase_of[a] < phase_of[b])) {
                                    if (g_bad < 8)
                                        std::printf("tiles %u (phase %d) and %u (phase %d) meet (W %d H %d tile %dx%d wu %d)\n",
                                                    a, phase_of[a], b, phase_of[b], W, H, tw, th, wu);
                                    ++g_bad;
                                }
                            }
                        ++configs;
                    }
    std::printf("configs=%ld pairs=%ld bad=%ld\n", configs, pairs, g_bad);
    return g_bad ? 1 : 0;
}
