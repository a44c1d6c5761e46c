// Host check of the tensor-core update tiling (compiled by tests/test_tile_decode.py):
// for update jobs over a sweep of front shapes, tc_job_tiles (the plan's tile count) equals
// the number of (column tile, row tile) pairs of the job's lower trapezoid, and
// tc_decode_tile (the kernel's tile order) maps [0, tiles) one to one onto them.
#include <cstdio>
#include <set>
#include <utility>

#include "common.cuh"

using namespace uchol_dev;

static int check(int c0, int cend, int m) {
    long long expect = 0;
    std::set<std::pair<int, int>> all;
    for (int j0 = c0; j0 < cend; j0 += kTcCols)
        for (int i0 = j0; i0 < m; i0 += kTcRows) {
            all.insert({i0, j0});
            ++expect;
        }
    const long long tiles = tc_job_tiles(c0, cend, m);
    if (tiles != expect) {
        std::printf("count mismatch: c0 %d cend %d m %d: %lld vs %lld\n", c0, cend, m, tiles, expect);
        return 1;
    }
    std::set<std::pair<int, int>> seen;
    for (long long t = 0; t < tiles; ++t) {
        int i0, j0, jend;
        tc_decode_tile(c0, cend, m, t, i0, j0, jend);
        const int jlim = j0 + kTcCols < cend ? j0 + kTcCols : cend;
        if (!all.count({i0, j0}) || !seen.insert({i0, j0}).second || jend != jlim) {
            std::printf("decode error: c0 %d cend %d m %d tile %lld -> (%d, %d, %d)\n", c0, cend, m, t, i0, j0, jend);
            return 1;
        }
    }
    return 0;
}

int main() {
    long long jobs = 0;
    for (int m = 1; m <= 3000; m += (m < 600 ? 7 : 97))
        for (int c0 = 0; c0 < m; c0 += (c0 < 300 ? 13 : 211)) {
            const int cends[] = {c0 + 1, c0 + 64, c0 + 128, c0 + 129, c0 + 512, c0 + 700, c0 + 1100, c0 + 2049, m};
            for (int cend : cends) {
                if (cend > m) continue;
                if (check(c0, cend, m)) return 1;
                ++jobs;
            }
        }
    // large fronts (a few shapes of the benchmark's sizes)
    const int big[][3] = {{0, 28629, 28629}, {128, 640, 28629}, {19456, 19932, 19932}, {2867, 12000, 12000}};
    for (const auto& b : big) {
        if (check(b[0], b[1], b[2])) return 1;
        ++jobs;
    }
    std::printf("ok %lld jobs\n", jobs);
    return 0;
}
