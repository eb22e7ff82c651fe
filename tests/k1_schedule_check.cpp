// Coverage check of the mixed path's flux-kernel schedule (shark_gb300/csrc/k1_schedule.h): for
// each case on the command line (nx ny ndust warps iso), every row of every column block of the
// gas and of every dust species is marched by exactly one piece of one warp; a persistent
// schedule uses at most one wave of warps; no piece is shorter than one row.  Prints one line per
// case and exits non-zero on the first failure.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../shark_gb300/csrc/k1_schedule.h"

using shark::K1Class;

static bool cover(const char* name, const K1Class& c, int ny, long long& pieces) {
    std::vector<unsigned char> seen((size_t)c.B * ny, 0);
    for (int i = 0; i < c.n; ++i) {
        int t, r0, r1;
        for (int ph = 0; shark::k1_piece(c, ny, i, ph, t, r0, r1); ++ph) {
            if (t < 0 || t >= c.B || r0 < 0 || r1 >= ny || r1 < r0) {
                std::printf("%s: bad piece warp %d phase %d: block %d rows %d..%d\n", name, i, ph, t, r0, r1);
                return false;
            }
            ++pieces;
            for (int r = r0; r <= r1; ++r) {
                if (seen[(size_t)t * ny + r]++) {
                    std::printf("%s: row %d of block %d marched twice\n", name, r, t);
                    return false;
                }
            }
        }
    }
    for (size_t e = 0; e < seen.size(); ++e)
        if (!seen[e]) {
            std::printf("%s: row %zu of block %zu not marched\n", name, e % ny, e / ny);
            return false;
        }
    return true;
}

int main(int argc, char** argv) {
    if ((argc - 1) % 5 != 0) return 2;
    for (int a = 1; a + 4 < argc; a += 5) {
        const int nx = std::atoi(argv[a]), ny = std::atoi(argv[a + 1]), nd = std::atoi(argv[a + 2]);
        const int warps = std::atoi(argv[a + 3]);
        const bool iso = std::atoi(argv[a + 4]) != 0;
        const shark::K1Work w = shark::k1_work(nx, ny, nd, warps, iso);
        long long pieces = 0;
        if (w.g.B != w.nbx || w.d.B != w.nbx * nd) { std::printf("block counts\n"); return 1; }
        if (!cover("gas", w.g, ny, pieces) || !cover("dust", w.d, ny, pieces)) return 1;
        const bool persistent = w.g.P > 1 || w.d.P > 1 || w.g.n + w.d.n <= warps;
        if (persistent && w.g.n + w.d.n > warps && warps >= 2) {
            std::printf("persistent schedule over one wave: %d warps of %d\n", w.g.n + w.d.n, warps);
            return 1;
        }
        std::printf("%d %d %d %d %d: warps %d + %d, pieces %lld, gas P %d m %d, dust P %d m %d\n", nx, ny, nd,
                    warps, (int)iso, w.g.n, w.d.n, pieces, w.g.P, w.g.m, w.d.P, w.d.m);
    }
    return 0;
}
