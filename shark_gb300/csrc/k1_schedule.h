// k1_schedule.h -- which rows of which column blocks each warp of the mixed path's one-launch flux
// kernel (k_flux_strip_mixed, flux_strip2.cuh) marches.  Host code (k1_work, called per launch) and
// the decode of one warp's pieces (k1_piece, called by the kernel); no CUDA types, so that a host
// program can check the coverage of every schedule.
#pragma once

#include <algorithm>

#if defined(__CUDACC__)
#define SHARK_K1_HD __host__ __device__
#else
#define SHARK_K1_HD
#endif

namespace shark {

// columns updated per warp of a strip: 32 lanes x 2 columns, lanes 0 and 31 the x halo
constexpr int K1_STRIP_UX = 60;

// Gas and dust of the mixed path's K1 in one launch.  Each class (the gas; the dust of every
// species) has B column blocks of 60 columns and ny active rows (gas: nbx blocks; dust: ndust x
// nbx blocks, species-major), cut into pieces of rows; a piece is a strip of flux_strip_gas2 /
// flux_strip_dust2 with its own two halo rows above and below.  A class's warps sweep its blocks
// in P phases of Q consecutive blocks; in a phase, every block is cut into m pieces at the same
// rows (k ny / m, k = 0 .. m), and warp i marches piece i % m of block phase Q + i / m.  So the
// warps of neighbouring column blocks pass the same rows at about the same time, and the x halo
// they share is still in L2 when the second one reads it (pieces cut at different rows in
// neighbouring blocks read the halo from DRAM again: +36 % DRAM reads on the SI box), and only
// the blocks of one phase are in flight, not every plane of a multi-GB state at once.
//
// k1_work chooses between two schedules of this form:
// * many pieces (at least K1_WAVES waves of 32-row pieces): one piece per warp, P = 1, pieces of
//   32, 64 or 128 rows (the longest that still fills K1_WAVES waves), gas warps first; the block
//   scheduler balances the load and the last wave is a small part of the launch.
// * few pieces: one wave of blocks (SMs x resident blocks), persistent warps.  The warps are split
//   between the classes and P, Q and m chosen so that every warp has about the same work: cost =
//   phases x (rows per piece + K1_PIECE_ROWS) x the class's weight per row (gas 6 isothermal or
//   8 adiabatic, dust 4),
//   K1_PIECE_ROWS standing for a piece's halo rows and its ring refill, pieces of at most
//   K1_MAX_ROWS rows unless that needs more phases and of at least K1_MIN_ROWS rows.  On the SI box
//   (1024^2, 8 species: 32-row strips are 2.13 waves) this is 14 dust pieces of 73 rows and 23 gas
//   pieces of 44.5 rows per column block, 2430 warps (K1 0.1085 -> 0.1020 ms).
// Rows reach the strips through a per-warp ring of TMA stages in dynamic shared memory (K1_R rows
// per stage, K1_NST stages; the maps of the gas and of the dust planes of this step's state), kept
// from piece to piece.
struct K1Class {
    int B, P, Q, m, n;   // column blocks, phases, blocks per phase, pieces per block, warps (Q m)
};
struct K1Work {
    int nbx;             // column blocks per species
    K1Class g, d;        // gas, dust
};
// weights per row: isothermal gas, adiabatic gas (it carries the pressure and the energy), dust
// species (measured best of 5-9 on the SI box, of 6 and 8 on the adiabatic dusty KH box)
constexpr int K1_WG_ISO = 6, K1_WG_ADI = 8, K1_WD = 4, K1_PIECE_ROWS = 4, K1_MIN_ROWS = 16, K1_MAX_ROWS = 128,
              K1_WAVES = 8;

// `warps`: the warps of one wave (SMs x resident blocks x warps per block); `iso`: the gas is
// isothermal
inline K1Work k1_work(int nx, int ny, int ndust, int warps, bool iso) {
    const int K1_WG = iso ? K1_WG_ISO : K1_WG_ADI;
    K1Work w;
    w.nbx = (nx + K1_STRIP_UX - 1) / K1_STRIP_UX;
    const int Bg = w.nbx, Bd = w.nbx * ndust;
    const int W = std::max(warps, 2);
    for (int L = 128; L >= 32; L /= 2) {
        const int m = (ny + L - 1) / L;
        if ((long long)(Bg + Bd) * m >= (long long)K1_WAVES * W) {
            w.g = K1Class{Bg, 1, Bg, m, Bg * m};
            w.d = K1Class{Bd, 1, Bd, m, Bd * m};
            return w;
        }
    }
    const int mmax = std::max(1, ny / K1_MIN_ROWS);
    auto cost = [&](int P, int m, int wt) { return (double)P * ((ny + m - 1) / m + K1_PIECE_ROWS) * wt; };
    const long long want = ((long long)Bd * ny + (long long)W * K1_MAX_ROWS - 1) / ((long long)W * K1_MAX_ROWS);
    const int Pd0 = (int)std::max(1LL, std::min<long long>(want, Bd));
    double best = 1e300;
    K1Class bg{Bg, 1, Bg, 1, Bg}, bd{Bd, Bd, 1, 1, 1};
    for (int Pd = Pd0; Pd <= std::min(Bd, Pd0 + 2); ++Pd) {
        const int Qd = (Bd + Pd - 1) / Pd;
        for (int md = 1; md <= mmax && (long long)Qd * md < W; ++md) {
            const double cd = cost(Pd, md, K1_WD);
            const int rest = W - Qd * md;
            for (int Pg = 1; Pg <= std::min(Bg, 4); ++Pg) {
                const int Qg = (Bg + Pg - 1) / Pg, mg = std::min(mmax, rest / Qg);
                if (mg < 1) continue;
                const double c = std::max(cd, cost(Pg, mg, K1_WG));
                if (c < best) {
                    best = c;
                    bg = K1Class{Bg, Pg, Qg, mg, Qg * mg};
                    bd = K1Class{Bd, Pd, Qd, md, Qd * md};
                }
            }
        }
    }
    w.g = bg;
    w.d = bd;
    return w;
}

// Piece `ph` (phase) of warp i of class c: column block t and active rows r0 .. r1 (numbered from
// 0); false when the warp has no block in that phase.
SHARK_K1_HD inline bool k1_piece(const K1Class& c, int ny, int i, int ph, int& t, int& r0, int& r1) {
    t = i / c.m + ph * c.Q;
    if (i >= c.n || t >= c.B) return false;
    const int k = i % c.m;
    r0 = k * ny / c.m;
    r1 = (k + 1) * ny / c.m - 1;
    return true;
}

}  // namespace shark
