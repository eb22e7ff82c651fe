// rows.cuh -- where the column-march strips of the mixed path (flux_strip2.cuh,
// flux_strip_gas2.cuh) read their rows of conserved values from.
//
// A strip warp covers 64 adjacent columns (two per lane) and walks its rows from top to bottom:
// row r is fetched once (it enters the three-row window of primitives) and read once more one
// iteration later (the conserved values of the row being updated).  The rows come from a
// per-warp ring of shared-memory stages filled by the tensor-memory accelerator (TmaRows): one
// lane issues one cp.async.bulk.tensor per stage (a box of 64 columns x R rows x every variable
// of the species), completion is tracked by one mbarrier per stage, and up to NST stages are in
// flight ahead of the warp.  The loads need no per-element address arithmetic or bounds clamps
// (the box's out-of-range part is filled with zeros and never used), and how many bytes a warp
// keeps in flight does not depend on its registers.
//
// Interface used by the strips: begin(), fetch(row, us) (rows in increasing order), get(row, k)
// (the row before the last fetched one), done(row) at the end of the iteration that fetched
// row + 1 and re-read row - 1, ok() (false once a wait gave up), finish().
//
// One warp may march several strips in turn through the same ring (a persistent launch): every
// strip starts its stages at slot 0, the barriers are initialised once, before the warp's first
// strip, and the phase each barrier is waited on is carried from strip to strip as one bit per
// slot (flipped after every completed wait on that slot).
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "umma.cuh"

namespace shark {

// Columns of one strip box: 32 lanes x 2.
constexpr int ROWS_BOX_X = 64;

// ------------------------------------------------------------------------------------------------
namespace tma {

__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(umma::smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Box of a 3D tensor map (x, y, variable) into shared memory, completion on `bar`.
__device__ __forceinline__ void load3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
        "[%2];" ::"r"(umma::smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(umma::smem_addr(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

// Box of a 4D tensor map (x, y, species, component).
__device__ __forceinline__ void load4d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int s, int k) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, "
        "%6}], [%2];" ::"r"(umma::smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(umma::smem_addr(bar)), "r"(x), "r"(y), "r"(s), "r"(k)
        : "memory");
}

// Polls of one mbarrier wait before the warp gives up (each poll is a try_wait, which itself
// suspends for a while): far beyond any TMA latency, so only a broken copy reaches it.
constexpr uint32_t WAIT_POLLS = 1u << 22;

}  // namespace tma

// Shared memory of one warp's ring: NST stages of NVMAX variables x R rows x 64 columns.
template <int R, int NST, int NVMAX>
struct RingSize {
    static constexpr int stage_floats = NVMAX * R * ROWS_BOX_X;
    static constexpr int ring_bytes = NST * stage_floats * 4;
    static constexpr int bar_bytes = NST * 8;
};

// Rows of NV variables through a ring of NST stages of R rows.  Stage k holds rows
// r0 + k R .. r0 + k R + R - 1 in slot k % NST, laid out [variable][row][64 columns].  sp < 0:
// the 3D gas map (x, y, variable); sp >= 0: the 4D dust map (x, y, species sp, component).
template <int NV, int R, int NST>
struct TmaRows {
    // rows row - 1 .. row + 1 are live in iteration `row`; the next stage must already be in
    // flight when its first row is fetched, and done() releases at most one stage per row
    // (checked for every strip height by a model of this protocol): R >= 2, (NST - 1) R >= 2
    static_assert(R >= 2 && (NST - 1) * R >= 2, "ring too shallow for the strip's row window");
    static constexpr int SLOT = NV * R * ROWS_BOX_X;      // floats per stage of this strip
    const CUtensorMap* map;
    float* ring;          // this warp's ring, 128-byte aligned
    uint64_t* bar;        // NST barriers
    int x0, r0, sp, lane, nstages;
    int issued, waited;   // stages of this strip issued / waited for
    uint32_t phase;       // bit i: the phase parity the next wait on barrier i waits for
    bool fresh;           // the barriers are not initialised yet (the warp's first strip)
    bool good;

    __device__ __forceinline__ void issue(int k) {
        if (lane == 0) {
            uint64_t* b = bar + (k % NST);
            float* dst = ring + (k % NST) * SLOT;
            tma::expect_tx(b, SLOT * 4);
            if (sp < 0) tma::load3d(dst, map, b, x0, r0 + k * R, 0);
            else tma::load4d(dst, map, b, x0, r0 + k * R, sp, 0);
        }
        ++issued;
    }
    // rows r0 .. r0 + nrows - 1 are the ones the strip will fetch
    __device__ __forceinline__ void setup(int nrows) {
        nstages = (nrows + R - 1) / R;
        issued = waited = 0;
        good = true;
    }
    __device__ __forceinline__ void begin() {
        if (fresh) {
            if (lane == 0) {
#pragma unroll
                for (int i = 0; i < NST; ++i) umma::mbar_init(bar + i, 1);
                umma::fence_proxy_async();
            }
        } else {
            // the previous strip's generic reads of the ring come before the copies into it
            __syncwarp();
            if (lane == 0) umma::fence_proxy_async();
        }
        __syncwarp();
        const int n0 = nstages < NST ? nstages : NST;
        for (int k = 0; k < n0; ++k) issue(k);
    }
    __device__ __forceinline__ const float* row_ptr(int row) const {
        const int j = row - r0;
        return ring + ((j / R) % NST) * SLOT + (j % R) * ROWS_BOX_X + 2 * lane;
    }
    __device__ __forceinline__ void fetch(int row, float2* us) {
        const int j = row - r0;
        if (j % R == 0) {   // first row of stage j / R: wait for its copy
            const int slot = (j / R) % NST;
            const bool w = __all_sync(0xffffffffu,
                                      umma::mbar_wait(bar + slot, (phase >> slot) & 1u, tma::WAIT_POLLS));
            good = good && w;
            if (w) {
                ++waited;
                phase ^= 1u << slot;
            }
        }
        const float* pr = row_ptr(row);
#pragma unroll
        for (int k = 0; k < NV; ++k) us[k] = *reinterpret_cast<const float2*>(pr + k * R * ROWS_BOX_X);
    }
    __device__ __forceinline__ float2 get(int row, int k) const {
        return *reinterpret_cast<const float2*>(row_ptr(row) + k * R * ROWS_BOX_X);
    }
    // after the iteration that re-read row - 1: a stage whose rows all lie at or before row - 1
    // is no longer read; refill its slot with the stage NST further on
    __device__ __forceinline__ void done(int row) {
        if (!good) return;        // a wait gave up: issue nothing more into this ring
        const int j = row - r0;   // rows r0 .. row - 1 are finished: j of them
        if (j % R == 0 && j >= R) {
            const int k = j / R - 1 + NST;
            if (k < nstages) {
                __syncwarp();
                if (lane == 0) umma::fence_proxy_async();
                issue(k);
            }
        }
    }
    __device__ __forceinline__ bool ok() const { return good; }
    // on an early exit: wait (bounded) for the copies still in flight into this warp's ring
    __device__ __forceinline__ void finish() {
        for (int k = waited; k < issued; ++k) {
            const int slot = k % NST;
            (void)umma::mbar_wait(bar + slot, (phase >> slot) & 1u, tma::WAIT_POLLS);
            phase ^= 1u << slot;
        }
        waited = issued;
    }
};

}  // namespace shark
