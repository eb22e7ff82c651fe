// fargo.cuh -- K3: the FARGO orbital remap (src/solver/fargo_scheme.f90:2-81) of the polar disk.
//
// After the conservative update every ring (fixed radius, all phi) is shifted by vk*dt: the shift
// splits into whole cells nshft and a fraction eps of a cell, and each cell's new value is the
// linear remap of its two donor cells plus their limited-slope correction.  The remap is a
// rotation of the ring, so it cannot run in place: the kernel reads the flux kernel's output and
// writes a third state buffer.
//
// One CTA per (W adjacent columns, one conserved variable): the W rings of that variable are
// staged in shared memory whole (W = 16 FP32 / 8 FP64 columns = 64-byte row segments, ny*64 bytes),
// each output cell then reads its four donor values (two cells and their neighbours for the
// slopes) from shared memory at the column's own offset.  Row-major [phi][W] staging keeps the
// 32 lanes of a warp on distinct banks: lanes of one column sit on adjacent rows.
// The per-column shift is computed in FP64 from the FP64 metrics in both precisions.
//
// Restated with the defects of the reference fixed (the oracle does the same):
//   `one` is 1 and `eps` FP64 (an undeclared uninitialised REAL and an implicit REAL*4 there);
//   slopes exist for every active cell, with the ring's periodic wrap;
//   donor rows wrap modulo ny (the reference wraps once).
#pragma once

#include "step_kernels.cuh"

namespace shark {

template <typename R> struct Fargo {
    static constexpr int W = sizeof(R) == 4 ? 16 : 8;   // columns per CTA: 64-byte row segments
    static constexpr int THREADS = 256;
    static size_t smem_bytes(int ny) { return (size_t)ny * W * sizeof(R); }
};
// largest ring that fits the shared memory of one CTA (checked at init)
constexpr size_t FARGO_MAX_SMEM = 200 * 1024;

template <typename R, int ST>
__global__ void __launch_bounds__(256) k_fargo(KParams<R> p, const R* __restrict__ src, R* __restrict__ dst) {
    constexpr int W = Fargo<R>::W;
    extern __shared__ __align__(16) unsigned char fargo_smem[];
    R* ring = reinterpret_cast<R*>(fargo_smem);
    __shared__ int s_off[W];
    __shared__ R s_w0[W], s_w1[W], s_c1[W], s_c2[W];
    const int ny = p.ny, ng = p.ng, nxa = p.ng + p.nx;
    const int x0 = ng + blockIdx.x * W;
    const long long vb = (long long)blockIdx.y * p.plane;
    if (threadIdx.x < W) {
        const int c = threadIdx.x, gx = x0 + c;
        long long off = 0;
        R w0 = R(1), w1 = R(0), c1 = R(0), c2 = R(0);
        if (gx < nxa) {
            const double one = 1.0, half = 0.5, forth = 0.25;
            const double vk = p.vkd[gx];
            const double dy_loc = p.dx2d[gx] * p.radcd[gx];
            const double shift = fabs(vk * (*p.dt));
            const double ns = shift / dy_loc;
            const long long nshft = ns < 9.0e18 ? (long long)ns : 0;
            const double eps = fmod(shift, dy_loc) / dy_loc;
            if (vk > 0.0) { off = -(nshft % ny) - 1; w0 = R(eps); w1 = R(one - eps); }
            else { off = nshft % ny; w0 = R(one - eps); w1 = R(eps); }
            if (off < 0) off += ny;
            c1 = R(forth - (half - eps) * (half - eps));
            c2 = R((half - eps) * (half - eps) - forth);
        }
        s_off[c] = (int)off; s_w0[c] = w0; s_w1[c] = w1; s_c1[c] = c1; s_c2[c] = c2;
    }
    const int n = ny * W;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int a = i / W, c = i - a * W, gx = x0 + c;
        ring[i] = gx < nxa ? src[vb + (long long)(ng + a) * p.pitch + gx] : R(0);
    }
    __syncthreads();
    const R half = R(0.5);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int a = i / W, c = i - a * W, gx = x0 + c;
        if (gx >= nxa) continue;
        int j = a + s_off[c];
        if (j >= ny) j -= ny;
        const int jm = j == 0 ? ny - 1 : j - 1;
        const int jp = j + 1 == ny ? 0 : j + 1;
        const int jpp = jp + 1 == ny ? 0 : jp + 1;
        const R um = ring[jm * W + c], u0 = ring[j * W + c], u1 = ring[jp * W + c], u2 = ring[jpp * W + c];
        const R du0 = slope_limit_t<ST, R>(u0 - um, u1 - u0);
        const R du1 = slope_limit_t<ST, R>(u1 - u0, u2 - u1);
        R un = u0 * s_w0[c] + u1 * s_w1[c];
        un = un + half * du0 * s_c1[c] + half * du1 * s_c2[c];
        dst[vb + (long long)(ng + a) * p.pitch + gx] = un;
    }
}

}  // namespace shark
