// launch.h -- interface between the C-ABI host code (shark_gpu.cu) and the per-precision kernel
// translation units (kernels_f64.cu compiled without FMA contraction, kernels_f32.cu with it).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/shark_gpu.h"
#include "growth.cuh"

namespace shark {

// Rows per TMA stage and stages per warp of the mixed path's flux kernel (K1): each warp's ring
// holds K1_TMA_STAGES boxes of 64 columns x K1_TMA_ROWS rows x the variables of one species
// (4 x 2 measured best on the SI 1024^2 x 8 box; 2 x 3 and 2 x 4 within 4 %).
#ifndef SHARK_K1_TMA_ROWS
#define SHARK_K1_TMA_ROWS 4
#endif
#ifndef SHARK_K1_TMA_STAGES
#define SHARK_K1_TMA_STAGES 2
#endif
constexpr int K1_TMA_ROWS = SHARK_K1_TMA_ROWS;
constexpr int K1_TMA_STAGES = SHARK_K1_TMA_STAGES;

// Floats of the buffer `coef`: the per-step drag coefficients 1/(1+a_k), a_k/(1+a_k) of the
// species, the step's dt as float, then (from SHARK_COEF_INVTS, written once) 1/C_k as float.
constexpr int SHARK_COEF_INVTS = 2 * SHARK_MAX_DUST + 4;
constexpr int SHARK_COEF_FLOATS = SHARK_COEF_INVTS + SHARK_MAX_DUST;

// Charging (K5) tables, outputs and constants; see charge.cuh.
struct ChargeView {
    bool on;
    int res, use_seed, t_per_col;
    int analytical;                         // Fujii et al. per-species Newton instead of Marchand
    double smallr, mu_gas;
    const double *hs, *trow, *tau, *alpha, *l2, *mkum, *ak;
    const double *rtau, *nfac, *rmk, *pl2;  // mixed path: 1/tau [rows][N], unit_d/m_k, 1/m_k, pi l_k^2
    const float4* tf;                       // mixed path: [rows][N][2] FP32 species table
    double unH, ud, ul, x0, sig_att, thetai, th2, th3, psi0, eps, B0, mu_ions;
    int nitermax;
    double* psi_old;                        // FP64 [plane]
    void *zd, *ni, *ne, *eta, *gamma_d;     // state precision, plane layout
    const float* seed;                      // network start points [plane] or nullptr
    int32_t* iters;                         // Newton iterations per cell [plane]
    unsigned long long* hist;               // [CHARGE_HIST + 2]
};

// Device-side view of a context, shared by both precisions.  Metric arrays come in two copies:
// `m` in the state precision (flux/update) and `md` in FP64 (drag, courant).
struct DeviceView {
    int nx, ny, ng, nx_max, ny_max, pitch, ndim, nvar, ndust;
    long long plane;            // elements per variable plane
    const shark_gpu_config* cfg;
    void* u[3];                 // state buffers (float or double): 2 in rotation, 3 with FARGO
    int nbuf;                   // buffers in rotation
    int cur;                    // index of the current state
    const void* u_init;         // relaxation reference state (polar disk), state precision
    const void* m[14];          // dx1, dx2, surf1, surf2, vol, radc, xpos, cs, sfx, sfy, irp, rvol,
                                // fgrav, etav (state precision; sfx..rvol are derived tables, fgrav
                                // the radial point-mass gravity of the polar disk, etav its viscosity)
    const double* md[9];        // dx1, dx2, radc, xpos, cs, fgrav, trel, hs, vk (FP64): trel the
                                // disk relaxation time (0 outside r_relax), hs = sqrt(2 pi) H,
                                // vk the FARGO orbital velocity
    const double* dK;           // per-species constants (device)
    const double* dtstop;
    const double* dsize;
    const double* dstokes;
    const double* dinvts;       // 1/C_k with t_k = C_k / (cell factor) for the per-cell stopping times
    double* dt_slots;           // [2] dt of step n lives in slot n % 2
    double* dt_log = nullptr;   // when set, the step's preparation kernel stores the step's dt there
                                // (pinned host memory of a timed run: no copy per step)
    unsigned int* status;       // OR of SHARK_STATUS_* bits
    float* coef;                // [SHARK_COEF_FLOATS] per-step drag coefficients (mixed path), float dt
    cudaStream_t stream;
    cudaStream_t stream2;       // side stream for the gas flux kernel (forked/joined per step)
    cudaEvent_t fork, join;
    cudaEvent_t ev[4];          // timing: before boundaries, before flux, before finalize, end
    bool time_kernels;
    ChargeView chg;
    GrowthDev gw;               // dust growth (gw.on = 0: off)
    // dustyTurb Ornstein-Uhlenbeck forcing (ou_nm = 0: off)
    int ou_nm;
    double* ou;                 // [2 nm] coefficients (a_m, b_m)
    const double* ou_modes;     // [3 nm] k_x', k_y', |k'|
    double ou_sigma, ou_tcorr;
    unsigned long long ou_seed;
    long long step;             // 1-based number of the step being launched
    // mixed path, 2D: tensor maps of each state buffer for K1's TMA row staging, the gas planes
    // (x, y, variable 0..4) and the dust planes (x, y, species, component)
    CUtensorMap k1_gas[3], k1_dust[3];
    int k1_warps;               // warps of one wave of the mixed 2D K1: SMs x resident blocks x warps per block
    bool uniform;               // Cartesian grid with the same dx1, dx2, surf1, surf2, vol in every column
    bool cs_uniform;            // the same isothermal sound speed in every column
    // reference gas density of the mixed fused flux kernel: the mean active density of the first
    // uploaded state on a uniform grid with an isothermal, uniform sound speed (0 otherwise); the
    // kernel carries rho - rho_ref and c^2 (rho - rho_ref) (flux_strip_gas2.cuh)
    double rho_ref;
    // Cartesian disk per-cell tables (on = false for every other setup): FP64 cs and
    // sqrt(2 pi H); in state precision r = cs | force x | force y | viscosity (4 planes); the
    // setup_inloop targets (7 FP64 planes, rho_ana = 0 outside the buffers); the ghost state
    // gs[2 nvar] (state precision) that zero_gradients copies into the ghost cells
    struct {
        bool on = false;
        const double* csd = nullptr;
        const double* hsd = nullptr;
        const double* tgt = nullptr;
        const void* r = nullptr;
        void* gs = nullptr;
    } cdisk;
};

// Record `msg` as this thread's shark_gpu_last_error text and return `code`.
int32_t set_error(int32_t code, const char* msg);

// Index of the state a step leaves: the flux kernel writes u[(cur+1) % nbuf]; with FARGO the
// orbital remap moves that into u[(cur+2) % 3], where the finalize kernel completes the step.
inline int next_cur(const DeviceView& v) { return v.nbuf == 3 ? (v.cur + 2) % 3 : 1 - v.cur; }

// one full step on view.u[view.cur] -> view.u[next_cur(view)]; dt read from slot `slot`, next dt
// written to slot 1-slot.  Returns a cudaError_t.
template <typename R> cudaError_t launch_step(const DeviceView& v, int slot);
// warps of one wave of the mixed-precision 2D flux kernel on `nsm` SMs (resident blocks x warps per
// block x nsm; 0 for the FP64 instantiation, which has no such kernel)
template <typename R> int k1_resident_warps(int nsm);
// courant only on the current state into dt slot `slot`
template <typename R> cudaError_t launch_courant(const DeviceView& v, int slot);
template <typename R> cudaError_t launch_boundaries(const DeviceView& v);
template <typename R> cudaError_t launch_from_fortran(const DeviceView& v, const double* src_dev, void* dst);
template <typename R> cudaError_t launch_to_fortran(const DeviceView& v, const void* src, double* dst_dev);
template <typename R> cudaError_t launch_ctoprim(const DeviceView& v, double* q_dev, double* cs_dev);
template <typename R> cudaError_t launch_totals(const DeviceView& v, double* part_dev, int nblocks, double* out_dev);
// charging (K5) on the current state; resets the iteration histogram first
template <typename R> cudaError_t launch_charge(const DeviceView& v);
// network features of every cell of the current state ([plane][SHARK_MLP_NFEAT] floats)
template <typename R> cudaError_t launch_charge_features(const DeviceView& v, float* feat);
// append (features, t) of the cells the last charging call converged to a training buffer
template <typename R>
cudaError_t launch_charge_collect(const DeviceView& v, const float* feat, float* out, unsigned long long* count, long long cap);
// plane-layout array of `count` planes -> Fortran-order FP64 (ncells per plane)
template <typename R> cudaError_t launch_planes_to_fortran(const DeviceView& v, const void* src, int count, double* dst_dev);
// unit factors of the output streams: rho / rhod, velocities, pressure (unit_P, times unit_l for
// GEOM 2), grain sizes
struct OutScale {
    double urho, uv, uP, ul;
};
template <typename R> cudaError_t launch_output_pack(const DeviceView& v, const double* q, OutScale sc, double* out);

}  // namespace shark
