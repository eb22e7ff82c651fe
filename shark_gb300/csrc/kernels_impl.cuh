// kernels_impl.cuh -- launch wrappers, instantiated once per state precision by
// kernels_f64.cu and kernels_f32.cu.
#pragma once

#include "launch.h"
#include "step_kernels.cuh"
#include "fargo.cuh"
#include "charge.cuh"

#include <type_traits>

namespace shark {

template <typename R>
static KParams<R> make_params(const DeviceView& v) {
    const shark_gpu_config& c = *v.cfg;
    KParams<R> p;
    p.nx = v.nx; p.ny = v.ny; p.ng = v.ng; p.nx_max = v.nx_max; p.ny_max = v.ny_max; p.pitch = v.pitch;
    p.plane = v.plane;
    p.ndust = v.ndust; p.nvar = v.nvar; p.ndim = v.ndim; p.geom = c.geom; p.solver = c.solver;
    p.solverdust = c.solverdust; p.slope_type = c.slope_type; p.iso = c.iso_cs; p.setup = c.setup;
    p.flags = c.flags; p.sod_dir = c.sod_direction;
    p.gamma = c.gamma; p.cfl = c.cfl; p.smallr = c.smallr; p.smallp = c.smallp;
    p.dust_ratio_min = c.dust_ratio_min; p.box_l = c.box_l; p.rhograin = c.rhograin;
    p.si_q = c.si_q_shear; p.si_om = c.si_omega; p.si_eta = c.si_eta_stream; p.si_r0 = c.si_rad0;
    p.sod_rho_l = c.sod_rho_l; p.sod_rho_r = c.sod_rho_r; p.sod_P_l = c.sod_P_l; p.sod_P_r = c.sod_P_r;
    p.dx1 = (const R*)v.m[0]; p.dx2 = (const R*)v.m[1]; p.surf1 = (const R*)v.m[2]; p.surf2 = (const R*)v.m[3];
    p.vol = (const R*)v.m[4]; p.radc = (const R*)v.m[5]; p.xpos = (const R*)v.m[6]; p.cs = (const R*)v.m[7];
    p.sfx = (const R*)v.m[8]; p.sfy = (const R*)v.m[9]; p.irp = (const R*)v.m[10]; p.rvol = (const R*)v.m[11];
    p.fgrav = (const R*)v.m[12];
    p.etav = (const R*)v.m[13];
    p.visc = (c.flags & SHARK_FLAG_VISCOSITY) ? 1 : 0;
    p.dx1d = v.md[0]; p.dx2d = v.md[1]; p.radcd = v.md[2]; p.xposd = v.md[3]; p.csd = v.md[4];
    p.fgravd = v.md[5]; p.treld = v.md[6]; p.hsd = v.md[7]; p.vkd = v.md[8];
    p.u_init = (const R*)v.u_init;
    p.gw = v.gw;
    p.ou_nm = v.ou_nm;
    p.ou = v.ou;
    p.ou_modes = v.ou_modes;
    p.box_l_y = c.box_l_y;
    p.chg_eta = (const R*)v.chg.eta;
    p.chg_gamma_d = (const R*)v.chg.gamma_d;
    p.dK = v.dK; p.dtstop = v.dtstop; p.dsize = v.dsize; p.dstokes = v.dstokes; p.dinvts = v.dinvts;
    p.turb_rho0 = c.turb_rho0;
    p.dt = nullptr; p.dt_next = nullptr; p.status = v.status; p.coef = v.coef;
    p.dtf = v.coef + 2 * SHARK_MAX_DUST;
    p.dinvts_f = v.coef + SHARK_COEF_INVTS;
    p.f_gamma = (float)c.gamma; p.f_gm1 = (float)(c.gamma - 1.0); p.f_inv_g1 = (float)(1.0 / (c.gamma - 1.0));
    p.f_cfl = (float)c.cfl; p.f_smallr = (float)c.smallr; p.f_smallp = (float)c.smallp;
    p.f_dust_ratio_min = (float)c.dust_ratio_min;
    p.f_box_l = (float)c.box_l; p.f_half_box_l = 0.5f * (float)c.box_l;
    p.f_si_q = (float)c.si_q_shear; p.f_si_om = (float)c.si_omega;
    p.f_si_r0 = (float)c.si_rad0; p.f_si_eta = (float)c.si_eta_stream;
    p.f_rho_ref = (float)v.rho_ref;
    p.ccs = p.cfx = p.cfy = p.ceta = nullptr;
    p.ccsd = p.chsd = p.ctgt = nullptr;
    p.cgs = nullptr;
    if (v.cdisk.on) {
        p.ccs = (const R*)v.cdisk.r;
        p.cfx = p.ccs + v.plane;
        p.cfy = p.ccs + 2 * v.plane;
        p.ceta = p.ccs + 3 * v.plane;
        p.ccsd = v.cdisk.csd;
        p.chsd = v.cdisk.hsd;
        p.ctgt = v.cdisk.tgt;
        p.cgs = (R*)v.cdisk.gs;
    }
    p.u_cur = (const R*)v.u[v.cur];
    p.u_next = (R*)v.u[(v.cur + 1) % v.nbuf];
    return p;
}

template <typename R, int NS, int MODE, bool GROW = false>
static void finalize_launch(const KParams<R>& p, dim3 grid, cudaStream_t st) {
    if constexpr (std::is_same<R, float>::value) {
        if constexpr (GROW) {
            k_finalize_mixed<NS, MODE, GROW><<<grid, 256, 0, st>>>(p);
        } else {
            dim3 g = grid;
            g.x = (p.nx + K2M_THREADS - 1) / K2M_THREADS;
            k_finalize_mixed<NS, MODE, GROW><<<g, K2M_THREADS, 0, st>>>(p);
        }
    }
    else k_finalize<R, NS, MODE, GROW><<<grid, 256, 0, st>>>(p);
}

template <typename R, int MODE>
static void finalize_dispatch(const KParams<R>& p, dim3 grid, cudaStream_t st) {
    if (MODE == 0 && p.gw.on) {   // dust growth: run-time species count, growth in the epilogue
        finalize_launch<R, -1, MODE, true>(p, grid, st);
        return;
    }
    switch (p.ndust) {
        case 0: finalize_launch<R, 0, MODE>(p, grid, st); break;
        case 1: finalize_launch<R, 1, MODE>(p, grid, st); break;
        case 2: finalize_launch<R, 2, MODE>(p, grid, st); break;
        case 4: finalize_launch<R, 4, MODE>(p, grid, st); break;
        case 8: finalize_launch<R, 8, MODE>(p, grid, st); break;
        case 16: finalize_launch<R, 16, MODE>(p, grid, st); break;
        default: finalize_launch<R, -1, MODE>(p, grid, st); break;
    }
}

// The Cartesian disk's zero_gradients (boundary_types.f90:48-100) as written, first call, on an
// uploaded state: its sources are the cells numbered first_active_y, last_active_y,
// first_active and last_active, i.e. cells (2, 0), (ny + 1, 0), (2, 0) and (nx + 1, 0) of the
// first ghost row (0-based; ny <= nx is validated).  The loops fill the y ghosts of the active
// columns column by column (bottom from cell (2, 0), top from cell (ny + 1, 0)), then the x
// ghosts of every row from cells (2, 0) and (nx + 1, 0).  Cell (ny + 1, 0) is itself the bottom
// ghost of column ny + 1 and takes cell (2, 0)'s state when the loop reaches that column, so the
// top ghosts of the active columns left of column ny + 1 keep its uploaded state and every other
// ghost takes cell (2, 0)'s.  From the second call on every ghost takes cell (2, 0)'s state, which
// no step changes: k_finalize writes it (fill_ghost_images).
template <typename R>
__global__ void k_cdisk_snapshot(KParams<R> p, const R* u) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= p.nvar) return;
    p.cgs[v] = u[uidx(p, v, 0, 2)];
    p.cgs[p.nvar + v] = u[uidx(p, v, 0, p.ny + 1)];
}

template <typename R>
__global__ void k_cdisk_ghosts(KParams<R> p, R* u) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)p.nx_max * p.ny_max) return;
    const int ix = (int)(t % p.nx_max), iy = (int)(t / p.nx_max);
    const bool ax = ix >= p.ng && ix < p.ng + p.nx, ay = iy >= p.ng && iy < p.ng + p.ny;
    if (ax && ay) return;
    const int src = (ax && iy >= p.ng + p.ny && ix < p.ny + 1) ? p.nvar : 0;
    for (int v = 0; v < p.nvar; ++v) u[uidx(p, v, iy, ix)] = p.cgs[src + v];
}

// Full ghost fill of the current state (used after an upload; the steps themselves refill the
// ghosts in k_finalize).
template <typename R>
cudaError_t launch_boundaries(const DeviceView& v) {
    KParams<R> p = make_params<R>(v);
    if (v.cdisk.on) {
        R* u = (R*)v.u[v.cur];
        k_cdisk_snapshot<R><<<(v.nvar + 127) / 128, 128, 0, v.stream>>>(p, u);
        const long long n = (long long)v.nx_max * v.ny_max;
        k_cdisk_ghosts<R><<<(unsigned)((n + 255) / 256), 256, 0, v.stream>>>(p, u);
        return cudaGetLastError();
    }
    const long long n = (v.ndim == 2 ? 2LL * v.ng * v.nx_max : 0) + 2LL * v.ng * (v.ndim == 2 ? v.ny : 1);
    k_boundaries<R><<<(unsigned)((n + 255) / 256), 256, 0, v.stream>>>(p, (R*)v.u[v.cur]);
    return cudaGetLastError();
}

template <typename R, int NDIM>
static cudaError_t flux_launch(const KParams<R>& p, cudaStream_t st) {
    using T = Tile<R, NDIM>;
    const size_t smem = TileSmem<R, NDIM>::bytes;
    cudaError_t e = cudaFuncSetAttribute(k_flux<R, NDIM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((p.nx + T::TX - 1) / T::TX, NDIM == 2 ? (p.ny + T::TY - 1) / T::TY : 1, p.ndust + 1);
    k_flux<R, NDIM><<<grid, T::NT, smem, st>>>(p);
    return cudaGetLastError();
}

template <typename R, bool IS_GAS, int ST, int SOLV>
static void strip_kernel(const KParams<R>& p, dim3 grid, cudaStream_t st) {
    k_flux_strip<R, IS_GAS, ST, SOLV><<<grid, 32 * STRIP_WARPS, 0, st>>>(p);
}

template <typename R, bool IS_GAS, int ST>
static void strip_by_solver(const KParams<R>& p, dim3 grid, cudaStream_t st) {
    if constexpr (!IS_GAS) {
        if (p.solverdust == 3) {   // HLLC dust (solver_hllc_dust)
            strip_kernel<R, false, ST, 3>(p, grid, st);
            return;
        }
    }
    switch (IS_GAS ? p.solver : p.solverdust) {
        case 0: strip_kernel<R, IS_GAS, ST, 0>(p, grid, st); break;
        case 1: strip_kernel<R, IS_GAS, ST, 1>(p, grid, st); break;
        default: strip_kernel<R, IS_GAS, ST, 2>(p, grid, st); break;
    }
}

template <typename R, bool IS_GAS>
static void strip_dispatch(const KParams<R>& p, dim3 grid, cudaStream_t st) {
    switch (p.slope_type) {
        case 0: strip_by_solver<R, IS_GAS, 0>(p, grid, st); break;
        case 1: strip_by_solver<R, IS_GAS, 1>(p, grid, st); break;
        case 2: strip_by_solver<R, IS_GAS, 2>(p, grid, st); break;
        default: strip_by_solver<R, IS_GAS, 3>(p, grid, st); break;
    }
}

// 2D K1: the dust species on the main stream and the gas concurrently on the side stream
// (forked and joined with events), so the small gas grid does not run alone.
template <typename R>
static cudaError_t strip_launch(const DeviceView& v, const KParams<R>& p) {
    const int nbx = (p.nx + STRIP_UX - 1) / STRIP_UX;
    const int nstrips = (p.ny + STRIP_H - 1) / STRIP_H;
    dim3 grid(nbx, (nstrips + STRIP_WARPS - 1) / STRIP_WARPS, 1);
    if constexpr (std::is_same<R, float>::value) {
        if (p.ndust > 0 && p.geom != 2 && p.solverdust == 0 && p.ng % 2 == 0 && v.uniform && !v.cdisk.on) {
            // mixed path, uniform Cartesian grid, Huang & Bai dust: gas and dust strips in one
            // launch (K1Work: one persistent wave, or one piece per warp when the pieces fill many waves)
            const K1Work wk = k1_work(p.nx, p.ny, p.ndust, v.k1_warps, p.iso == 1);
            const dim3 g1((unsigned)((wk.g.n + wk.d.n + STRIP_WARPS - 1) / STRIP_WARPS), 1, 1), b1(32 * STRIP_WARPS, 1, 1);
            const int gs = p.solver == 0 ? 0 : p.solver == 1 ? 1 : 2;
            K1Maps maps;
            maps.gas = v.k1_gas[v.cur];
            maps.dust = v.k1_dust[v.cur];
            switch ((p.slope_type * 3 + gs) * 2 + (p.iso == 1 ? 1 : 0)) {
#define SHARK_K1M(ST, GS)                                                                                \
    case (ST * 3 + GS) * 2:                                                                              \
        k_flux_strip_mixed<ST, GS, false><<<g1, b1, K1_SMEM, v.stream>>>(maps, p, wk); break;            \
    case (ST * 3 + GS) * 2 + 1:                                                                          \
        k_flux_strip_mixed<ST, GS, true><<<g1, b1, K1_SMEM, v.stream>>>(maps, p, wk); break;
                SHARK_K1M(0, 0) SHARK_K1M(0, 1) SHARK_K1M(0, 2)
                SHARK_K1M(1, 0) SHARK_K1M(1, 1) SHARK_K1M(1, 2)
                SHARK_K1M(2, 0) SHARK_K1M(2, 1) SHARK_K1M(2, 2)
                SHARK_K1M(3, 0) SHARK_K1M(3, 1)
                case (3 * 3 + 2) * 2: k_flux_strip_mixed<3, 2, false><<<g1, b1, K1_SMEM, v.stream>>>(maps, p, wk); break;
                default: k_flux_strip_mixed<3, 2, true><<<g1, b1, K1_SMEM, v.stream>>>(maps, p, wk); break;
#undef SHARK_K1M
            }
            return cudaGetLastError();
        }
    }
    if (p.ndust > 0) {
        cudaEventRecord(v.fork, v.stream);
        cudaStreamWaitEvent(v.stream2, v.fork, 0);
        strip_dispatch<R, true>(p, grid, v.stream2);
        cudaEventRecord(v.join, v.stream2);
        dim3 gd = grid;
        gd.z = p.ndust;
        strip_dispatch<R, false>(p, gd, v.stream);
        cudaStreamWaitEvent(v.stream, v.join, 0);
    } else {
        strip_dispatch<R, true>(p, grid, v.stream);
    }
    return cudaGetLastError();
}

// K3: FARGO remap of p.u_next into `dst` (polar disk with FARGO only)
template <typename R>
static cudaError_t fargo_launch(const KParams<R>& p, R* dst, cudaStream_t st) {
    const size_t smem = Fargo<R>::smem_bytes(p.ny);
    dim3 grid((p.nx + Fargo<R>::W - 1) / Fargo<R>::W, p.nvar, 1);
    cudaError_t e = cudaSuccess;
    switch (p.slope_type) {
#define SHARK_FARGO_CASE(ST)                                                                       \
    case ST:                                                                                      \
        e = cudaFuncSetAttribute(k_fargo<R, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        if (e == cudaSuccess) k_fargo<R, ST><<<grid, Fargo<R>::THREADS, smem, st>>>(p, p.u_next, dst);  \
        break;
        SHARK_FARGO_CASE(0)
        SHARK_FARGO_CASE(1)
        SHARK_FARGO_CASE(2)
        default: SHARK_FARGO_CASE(3)
#undef SHARK_FARGO_CASE
    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_step(const DeviceView& v, int slot) {
    KParams<R> p = make_params<R>(v);
    p.dt = v.dt_slots + slot;
    p.dt_next = reinterpret_cast<unsigned long long*>(v.dt_slots + (1 - slot));
    cudaError_t e;
    // ghost cells of the current state were written by the previous step's k_finalize (or by
    // launch_boundaries after an upload)
    if (v.time_kernels) cudaEventRecord(v.ev[0], v.stream);
    k_prepare_step<<<1, SHARK_MAX_DUST, 0, v.stream>>>(p.dt_next, p.dt, p.dtstop, p.ndust,
                                                      (p.setup == SHARK_SETUP_SI && std::is_same<R, float>::value) ? 1 : 0,
                                                      p.coef, v.dt_log);
    if (v.chg.on && (e = launch_charge<R>(v)) != cudaSuccess) return e;   // charge: solve.f90:36-42
    if (v.ou_nm > 0)   // this step's forcing coefficients, from the dt on the device
        k_ou_update<<<1, 2 * v.ou_nm, 0, v.stream>>>(v.ou, v.ou_nm, p.dt, v.ou_sigma, v.ou_tcorr, v.ou_seed, v.step);
    if (v.time_kernels) cudaEventRecord(v.ev[1], v.stream);
    e = (v.ndim == 2) ? strip_launch<R>(v, p) : flux_launch<R, 1>(p, v.stream);
    if (e != cudaSuccess) return e;
    if (v.nbuf == 3) {   // fargo_scheme after source_terms (solve.f90:105), into the third buffer
        R* dst = (R*)v.u[(v.cur + 2) % 3];
        if ((e = fargo_launch<R>(p, dst, v.stream)) != cudaSuccess) return e;
        p.u_next = dst;
    }
    if (v.time_kernels) cudaEventRecord(v.ev[2], v.stream);
    dim3 g2((v.nx + 255) / 256, v.ndim == 2 ? v.ny : 1, 1);
    finalize_dispatch<R, 0>(p, g2, v.stream);
    if (v.time_kernels) cudaEventRecord(v.ev[3], v.stream);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_courant(const DeviceView& v, int slot) {
    KParams<R> p = make_params<R>(v);
    // dt-only mode reads the current state through u_next
    p.u_next = (R*)v.u[v.cur];
    p.u_cur = (const R*)v.u[v.cur];
    p.dt = v.dt_slots + slot;   // unused in MODE 1 except by the drag (disabled)
    p.dt_next = reinterpret_cast<unsigned long long*>(v.dt_slots + slot);
    k_prepare_step<<<1, 1, 0, v.stream>>>(p.dt_next, p.dt, p.dtstop, 0, 0, p.coef, nullptr);
    dim3 g2((v.nx + 255) / 256, v.ndim == 2 ? v.ny : 1, 1);
    finalize_dispatch<R, 1>(p, g2, v.stream);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_from_fortran(const DeviceView& v, const double* src_dev, void* dst) {
    const long long n = (long long)v.nx_max * v.ny_max * v.nvar;
    k_from_fortran<R><<<(unsigned)((n + 255) / 256), 256, 0, v.stream>>>(src_dev, (R*)dst, v.nx_max, v.ny_max,
                                                                          v.pitch, v.plane, v.nvar);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_to_fortran(const DeviceView& v, const void* src, double* dst_dev) {
    const long long n = (long long)v.nx_max * v.ny_max * v.nvar;
    k_to_fortran<R><<<(unsigned)((n + 255) / 256), 256, 0, v.stream>>>((const R*)src, dst_dev, v.nx_max, v.ny_max,
                                                                        v.pitch, v.plane, v.nvar);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_ctoprim(const DeviceView& v, double* q_dev, double* cs_dev) {
    KParams<R> p = make_params<R>(v);
    const long long n = (long long)v.nx_max * v.ny_max;
    k_ctoprim<R><<<(unsigned)((n + 255) / 256), 256, 0, v.stream>>>(p, (const R*)v.u[v.cur], q_dev, cs_dev);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_totals(const DeviceView& v, double* part_dev, int nblocks, double* out_dev) {
    KParams<R> p = make_params<R>(v);
    const long long nact = (long long)v.nx * (v.ndim == 2 ? v.ny : 1);
    const long long per = (nact + nblocks - 1) / nblocks;
    k_totals_stage1<R><<<nblocks, 128, 0, v.stream>>>(p, (const R*)v.u[v.cur], part_dev, per);
    k_totals_stage2<<<1, 128, 0, v.stream>>>(part_dev, nblocks, 4 * (v.ndust + 1), out_dev);
    return cudaGetLastError();
}

template <typename R>
static ChargeParams<R> charge_params(const DeviceView& v) {
    const ChargeView& c = v.chg;
    ChargeParams<R> q;
    q.u = (const R*)v.u[v.cur];
    q.plane = v.plane; q.pitch = v.pitch; q.nx_max = v.nx_max; q.ny_max = v.ny_max;
    q.ndust = v.ndust; q.nvar = v.nvar;
    q.t_per_col = c.t_per_col; q.res = c.res; q.use_seed = c.use_seed;
    q.hs = c.hs; q.trow = c.trow; q.tau = c.tau; q.alpha = c.alpha; q.l2 = c.l2; q.mkum = c.mkum; q.ak = c.ak;
    q.rtau = c.rtau; q.nfac = c.nfac; q.rmk = c.rmk; q.pl2 = c.pl2; q.tf = c.tf;
    q.unH = c.unH; q.ud = c.ud; q.ul = c.ul; q.x0 = c.x0; q.sig_att = c.sig_att;
    q.thetai = c.thetai; q.th2 = c.th2; q.th3 = c.th3; q.psi0 = c.psi0; q.eps = c.eps; q.B0 = c.B0;
    q.mu_ions = c.mu_ions; q.nitermax = c.nitermax;
    q.psi_old = c.psi_old; q.zd = (R*)c.zd; q.ni = (R*)c.ni; q.ne = (R*)c.ne; q.eta = (R*)c.eta;
    q.gamma_d = (R*)c.gamma_d; q.seed = c.seed; q.hist = c.hist; q.iters = c.iters;
    q.status = v.status;
    return q;
}

template <typename R>
cudaError_t launch_charge(const DeviceView& v) {
    const ChargeView& c = v.chg;
    ChargeParams<R> q = charge_params<R>(v);
    cudaError_t e = cudaMemsetAsync(c.hist, 0, (CHARGE_HIST + 2) * sizeof(unsigned long long), v.stream);
    if (e != cudaSuccess) return e;
    const long long n = (long long)v.nx_max * v.ny_max;
    if (c.analytical) k_charge_fujii<R><<<(unsigned)((n + 127) / 128), 128, 0, v.stream>>>(q, c.smallr, c.mu_gas, c.ul);
    else k_charge<R><<<(unsigned)((n + 127) / 128), 128, 0, v.stream>>>(q);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_charge_features(const DeviceView& v, float* feat) {
    ChargeParams<R> q = charge_params<R>(v);
    k_charge_features<R><<<(unsigned)((v.plane + 127) / 128), 128, 0, v.stream>>>(q, feat);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_charge_collect(const DeviceView& v, const float* feat, float* out, unsigned long long* count,
                                  long long cap) {
    ChargeParams<R> q = charge_params<R>(v);
    k_charge_collect<R><<<(unsigned)((v.plane + 255) / 256), 256, 0, v.stream>>>(q, feat, out, count, cap);
    return cudaGetLastError();
}

// Output streams (write_output.f90:46-296) of the active cells from ctoprim's FP64 q (Fortran
// order) and the charging outputs, in file order, each stream nact long, dust streams
// species-major: rho, v, vy, vz, P, [rhod_tot, rhod(N), sd(N), vd(N), vdy(N), vdz(N)],
// [eta_a, eta_o, eta_h, ni, ne, zd(N)].  One thread per active cell.
template <typename R>
__global__ void k_output_pack(const double* __restrict__ q, long long ncells, int nx_max, int ng, int nx, int ndim,
                              long long nact, int N, OutScale sc, const double* __restrict__ dsize, int chg,
                              const R* __restrict__ zd, const R* __restrict__ ni, const R* __restrict__ ne,
                              const R* __restrict__ eta, long long plane, int pitch, double* __restrict__ out) {
    const long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (a >= nact) return;
    const int ix = ng + (ndim == 2 ? (int)(a % nx) : (int)a);
    const int iy = ndim == 2 ? ng + (int)(a / nx) : 0;
    const long long c = (long long)iy * nx_max + ix;
    auto Q = [&](int v) { return q[(long long)v * ncells + c]; };
    long long s = 0;
    auto put = [&](double x) { out[s * nact + a] = x; ++s; };
    put(Q(0) * sc.urho);
    put(Q(1) * sc.uv);
    put(Q(2) * sc.uv);
    put(Q(3) * sc.uv);
    put(Q(4) * sc.uP);
    if (N > 0) {
        double t = 0.0;
        for (int k = 0; k < N; ++k) t = t + Q(5 + k) * sc.urho;
        put(t);
        for (int k = 0; k < N; ++k) put(Q(5 + k) * sc.urho);
        for (int k = 0; k < N; ++k) put(dsize[k] * sc.ul);
        for (int k = 0; k < N; ++k) put(Q(5 + N + k) * sc.uv);
        for (int k = 0; k < N; ++k) put(Q(5 + 2 * N + k) * sc.uv);
        for (int k = 0; k < N; ++k) put(Q(5 + 3 * N + k) * sc.uv);
    }
    if (chg) {
        const long long pc = (long long)iy * pitch + ix;
        put((double)eta[2 * plane + pc]);
        put((double)eta[pc]);
        put((double)eta[plane + pc]);
        put((double)ni[pc]);
        put((double)ne[pc]);
        for (int k = 0; k < N; ++k) put((double)zd[(long long)k * plane + pc]);
    }
}

template <typename R>
cudaError_t launch_output_pack(const DeviceView& v, const double* q, OutScale sc, double* out) {
    const long long nact = (long long)v.nx * (v.ndim == 2 ? v.ny : 1);
    const ChargeView& c = v.chg;
    k_output_pack<R><<<(unsigned)((nact + 255) / 256), 256, 0, v.stream>>>(
        q, (long long)v.nx_max * v.ny_max, v.nx_max, v.ng, v.nx, v.ndim, nact, v.ndust, sc, v.dsize, c.on ? 1 : 0,
        (const R*)c.zd, (const R*)c.ni, (const R*)c.ne, (const R*)c.eta, v.plane, v.pitch, out);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_planes_to_fortran(const DeviceView& v, const void* src, int count, double* dst_dev) {
    const long long n = (long long)v.nx_max * v.ny_max * count;
    k_to_fortran<R><<<(unsigned)((n + 255) / 256), 256, 0, v.stream>>>((const R*)src, dst_dev, v.nx_max, v.ny_max,
                                                                        v.pitch, v.plane, count);
    return cudaGetLastError();
}

template <typename R>
int k1_resident_warps(int nsm) {
    if constexpr (std::is_same<R, float>::value) {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_flux_strip_mixed<3, 2, true>, 32 * STRIP_WARPS, K1_SMEM) !=
                cudaSuccess ||
            nb < 1) {
            cudaGetLastError();
            nb = 1;
        }
        return nsm * nb * STRIP_WARPS;
    } else {
        return 0;
    }
}

#define SHARK_INSTANTIATE(R)                                                                       \
    template int k1_resident_warps<R>(int);                                                        \
    template cudaError_t launch_step<R>(const DeviceView&, int);                                   \
    template cudaError_t launch_courant<R>(const DeviceView&, int);                                \
    template cudaError_t launch_boundaries<R>(const DeviceView&);                                  \
    template cudaError_t launch_from_fortran<R>(const DeviceView&, const double*, void*);          \
    template cudaError_t launch_to_fortran<R>(const DeviceView&, const void*, double*);            \
    template cudaError_t launch_ctoprim<R>(const DeviceView&, double*, double*);                   \
    template cudaError_t launch_totals<R>(const DeviceView&, double*, int, double*);               \
    template cudaError_t launch_charge<R>(const DeviceView&);                                      \
    template cudaError_t launch_charge_features<R>(const DeviceView&, float*);                     \
    template cudaError_t launch_charge_collect<R>(const DeviceView&, const float*, float*, unsigned long long*, long long); \
    template cudaError_t launch_planes_to_fortran<R>(const DeviceView&, const void*, int, double*);                  \
    template cudaError_t launch_output_pack<R>(const DeviceView&, const double*, OutScale, double*);

}  // namespace shark
