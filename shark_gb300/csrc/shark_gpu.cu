// shark_gpu.cu -- host side of the C ABI declared in include/shark_gpu.h.
//
// Owns the device-resident state of one run and sequences the kernels of one `solve`
// (src/solver/solve.f90:10-181).  The conserved state never leaves the GPU between steps; the
// only per-step device->host traffic is the 8-byte dt (plus the 4-byte status word) that the
// Fortran driver needs for `time = time + dt` (src/shark.f90:107).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include <cerrno>
#include <cstdlib>
#include <sys/stat.h>
#include <map>

#include "../../include/shark_gpu.h"
#include "launch.h"
#include "mlp.h"

#include <random>

namespace {

thread_local std::string g_last_error;

int32_t fail(int32_t code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int32_t fail(int32_t code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CUDA_TRY(call)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(SHARK_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                \
    } while (0)

constexpr double kPi = 3.141592653589793238462643383279;   // src/commons/phys_const.f90:14

// x**n for integer n, square-and-multiply (the evaluation gfortran uses for integer powers)
double powi(double x, int n) {
    double r = 1.0, a = x;
    unsigned b = n < 0 ? -n : n;
    for (;;) {
        if (b & 1u) r *= a;
        b >>= 1;
        if (!b) break;
        a *= a;
    }
    return n < 0 ? 1.0 / r : r;
}

}  // namespace

int32_t shark::set_error(int32_t code, const char* msg) {
    g_last_error = msg ? msg : "";
    return code;
}

struct shark_gpu_ctx {
    shark_gpu_config cfg;
    shark::DeviceView v;
    size_t elem = 8;                 // bytes per state element
    size_t state_bytes = 0;          // one buffer
    void* ubuf[3] = {nullptr, nullptr, nullptr};
    void* uinit = nullptr;           // polar disk: relaxation reference state (the first upload)
    bool have_uinit = false;
    void* metrics = nullptr;         // 13 arrays x nx_max in state precision
    double* metrics_d = nullptr;     // 9 arrays x nx_max FP64
    double* species = nullptr;       // dK | dtstop | dsize | dstokes | dinvts (5 x SHARK_MAX_DUST)
    double* dt_slots = nullptr;      // [2]
    unsigned int* status = nullptr;
    float* coef = nullptr;           // per-step drag coefficients, then the step's dt as float
    double* staging = nullptr;       // ncells*nvar FP64 (Fortran order) for uploads/downloads
    double* part = nullptr;          // totals partials
    double* tot_out = nullptr;
    double* host_ring = nullptr;     // pinned: [2] dt + [2] status (as doubles)
    cudaEvent_t ev_read[2] = {nullptr, nullptr};
    cudaEvent_t ev_time[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // charging: tables (FP64) and outputs
    double* chg_tables = nullptr;
    float* chg_tf = nullptr;         // charging: FP32 per-row species table of the mixed path
    double* chg_psi = nullptr;
    void* chg_out = nullptr;         // zd | ni | ne | eta | gamma_d in state precision
    unsigned long long* chg_hist = nullptr;
    float* chg_seed = nullptr;       // network start points (plane layout)
    int32_t* chg_iters = nullptr;    // Newton iterations per cell (plane layout)
    double* grw_d = nullptr;         // dust growth tables (FP64)
    double* ou_d = nullptr;          // forcing: modes [3 nm] | coefficients [2 nm]
    std::vector<double> ou_init;     // initial coefficients (stationary law, seeded)
    std::vector<double> out_x, out_y;   // output positions of the active cells (x / radius, y)
    int32_t* grw_i = nullptr;        // dust growth target bins | net-transfer bins
    float* grw_f = nullptr;          // dust growth net-transfer coefficients (mixed path)
    // Cartesian disk per-cell tables (plane layout): cs, sqrt(2 pi H) in FP64; cs, force x, force y,
    // viscosity in state precision; setup_inloop targets (7 FP64 planes); ghost state (2 nvar)
    double* cdisk_d = nullptr;
    void* cdisk_r = nullptr;
    double* cdisk_tgt = nullptr;
    void* cdisk_gs = nullptr;
    bool chg_cold = true;            // psi_old is zero everywhere (no charging call since reset)
    // charging network
    float* mlp_blob = nullptr;       // SHARK_MLP_NBLOB FP32
    uint8_t* mlp_packed = nullptr;   // BF16 operand packs
    float* mlp_grad = nullptr;       // SHARK_MLP_NPARAM
    float* mlp_adam = nullptr;       // m | v (2 x SHARK_MLP_NPARAM)
    int mlp_step = 0;
    bool mlp_ready = false;          // weights loaded or trained
    float* mlp_feat = nullptr;       // [plane][SHARK_MLP_NFEAT]
    float* mlp_train = nullptr;      // [cap][SHARK_MLP_NFEAT + 1] training pairs
    long long mlp_cap = 0;
    unsigned long long* mlp_count = nullptr;
    int32_t* mlp_perm = nullptr;     // [cap]
    float* mlp_scratch = nullptr;    // losses / eval inputs
    size_t mlp_scratch_n = 0;
    unsigned int* mlp_err = nullptr;
    long long nstep = 0;             // steps launched since upload
    bool uploaded = false;
    bool rho_ref_set = false;        // the mixed flux kernel's reference density is fixed at the first upload
    bool pending_read[2] = {false, false};
    int totals_blocks = 0;
    unsigned int status_seen = 0;
};

namespace {

// ---- per-column grid metrics (src/grid/grid.f90:104-240) -----------------------------------
struct Columns {
    std::vector<double> dx1, dx2, surf1, surf2, vol, radc, xpos, cs;
    // polar disk (disk_polar/setup.f90): point-mass gravity -Mstar/r^2, relaxation time t_rel
    // inside r_relax (0 elsewhere), sqrt(2 pi) H for the midplane density, FARGO velocity -Omega r
    std::vector<double> fgrav, trel, hs, vk, etav;
    // derived tables used by the mixed-precision kernels (division-free slopes and update):
    // sfx[i] = 2/(dx1[i]+dx1[i-1]), sfy[i] = 1/(dx2[i]*r_i), irp[i] = 1/r_i, rvol[i] = 1/vol[i]
    std::vector<double> sfx, sfy, irp, rvol;
};

void derive_tables(const shark_gpu_config& c, Columns& col) {
    const size_t n = col.dx1.size();
    col.sfx.assign(n, 0.0); col.sfy.assign(n, 0.0); col.irp.assign(n, 1.0); col.rvol.assign(n, 0.0);
    for (size_t i = 0; i < n; ++i) {
        const double rp = (c.geom == 2) ? col.radc[i] : 1.0;
        if (i > 0) col.sfx[i] = 2.0 / (col.dx1[i] + col.dx1[i - 1]);
        col.sfy[i] = 2.0 / (col.dx2[i] + col.dx2[i]) / rp;
        col.irp[i] = 1.0 / rp;
        col.rvol[i] = col.vol[i] != 0.0 ? 1.0 / col.vol[i] : 0.0;
    }
}

// Every column has the same spacing, face areas and volume (to 1e-12 relative): the mixed
// path's fused flux kernel then takes the grid factors as scalars.
bool uniform_columns(const Columns& col) {
    const std::vector<double>* t[] = {&col.dx1, &col.dx2, &col.surf1, &col.surf2, &col.vol};
    for (const auto* a : t) {
        const double ref = (*a)[a->size() / 2];
        for (double x : *a)
            if (!(std::fabs(x - ref) <= 1e-12 * std::fabs(ref))) return false;
    }
    return true;
}

// Positions written by the output routine (write_output.f90:46-96): position(:,1) (radii_c for
// GEOM 2) and in 2D position(:,2), active cells in cell order, with gridinit's operations
// (grid.f90:104-240): right cell edges in 1D, cell centres in 2D Cartesian, r (cos phi, sin phi)
// on the polar grids; the caller's arrays when it passed its own grid.
void output_positions(const shark_gpu_config& c, const Columns& col, int nx_max, int ny_max, std::vector<double>& x,
                      std::vector<double>& y) {
    const int ng = c.nghost, nx = c.nx, ny = c.ny;
    const bool one_d = ny <= 1;
    const long long ncells = (long long)nx_max * ny_max;
    x.clear();
    y.clear();
    for (int iy = one_d ? 0 : ng; iy < (one_d ? 1 : ng + ny); ++iy)
        for (int ix = ng; ix < ng + nx; ++ix) {
            const long long i = (long long)iy * nx_max + ix;
            if (c.position) {
                x.push_back(c.geom == 2 && c.radii_c ? c.radii_c[i] : c.position[i]);
                if (!one_d) y.push_back(c.position[ncells + i]);
                continue;
            }
            x.push_back(c.geom == 2 ? col.radc[ix] : col.xpos[ix]);
            if (one_d) continue;
            if (c.geom == 2) {
                const double phi = ((double)(float)(iy - ng) + 0.5) * 2.0 * kPi / (double)(float)ny;
                y.push_back(col.radc[ix] * std::sin(phi));
            } else {
                y.push_back(((double)(float)(iy - ng) + 0.5) * c.box_l_y / (double)(float)ny);
            }
        }
}

int32_t build_columns(const shark_gpu_config& c, int nx_max, int ny_max, Columns& col) {
    const int ng = c.nghost, nx = c.nx, ny = c.ny;
    const bool one_d = (ny == 1);
    col.dx1.assign(nx_max, 0.0); col.dx2.assign(nx_max, 1.0);
    col.surf1.assign(nx_max, 0.0); col.surf2.assign(nx_max, 0.0);
    col.vol.assign(nx_max, 0.0); col.radc.assign(nx_max, 1.0);
    col.xpos.assign(nx_max, 0.0); col.cs.assign(nx_max, c.cs0);
    const long long ncells = (long long)nx_max * ny_max;
    if (c.dx || c.surf || c.vol || c.radii_c || c.position) {
        if (!(c.dx && c.surf && c.vol && c.position))
            return fail(SHARK_ERR_INVALID_ARG, "grid metric pointers must be given together (dx, surf, vol, position)");
        const int ndim = one_d ? 1 : 2;
        const int row0 = one_d ? 0 : ng;
        for (int ix = 0; ix < nx_max; ++ix) {
            const long long i0 = (long long)row0 * nx_max + ix;
            col.dx1[ix] = c.dx[i0];
            if (ndim == 2) col.dx2[ix] = c.dx[ncells + i0];
            col.surf1[ix] = c.surf[i0];
            if (ndim == 2) col.surf2[ix] = c.surf[ncells + i0];
            col.vol[ix] = c.vol[i0];
            col.xpos[ix] = c.position[i0];
            if (c.radii_c) col.radc[ix] = c.radii_c[i0];
            // every row must agree (the reference grids depend on ix only)
            for (int iy = 0; iy < ny_max; ++iy) {
                const long long i = (long long)iy * nx_max + ix;
                bool same = c.dx[i] == col.dx1[ix] && c.surf[i] == col.surf1[ix] && c.vol[i] == col.vol[ix];
                if (ndim == 2) same = same && c.dx[ncells + i] == col.dx2[ix] && c.surf[ncells + i] == col.surf2[ix];
                if (c.radii_c) same = same && c.radii_c[i] == col.radc[ix];
                if (c.geom == 0 && ndim == 2) same = same && c.position[i] == col.xpos[ix];
                if (!same) return fail(SHARK_ERR_UNSUPPORTED, "grid metrics vary along y at ix=%d iy=%d", ix, iy);
            }
        }
    } else if (c.geom == 0) {
        const double dx = c.box_l / (double)(float)nx;
        if (one_d) {
            double acc = 0.0;
            for (int ix = 0; ix < nx_max; ++ix) {
                col.dx1[ix] = dx;
                col.vol[ix] = dx;
                col.surf1[ix] = 1.0;
                if (ix >= ng && ix < ng + nx) { acc = acc + dx; col.xpos[ix] = acc; }   // right edges
            }
        } else {
            const double dy = c.box_l_y / (double)(float)ny;
            for (int ix = 0; ix < nx_max; ++ix) {
                col.dx1[ix] = dx;
                col.dx2[ix] = dy;
                col.surf1[ix] = dx;   // the reference sets surf(:,1) = dx(:,1) (grid.f90:140)
                col.surf2[ix] = dy;
                col.vol[ix] = dx * dy;
                col.xpos[ix] = ((double)(float)(ix - ng) + 0.5) * c.box_l / (double)(float)nx;
            }
        }
    } else {   // polar face-on
        const double inner_r = c.inner_r;
        if (c.gridspace == 0) {
            for (int ix = 0; ix < nx_max; ++ix) {
                col.dx1[ix] = c.box_l / (double)(float)nx;
                col.dx2[ix] = 2.0 * kPi / (double)(float)ny;
                col.radc[ix] = inner_r + ((double)(float)(ix - ng) + 0.5) * c.box_l / (double)(float)nx;
                col.surf1[ix] = (col.radc[ix] - 0.5 * col.dx1[ix]) * (col.dx2[ix]);
                col.surf2[ix] = col.dx1[ix];
                col.vol[ix] = col.radc[ix] * col.dx1[ix] * col.dx2[ix];
                col.xpos[ix] = col.radc[ix];
            }
        } else {
            const double zeta = std::pow(c.box_l / inner_r, 1.0 / (double)(nx - 1));
            for (int ix = 0; ix < nx_max; ++ix) {
                const int k = ix - ng;
                col.radc[ix] = inner_r * 0.5 * (powi(zeta, k) + powi(zeta, k + 1));
                col.dx1[ix] = inner_r * (powi(zeta, k + 1) - powi(zeta, k));
                col.dx2[ix] = 2.0 * kPi / (double)(float)ny;
                col.surf1[ix] = inner_r * (powi(zeta, k)) * (col.dx2[ix]);
                col.surf2[ix] = col.dx1[ix];
                col.vol[ix] = col.radc[ix] * col.dx1[ix] * col.dx2[ix];
            }
            for (int g = 0; g < ng; ++g) {
                col.radc[g] = inner_r * 0.5;
                col.radc[nx_max - 1 - g] = c.box_l + 0.5 * col.dx1[ng + nx - 1];
                col.dx1[g] = col.dx1[ng];
                col.dx1[nx_max - 1 - g] = col.dx1[ng + nx - 1];
            }
            for (int ix = 0; ix < nx_max; ++ix) col.xpos[ix] = col.radc[ix];
        }
    }
    col.fgrav.assign(nx_max, 0.0); col.trel.assign(nx_max, 0.0);
    col.hs.assign(nx_max, 0.0); col.vk.assign(nx_max, 0.0); col.etav.assign(nx_max, 0.0);
    if (c.setup == SHARK_SETUP_DISK_POLAR) {
        const double M = c.disk_mstar, tw = c.disk_n_rel * 2.0 * kPi;
        for (int ix = 0; ix < nx_max; ++ix) {
            const double r = col.radc[ix];
            // aspect ratio h(r) = hoverr r^((T slope + 1)/2): the reference's constant h for slope -1
            const double H = c.disk_hoverr * std::pow(r, 0.5 * (c.disk_temp_slope + 1.0)) * r;
            col.cs[ix] = std::sqrt(M / (r * r * r)) * H;                          // Omega H
            col.fgrav[ix] = -M / (r * r);                                         // setup.f90:362
            col.hs[ix] = std::sqrt(2.0 * kPi) * H;
            col.etav[ix] = c.disk_alpha_visc * H * col.cs[ix];                     // setup.f90:67
            if (c.flags & SHARK_FLAG_FARGO) col.vk[ix] = -std::sqrt(M / powi(r, 3)) * r;   // setup.f90:33-36
            const bool act = ix >= ng && ix < ng + nx;
            if (act && r < c.disk_r_relax)                                        // setup.f90:226
                col.trel[ix] = tw / (std::sqrt(M / powi(r, 3))) - tw / (std::sqrt(M / powi(c.inner_r, 3)));
        }
    }
    if (c.iso_cs == 1 && c.cs) {
        for (int ix = 0; ix < nx_max; ++ix) col.cs[ix] = c.cs[(one_d ? 0 : (long long)ng * nx_max) + ix];
        for (long long i = 0; i < ncells; ++i)
            if (c.cs[i] != col.cs[i % nx_max]) return fail(SHARK_ERR_UNSUPPORTED, "cs varies along y");
    }
    return SHARK_OK;
}

// Cartesian disk (disk/setup.f90) per-cell tables over every cell of the plane layout, with the
// operations of the setup loop, update_force_setup and setup_inloop: sound speed HoverR
// sqrt(Mstar/rr), sqrt(2 pi H) (H = HoverR rr), viscosity alpha H cs, the star's softened force on
// the active cells (ghosts 0), and for the active cells of the buffers (rr < buffer_in box_l or
// rr > buffer_out box_l) the state setup_inloop resets them to with its rate 0 (rho_ana, m_x, m_y,
// the energy slot rho_ana cs0^2, and per dust species dust_to rho_ana, dust_to v_ana (-yy, xx)),
// rho_ana = 0 elsewhere.  rr = sqrt(xx^2 + yy^2 + smooth_r^2) from the cell centres of gridinit.
struct CdiskTables {
    std::vector<double> cs, hs, fx, fy, eta, tgt;   // tgt: 7 planes
};
void build_cdisk_tables(const shark_gpu_config& c, int nx_max, int ny_max, int pitch, long long plane, CdiskTables& t) {
    const int ng = c.nghost, nx = c.nx, ny = c.ny;
    const double M = c.disk_mstar, hr = c.disk_hoverr, sm = c.cdisk_smooth_r;
    const double R_out = c.cdisk_frac_r_disk * c.box_l;
    const double bin = c.cdisk_buffer_in * c.box_l, bout = c.cdisk_buffer_out * c.box_l;
    const double dust_to = c.dust_eps[0], rate = 0.0;
    const size_t pl = (size_t)plane;
    t.cs.assign(pl, 0.0); t.hs.assign(pl, 0.0); t.fx.assign(pl, 0.0); t.fy.assign(pl, 0.0); t.eta.assign(pl, 0.0);
    t.tgt.assign(7 * pl, 0.0);
    for (int iy = 0; iy < ny_max; ++iy)
        for (int ix = 0; ix < nx_max; ++ix) {
            const size_t e = (size_t)iy * pitch + ix;
            const double px = ((double)(float)(ix - ng) + 0.5) * c.box_l / (double)(float)nx;
            const double py = ((double)(float)(iy - ng) + 0.5) * c.box_l_y / (double)(float)ny;
            const double xx = px - 0.5 * c.box_l, yy = py - 0.5 * c.box_l_y;
            const double r_cyl = std::sqrt(xx * xx + yy * yy);
            const double rr = std::sqrt(xx * xx + yy * yy + sm * sm);
            const double H = hr * rr;
            t.cs[e] = hr * std::sqrt(M / rr);
            t.hs[e] = std::sqrt(2.0 * kPi * H);
            t.eta[e] = c.disk_alpha_visc * H * t.cs[e];
            const bool act = ix >= ng && ix < ng + nx && iy >= ng && iy < ng + ny;
            if (!act) continue;
            t.fx[e] = -M * xx / powi(rr, 3);
            t.fy[e] = -M * yy / powi(rr, 3);
            if (!(rr < bin || rr > bout)) continue;
            const double x_soft = xx * rr / r_cyl, y_soft = yy * rr / r_cyl;
            const double Omega = std::sqrt(M / powi(rr, 3));
            const double cs0 = H * Omega;
            double rho_ana = c.disk_sigma0 * (c.disk_r0 / rr);
            if (rr > R_out) rho_ana = c.disk_sigma0 * (c.disk_r0 / R_out) / 100.0;
            const double v_ana = -Omega * rho_ana;
            t.tgt[0 * pl + e] = rho_ana;
            t.tgt[1 * pl + e] = -y_soft * v_ana;
            t.tgt[2 * pl + e] = x_soft * v_ana;
            t.tgt[3 * pl + e] = (rho_ana + (rho_ana - rho_ana) * rate) * (cs0 * cs0);
            t.tgt[4 * pl + e] = dust_to * rho_ana;
            t.tgt[5 * pl + e] = -yy * v_ana * dust_to;
            t.tgt[6 * pl + e] = xx * v_ana * dust_to;
        }
}

int32_t validate(const shark_gpu_config* c) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "config is NULL");
    if (c->abi_version != SHARK_GPU_ABI_VERSION)
        return fail(SHARK_ERR_INVALID_ARG, "abi_version %d != %d", c->abi_version, SHARK_GPU_ABI_VERSION);
    if (c->nghost != 2) return fail(SHARK_ERR_UNSUPPORTED, "nghost must be 2");
    if (c->nx < 4 || c->ny < 1) return fail(SHARK_ERR_INVALID_ARG, "nx >= 4 and ny >= 1 required");
    if (c->ny > 1 && c->ny < 4) return fail(SHARK_ERR_INVALID_ARG, "2D runs need ny >= 4");
    if (c->ndust < 0 || c->ndust > SHARK_MAX_DUST) return fail(SHARK_ERR_INVALID_ARG, "ndust out of range");
    if (c->geom != 0 && c->geom != 2) return fail(SHARK_ERR_UNSUPPORTED, "geom %d not built (0, 2 only)", c->geom);
    if (c->geom == 2 && c->ny == 1) return fail(SHARK_ERR_UNSUPPORTED, "geom 2 needs ny > 1");
    if (c->solver < 0 || c->solver > 2) return fail(SHARK_ERR_INVALID_ARG, "solver must be 0..2");
    if (c->solverdust < 0 || c->solverdust > 3)
        return fail(SHARK_ERR_UNSUPPORTED, "solverdust %d not built (0 HB, 1 LLF, 2 HLL, 3 HLLC)", c->solverdust);
    // solver_hllc_dust bounds the dust signal speeds with the gas sound speeds of the face: with an
    // isothermal gas those are the cells' (per column), with an adiabatic gas they come from the
    // gas face states, which the per-species dust kernels do not form
    if (c->solverdust == 3 && c->iso_cs != 1 && c->ndust > 0)
        return fail(SHARK_ERR_UNSUPPORTED, "solverdust 3 (HLLC dust) needs an isothermal gas (iso_cs = 1)");
    if (c->slope_type < 0 || c->slope_type > 3) return fail(SHARK_ERR_INVALID_ARG, "unknown slope limiter");
    if (c->precision != SHARK_PREC_FP64 && c->precision != SHARK_PREC_MIXED)
        return fail(SHARK_ERR_INVALID_ARG, "precision must be FP64 or MIXED");
    if (c->setup < SHARK_SETUP_SOD || c->setup > SHARK_SETUP_DISK_CART)
        return fail(SHARK_ERR_UNSUPPORTED, "setup %d has no device hooks in this build", c->setup);
    const int f = c->flags;
    if (c->setup == SHARK_SETUP_KH || c->setup == SHARK_SETUP_SEDOV) {
        // both are 2D Cartesian periodic boxes on the adiabatic equation of state
        // (KH/setup.f90:17-33, sedov/setup.f90:15-33, */boundaries.f90, iso_cs = -1)
        const char* nm = c->setup == SHARK_SETUP_KH ? "KH" : "sedov";
        if (c->geom != 0 || c->ny < 4) return fail(SHARK_ERR_UNSUPPORTED, "%s is a 2D Cartesian box", nm);
        if (c->iso_cs == 1) return fail(SHARK_ERR_UNSUPPORTED, "%s is adiabatic (iso_cs < 1)", nm);
        if (f & SHARK_FLAG_FORCE_KICK)
            return fail(SHARK_ERR_UNSUPPORTED, "%s: explicit forces (force_kick) are not built", nm);
        if (c->setup == SHARK_SETUP_SEDOV && c->ndust > 0)
            return fail(SHARK_ERR_UNSUPPORTED, "sedov is a gas-only setup");
        if (c->setup == SHARK_SETUP_KH && (f & SHARK_FLAG_DRAG) && c->ndust > 0) {
            if (!(c->rhograin > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "rhograin must be > 0");
            for (int k = 0; k < c->ndust; ++k)
                if (!(c->dust_size[k] > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "dust_size[%d] must be > 0", k);
        }
    }
    if ((f & SHARK_FLAG_VISCOSITY) && c->setup != SHARK_SETUP_DISK_POLAR && c->setup != SHARK_SETUP_DISK_CART)
        return fail(SHARK_ERR_UNSUPPORTED, "viscosity: only the disks define eta_visc (disk_polar/setup.f90:67, disk/setup.f90)");
    if (c->setup == SHARK_SETUP_DISK_CART) {
        // disk/setup.f90: a 2D Cartesian isothermal box; the star's softened gravity, per-cell
        // sound speed and viscosity come from the config (no caller grid arrays)
        if (c->geom != 0 || c->ny < 4) return fail(SHARK_ERR_UNSUPPORTED, "the Cartesian disk is a 2D Cartesian box");
        if (c->iso_cs != 1) return fail(SHARK_ERR_UNSUPPORTED, "the Cartesian disk is isothermal (iso_cs 1)");
        // zero_gradients takes its sources from cells of the first row: cell ny + 2 must lie in it
        if (c->ny > c->nx) return fail(SHARK_ERR_UNSUPPORTED, "the Cartesian disk needs ny <= nx");
        if (c->dx || c->surf || c->vol || c->radii_c || c->position || c->cs)
            return fail(SHARK_ERR_UNSUPPORTED, "the Cartesian disk builds its own grid and sound speed");
        if (c->solverdust == 3) return fail(SHARK_ERR_UNSUPPORTED, "the Cartesian disk: HLLC dust is not built for a per-cell sound speed");
        if (f & (SHARK_FLAG_FARGO | SHARK_FLAG_GROWTH | SHARK_FLAG_CHARGING))
            return fail(SHARK_ERR_UNSUPPORTED, "the Cartesian disk: FARGO, growth and charging are not built");
        if (!(c->disk_mstar > 0.0) || !(c->disk_hoverr > 0.0) || !(c->cdisk_smooth_r > 0.0) || !(c->disk_r0 > 0.0) ||
            !(c->cdisk_frac_r_disk > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "disk_mstar, disk_hoverr, disk_r0, cdisk_smooth_r, cdisk_frac_r_disk must be > 0");
        if ((f & SHARK_FLAG_DRAG) && c->ndust > 0) {
            if (!(c->rhograin > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "rhograin must be > 0");
            for (int k = 0; k < c->ndust; ++k)
                if (!(c->dust_size[k] > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "dust_size[%d] must be > 0", k);
        }
    }
    if (f & SHARK_FLAG_GROWTH) {
        if (c->ndust < 1) return fail(SHARK_ERR_INVALID_ARG, "growth needs dust species");
        if (c->ndust > 32) return fail(SHARK_ERR_UNSUPPORTED, "growth is built for at most 32 dust species");
        if (c->setup != SHARK_SETUP_DISK_POLAR && c->setup != SHARK_SETUP_DUSTYTURB)
            return fail(SHARK_ERR_UNSUPPORTED, "growth needs the temperature of the polar disk or dustyTurb setup");
        if (c->grw_kernel < 0 || c->grw_kernel > 2) return fail(SHARK_ERR_INVALID_ARG, "grw_kernel must be 0, 1 or 2");
        if (!(c->grw_smin > 0.0) || !(c->grw_smax > c->grw_smin) || !(c->grw_cfl > 0.0) || !(c->mu_gas > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "growth needs 0 < grw_smin < grw_smax, grw_cfl > 0 and mu_gas > 0");
        if (c->grw_kernel == 0 && !(c->rhograin > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "rhograin must be > 0");
        if ((c->grw_mode & SHARK_GROWTH_AMBIPOLAR) &&
            (!(f & SHARK_FLAG_CHARGING) || !(c->chg_mode & SHARK_CHARGE_RESISTIVITIES)))
            return fail(SHARK_ERR_INVALID_ARG, "ambipolar growth needs charging with resistivities");
        if (c->grw_kernel == 0 && (c->grw_mode & SHARK_GROWTH_FRAGMENTATION) &&
            !(c->grw_size_mono > 0.0 && c->grw_Abr > 0.0 && c->grw_gamma_grains > 0.0 && c->grw_estar_grains > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "fragmentation needs positive monomer and binding parameters");
        for (int k = 0; k < c->ndust; ++k)
            if (!(c->dust_size[k] > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "dust_size[%d] must be > 0", k);
    }
    if (f & SHARK_FLAG_CHARGING) {
        if (c->ndust < 1) return fail(SHARK_ERR_INVALID_ARG, "charging needs dust species");
        if (c->setup != SHARK_SETUP_DISK_POLAR && c->setup != SHARK_SETUP_DUSTYTURB)
            return fail(SHARK_ERR_UNSUPPORTED, "charging needs the cgs map of the polar disk or dustyTurb setup");
        if ((c->chg_mode & SHARK_CHARGE_ANALYTICAL) && (c->chg_mode & SHARK_CHARGE_MLP_SEED))
            return fail(SHARK_ERR_INVALID_ARG, "the network seeds the Marchand iteration, not the analytical one");
        if (!(c->chg_x > 0.0) || !(c->chg_mu_ions > 0.0) || !(c->chg_stick_el > 0.0) || !(c->chg_eps > 0.0) ||
            c->chg_nitermax < 1 || !(c->mu_gas > 0.0) || !(c->rhograin > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "charging parameters must be positive");
        if (c->setup == SHARK_SETUP_DUSTYTURB && !(c->T_cloud > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "T_cloud must be > 0");
        for (int k = 0; k < c->ndust; ++k)
            if (!(c->dust_size[k] > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "dust_size[%d] must be > 0", k);
    }
    if (c->setup == SHARK_SETUP_DUSTYTURB && c->turb_mach > 0.0) {
        if (c->ny < 4) return fail(SHARK_ERR_UNSUPPORTED, "the 2D turbulence forcing needs a 2D box");
        if (!(c->turb_tcorr > 0.0) || c->turb_kmin < 1 || c->turb_kmax < c->turb_kmin || c->turb_kmax > 8 || !(c->cs0 > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "forcing needs turb_tcorr > 0, 1 <= turb_kmin <= turb_kmax <= 8, cs0 > 0");
    }
    if (c->setup == SHARK_SETUP_DUSTYTURB) {
        if (c->geom != 0) return fail(SHARK_ERR_UNSUPPORTED, "dustyTurb is Cartesian");
        if (c->iso_cs != 1) return fail(SHARK_ERR_UNSUPPORTED, "dustyTurb is isothermal (iso_cs 1)");
        if ((f & SHARK_FLAG_DRAG) && c->ndust > 0 && !(c->turb_rho0 > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "turb_rho0 must be > 0");
        for (int k = 0; k < c->ndust; ++k)
            if ((f & SHARK_FLAG_DRAG) && !(c->dust_stokes[k] > 0.0))
                return fail(SHARK_ERR_INVALID_ARG, "dust_stokes[%d] must be > 0", k);
    }
    if (c->setup == SHARK_SETUP_DISK_POLAR) {
        if (c->geom != 2) return fail(SHARK_ERR_UNSUPPORTED, "the polar disk needs geom 2");
        if (c->iso_cs != 1) return fail(SHARK_ERR_UNSUPPORTED, "the polar disk is isothermal (iso_cs 1)");
        if (!(c->disk_mstar > 0.0) || !(c->disk_hoverr > 0.0) || !(c->inner_r > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "disk_mstar, disk_hoverr and inner_r must be > 0");
        if (c->disk_r_relax > c->inner_r && !(c->disk_n_rel > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "disk_n_rel must be > 0 when disk_r_relax > inner_r");
        if ((f & SHARK_FLAG_DRAG) && c->ndust > 0 && !(c->rhograin > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "rhograin must be > 0");
    }
    if (f & SHARK_FLAG_FARGO) {
        // the orbital velocity is defined by the disk setups only (allocate_init.f90:109-111)
        if (c->setup != SHARK_SETUP_DISK_POLAR)
            return fail(SHARK_ERR_UNSUPPORTED, "FARGO needs the polar disk setup");
        const size_t ring = (size_t)c->ny * (c->precision == SHARK_PREC_MIXED ? 16 * 4 : 8 * 8);
        if (ring > 200 * 1024)
            return fail(SHARK_ERR_UNSUPPORTED, "FARGO ring of %d cells exceeds one CTA's shared memory", c->ny);
    }
    if (c->setup == SHARK_SETUP_SI && c->ndust > 0 && !(f & SHARK_FLAG_DRAG) && (f & SHARK_FLAG_FORCE_KICK))
        return fail(SHARK_ERR_UNSUPPORTED, "SI explicit drag forces (drag=.false.) are not built");
    if (!(c->gamma > 1.0) || !(c->cfl > 0.0)) return fail(SHARK_ERR_INVALID_ARG, "gamma > 1 and cfl > 0 required");
    for (int k = 0; k < c->ndust; ++k) {
        if (c->setup == SHARK_SETUP_SI && (f & SHARK_FLAG_DRAG) && !(c->dust_tstop[k] > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "dust_tstop[%d] must be > 0", k);
        if (c->setup == SHARK_SETUP_DUSTYWAVE && (f & SHARK_FLAG_DRAG) && !(c->dust_K[k] > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "dust_K[%d] must be > 0", k);
        if (c->setup == SHARK_SETUP_DISK_POLAR && (f & SHARK_FLAG_DRAG) && !(c->dust_size[k] > 0.0))
            return fail(SHARK_ERR_INVALID_ARG, "dust_size[%d] must be > 0", k);
    }
    return SHARK_OK;
}

// ---- charging tables (src/chemistry/ionisation.f90:4-214, phys_const.f90:5-13) ----------------
constexpr double kEl = 4.8e-10, kMel = 9.109e-28, kMH = 1.67e-24, kKB = 1.38e-16;
double unit1(double u) { return u != 0.0 ? u : 1.0; }

// start point of the reference's Newton (ionisation.f90:33-52)
double charge_psi0(double thetai) {
    const double epsone = 0.99999;
    double psi0 = -2.5, conv = 1e4;
    int n = 0;
    while (conv > 1e-6 && n < 1000) {
        double psi = psi0;
        const double f = (1.0 - psi) / (epsone * thetai) * std::exp(-psi) - 1.0;
        const double df = -std::exp(-psi) / (epsone * thetai) - (1.0 - psi) / (epsone * thetai) * std::exp(-psi);
        psi = psi - f / df;
        conv = std::fabs(f);
        n = n + 1;
        psi0 = psi;
    }
    return psi0;
}

// Host tables of the charging kernel: [hs | trow | tau | alpha | l2 | mkum | ak] and the
// constants of the view.  Temperature rows: one per column for the polar disk (T from the
// isothermal cs through cs_eos), one row (T_cloud) for dustyTurb.
void build_charge_tables(const shark_gpu_config& c, const Columns& col, int nx_max, std::vector<double>& h,
                         shark::ChargeView& cv, size_t off[11]) {
    const int N = c.ndust;
    const double ul = unit1(c.unit_l), ud = unit1(c.unit_d), ut = unit1(c.unit_t);
    const double um = ul * ul * ul * ud, uv = ul / ut;
    const bool disk = c.setup == SHARK_SETUP_DISK_POLAR;
    const int rows = disk ? nx_max : 1;
    off[0] = 0;                               // hs
    off[1] = off[0] + nx_max;                 // trow
    off[2] = off[1] + (size_t)rows * 8;       // tau
    off[3] = off[2] + (size_t)rows * N;       // alpha
    off[4] = off[3] + (size_t)rows * N;       // l2
    off[5] = off[4] + N;                      // mkum
    off[6] = off[5] + N;                      // ak
    off[7] = off[6] + N;                      // rtau: 1/tau (mixed path)
    off[8] = off[7] + (size_t)rows * N;       // nfac: unit_d / m_k (g), grain number per unit of rho_k
    off[9] = off[8] + N;                      // rmk: 1/m_k (g)
    off[10] = off[9] + N;                     // pl2: pi l_k^2
    h.assign(off[10] + N, 0.0);
    for (int ix = 0; ix < nx_max; ++ix) h[off[0] + ix] = disk ? col.hs[ix] : 1.0;
    const double mu = c.chg_mu_ions;
    const double as_He_ions = (double)1.14f, as_He_el = (double)1.16f;   // REAL*4 literals
    for (int r = 0; r < rows; ++r) {
        double T = c.T_cloud;
        if (disk) {
            const double csc = col.cs[r] * uv;
            T = c.mu_gas * kMH * (csc * csc) / (c.gamma * kKB);
        }
        double* tr = &h[off[1] + (size_t)r * 8];
        tr[0] = T;
        tr[1] = (2e-7) / std::sqrt(T / 300.0);
        tr[2] = std::sqrt(8.0 * kKB * T / (kPi * mu * kMH));
        tr[3] = std::sqrt(c.gamma * kKB * T / (c.mu_gas * kMH));
        const double mu_i = 2.0 * kMH * mu * kMH / (2.0 * kMH + mu * kMH);
        const double mu_e = 2.0 * kMH * kMel / (kMel + 2.0 * kMH);
        const double vrms_i = std::sqrt(8.0 * kKB * T / (kPi * mu_i)) * 1e-5;
        const double vrms_el = std::sqrt(8.0 * kKB * T / (kPi * mu_e)) * 1e-5;
        tr[6] = 3.16e-11 * std::pow(vrms_el, 1.3);
        tr[7] = 2.4e-9 * std::pow(vrms_i, 0.6);
        tr[4] = 1.0 / as_He_el * ((kMel + 2.0 * kMH) / (2.0 * kMH)) / tr[6];
        tr[5] = 1.0 / as_He_ions * ((mu * kMH + 2.0 * kMH) / (2.0 * kMH)) / tr[7];
        for (int k = 0; k < N; ++k) {
            const double lk = c.dust_size[k] * ul;
            const double tau = lk * kKB * T / (kEl * kEl);
            h[off[2] + (size_t)r * N + k] = tau;
            h[off[3] + (size_t)r * N + k] = std::sqrt(8.0 / (kPi * tau));
            h[off[7] + (size_t)r * N + k] = 1.0 / tau;
        }
    }
    const double f43 = (double)(4.0f / 3.0f);   // Fortran 4./3. is a default-REAL quotient
    for (int k = 0; k < N; ++k) {
        const double sk = c.dust_size[k], lk = sk * ul;
        h[off[4] + k] = lk * lk;
        h[off[5] + k] = (f43 * kPi * c.rhograin * (sk * sk * sk)) * um;
        h[off[6] + k] = std::sqrt(kPi * c.gamma / 8.0) * (c.rhograin * ud) * (lk);
        h[off[8] + k] = ud / h[off[5] + k];
        h[off[9] + k] = 1.0 / h[off[5] + k];
        h[off[10] + k] = kPi * h[off[4] + k];
    }
    cv.t_per_col = disk ? 1 : 0;
    cv.analytical = (c.chg_mode & SHARK_CHARGE_ANALYTICAL) ? 1 : 0;
    cv.smallr = c.smallr;
    cv.mu_gas = c.mu_gas;
    cv.res = (c.chg_mode & SHARK_CHARGE_RESISTIVITIES) && !(c.chg_mode & SHARK_CHARGE_ANALYTICAL) ? 1 : 0;
    cv.use_seed = 0;
    cv.unH = ud / (c.mu_gas * kMH);
    cv.ud = ud;
    cv.ul = ul;
    cv.x0 = c.chg_x;
    cv.sig_att = disk ? c.chg_sigma_att : 0.0;
    cv.thetai = c.chg_stick_el * std::sqrt(mu * kMH / kMel);
    cv.th2 = cv.thetai * cv.thetai;
    cv.th3 = cv.thetai * cv.thetai * cv.thetai;
    cv.psi0 = charge_psi0(cv.thetai);
    cv.eps = c.chg_eps;
    cv.B0 = c.chg_B0;
    cv.mu_ions = mu;
    cv.nitermax = c.chg_nitermax;
}

// ---- dust growth tables (src/dust/dust_growth.f90:3-256, dust_init.f90:11-45) --------------------
// The operations follow the CPU oracle's growth_grid so the tables are bit-identical to it.
void build_growth_tables(const shark_gpu_config& c, const Columns& col, int nx_max, std::vector<double>& hd,
                         std::vector<int32_t>& hi, std::vector<float>& hf, shark::GrowthDev& g, size_t off[9]) {
    const int N = c.ndust;
    const double ul = unit1(c.unit_l), ud = unit1(c.unit_d), ut = unit1(c.unit_t);
    const double um = ul * ul * ul * ud, uv = ul / ut;
    const double rg_cgs = c.rhograin * ud;
    const double f43 = (double)(4.0f / 3.0f);
    const bool disk = c.setup == SHARK_SETUP_DISK_POLAR;
    const int rows = disk ? nx_max : 1;
    const size_t NN = (size_t)N * N;
    off[0] = 0;                  // pA
    off[1] = off[0] + NN;        // pS
    off[2] = off[1] + NN;        // pD
    off[3] = off[2] + NN;        // peps
    off[4] = off[3] + NN;        // mk
    off[5] = off[4] + N;         // sk
    off[6] = off[5] + N;         // redis
    off[7] = off[6] + NN;        // col
    off[8] = off[7] + (size_t)rows * 4;   // pK
    hd.assign(off[8] + NN, 0.0);
    hi.assign(NN * 2, 1);
    const int P = N * (N + 1) / 2;
    std::vector<int32_t> pair(P);
    std::vector<float> pKf(P), pBf(P);
    std::vector<std::vector<std::pair<int32_t, float>>> gat(N);   // gather rows of the net transfers
    const double zeta = std::pow(c.grw_smax / c.grw_smin, 1.0 / N);
    const double eta = zeta * zeta * zeta;
    const double massmin = (c.grw_kernel == 0) ? f43 * kPi * rg_cgs * (c.grw_smin * c.grw_smin * c.grw_smin) / um
                                               : c.grw_smin * c.grw_smin * c.grw_smin;
    std::vector<double> am(N), ap(N), mk(N);
    for (int k = 0; k < N; ++k) {
        am[k] = c.grw_smin * powi(zeta, k) / ul;
        ap[k] = c.grw_smin * powi(zeta, k + 1) / ul;
        const double sz = c.dust_size[k];
        mk[k] = (c.grw_kernel == 0) ? f43 * kPi * c.rhograin * (sz * sz * sz) : sz * sz * sz;
        hd[off[4] + k] = mk[k];
        hd[off[5] + k] = sz;
    }
    const double e4 = 4.0 - c.grw_slope_mono;
    for (int i = 0; i < N; ++i) {
        double* r = &hd[off[6] + (size_t)i * N];
        for (int j = 0; j <= i; ++j)
            r[j] = (std::pow(ap[j], e4) - std::pow(am[j], e4)) / (std::pow(ap[i], e4) - std::pow(am[0], e4));
        double sum = 0.0;
        for (int j = 0; j < N; ++j) sum += r[j];
        for (int j = 0; j < N; ++j) r[j] = r[j] / sum;
    }
    const double cl = c.grw_clustered;
    for (int k = 0; k < N; ++k)
        for (int j = 0; j <= k; ++j) {
            const size_t q = (size_t)k * N + j;
            const double sk = c.dust_size[k], sj = c.dust_size[j];
            hd[off[0] + q] = (cl * cl) * kPi * ((sk + sj) * (sk + sj));
            const double rate = c.grw_kernel == 1 ? 1.0 : c.grw_kernel == 2 ? (mk[k] + mk[j]) : hd[off[0] + q];
            hd[off[8] + q] = rate / mk[k] / mk[j] * mk[0];   // in grains of the smallest mass
            hd[off[1] + q] = mk[k] * um + mk[j] * um;
            hd[off[2] + q] = mk[k] * mk[j] * (um * um);
            const double mc = (1.0 - 0.0) * (mk[k] + mk[j]);
            const int b = (int)std::floor(std::log(mc / massmin) / std::log(eta) + 1);
            const int ic1 = std::max(std::min(b, N), 1), ic2 = std::max(std::min(b + 1, N), 1);
            hi[q * 2] = ic1;
            hi[q * 2 + 1] = ic2;
            double e = 1.0;
            if (ic1 < ic2) {
                const double v = (mk[ic2 - 1] - (1.0 - 0.0) * (mk[k] + mk[j])) / (mk[ic2 - 1] - mk[ic1 - 1]);
                e = v < 1.0 ? v : 1.0;
            }
            hd[off[3] + q] = e;
            // net mass change of each bin per collision (times dndt and the sticking efficiency).
            // The share of ic2 is formed directly, (M - m_ic1)/(m_ic2 - m_ic1) M, and where ic1 is
            // bin k itself its net m_j - share is formed without m_k, so nothing cancels.
            const double M = mk[k] + mk[j];
            double sh2 = 0.0;
            if (ic1 < ic2) {
                const double frac = (M - mk[ic1 - 1]) / (mk[ic2 - 1] - mk[ic1 - 1]);
                sh2 = (e < 1.0 ? frac : 0.0) * M;
            }
            double cf[4] = {0, 0, 0, 0};
            int32_t bn[4] = {-1, -1, -1, -1};
            int nb = 0;
            auto add = [&](int bin, double v) {
                for (int t = 0; t < nb; ++t)
                    if (bn[t] == bin) { cf[t] += v; return; }
                bn[nb] = bin;
                cf[nb++] = v;
            };
            if (ic1 - 1 == k && k != j) {
                add(k, mk[j] - sh2);          // -m_k + (M - sh2)
                add(j, -mk[j]);
                if (sh2 != 0.0) add(ic2 - 1, sh2);
            } else if (ic1 - 1 == k && k == j) {
                add(k, -sh2);                 // -2 m_k + (M - sh2), M = 2 m_k
                if (sh2 != 0.0) add(ic2 - 1, sh2);
            } else {
                add(k, -mk[k]);
                add(j, -mk[j]);
                add(ic1 - 1, M - sh2);
                if (sh2 != 0.0) add(ic2 - 1, sh2);
            }
            const int pq = k * (k + 1) / 2 + j;
            pair[pq] = (k << 8) | j;
            pKf[pq] = (float)hd[off[8] + q];
            pBf[pq] = (float)((8.0 * kKB / kPi) * hd[off[1] + q] / hd[off[2] + q] / (uv * uv));
            for (int t = 0; t < nb; ++t) gat[bn[t]].emplace_back(pq, (float)(cf[t] / mk[0]));   // in units of m_0
        }
    for (int r = 0; r < rows; ++r) {
        double T = c.T_cloud;
        if (disk) {
            const double csc = col.cs[r] * uv;
            T = c.mu_gas * kMH * (csc * csc) / (c.gamma * kKB);
        }
        const double cs_T = std::sqrt(c.gamma * kKB * T / (c.mu_gas * kMH));
        double* cc = &hd[off[7] + (size_t)r * 4];
        cc[0] = T;
        cc[1] = cs_T;
        cc[2] = cs_T / uv;
        cc[3] = disk ? 1.0 / std::sqrt(c.disk_mstar / powi(col.radc[r], 3)) : 0.0;
    }
    g.on = 1;
    g.kernel = c.grw_kernel;
    g.mode = c.grw_mode;
    g.t_per_col = disk ? 1 : 0;
    g.massmin = massmin;
    g.eta = eta;
    g.mref = mk[0];
    // FP32 tables: [pair | gq] in hi after the target bins, [pKf | pBf | gc] in hf; the gather
    // table is transposed (entry t of bin b at t * 32 + b) so a warp reads it in one line per t
    size_t L = 1;
    for (const auto& r : gat) L = std::max(L, r.size());
    hi.insert(hi.end(), pair.begin(), pair.end());
    const size_t gq0 = hi.size();
    hi.resize(gq0 + L * 32, 0);
    hf.assign((size_t)2 * P + L * 32, 0.0f);
    std::copy(pKf.begin(), pKf.end(), hf.begin());
    std::copy(pBf.begin(), pBf.end(), hf.begin() + P);
    for (int b = 0; b < N; ++b)
        for (size_t t = 0; t < gat[b].size(); ++t) {
            hi[gq0 + t * 32 + b] = gat[b][t].first;
            hf[(size_t)2 * P + t * 32 + b] = gat[b][t].second;
        }
    g.npair = P;
    g.gL = (int)L;
    const double a_mu = c.grw_size_mono / 2.0;
    g.Ebr_mono = c.grw_Abr * std::pow(c.grw_gamma_grains, 5.0 / 3.0) * std::pow(a_mu, 4.0 / 3.0) /
                 std::pow(c.grw_estar_grains, 2.0 / 3.0) / (uv * uv * um);
    g.m_mono = 4.0 / 3.0 * kPi * rg_cgs * (c.grw_size_mono * c.grw_size_mono * c.grw_size_mono) / um;
    g.uv = uv;
    g.uv2 = uv * uv;
    g.ud = ud;
    g.ut = ut;
    g.mu_gas = c.mu_gas;
    g.dtctl = c.grw_dtcontrol > 0.0 ? c.grw_dtcontrol * (double)365.25f * 3600 * 24 / ut : -1.0;
    g.cfl = c.grw_cfl;
    g.sticking = c.grw_sticking;
    g.eps_thr = c.grw_eps_thr;
    g.eps_thr_frag = c.grw_eps_thr_frag;
    g.delta_vambi = c.grw_delta_vambi;
    g.alpha_turb = c.grw_alpha_turb;
    g.dust_ratio_min = c.dust_ratio_min;
}

// ---- dustyTurb Ornstein-Uhlenbeck forcing (the oracle's turb_modes / turb_init, same operations) --
double hash_uniform_h(uint64_t seed, uint64_t counter) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + counter + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

void build_forcing(const shark_gpu_config& c, std::vector<double>& modes, std::vector<double>& coef, double& sigma) {
    modes.clear();
    for (int kx = 0; kx <= c.turb_kmax; ++kx)
        for (int ky = -c.turb_kmax; ky <= c.turb_kmax; ++ky) {
            if (kx == 0 && ky <= 0) continue;
            const double kk = std::sqrt((double)(kx * kx + ky * ky));
            if (kk < c.turb_kmin || kk > c.turb_kmax) continue;
            const double kxp = 2.0 * kPi * kx / c.box_l, kyp = 2.0 * kPi * ky / c.box_l_y;
            modes.push_back(kxp);
            modes.push_back(kyp);
            modes.push_back(std::sqrt(kxp * kxp + kyp * kyp));
        }
    const int nm = (int)modes.size() / 3;
    sigma = std::pow(c.turb_mach, 1.5) * (c.cs0 * c.cs0) / c.box_l / std::sqrt((double)nm);
    coef.assign(2 * nm, 0.0);
    for (int m = 0; m < nm; ++m)
        for (int q = 0; q < 2; ++q) {
            const uint64_t cnt = (uint64_t)(m * 2 + q);
            const double u1 = hash_uniform_h(c.turb_seed, 2 * cnt), u2 = hash_uniform_h(c.turb_seed, 2 * cnt + 1);
            coef[2 * m + q] = sigma * (std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(2.0 * kPi * u2));
        }
}

template <typename T>
void upload_cols(std::vector<T>& dst, const Columns& col) {
    const std::vector<double>* src[14] = {&col.dx1, &col.dx2, &col.surf1, &col.surf2, &col.vol, &col.radc,
                                          &col.xpos, &col.cs, &col.sfx, &col.sfy, &col.irp, &col.rvol, &col.fgrav,
                                          &col.etav};
    const size_t n = col.dx1.size();
    dst.resize(14 * n);
    for (int a = 0; a < 14; ++a)
        for (size_t i = 0; i < n; ++i) dst[a * n + i] = (T)(*src[a])[i];
}

int32_t release(shark_gpu_ctx* c) {
    if (!c) return SHARK_OK;
    cudaStreamSynchronize(c->stream);
    for (void* p : {c->ubuf[0], c->ubuf[1], c->ubuf[2], c->uinit, c->metrics}) if (p) cudaFree(p);
    for (double* p : {c->metrics_d, c->species, c->dt_slots, c->staging, c->part, c->tot_out}) if (p) cudaFree(p);
    if (c->status) cudaFree(c->status);
    if (c->coef) cudaFree(c->coef);
    if (c->host_ring) cudaFreeHost(c->host_ring);
    for (auto& e : c->ev_read) if (e) cudaEventDestroy(e);
    for (auto& e : c->ev_time) if (e) cudaEventDestroy(e);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->chg_tables) cudaFree(c->chg_tables);
    if (c->chg_tf) cudaFree(c->chg_tf);
    if (c->chg_psi) cudaFree(c->chg_psi);
    if (c->chg_out) cudaFree(c->chg_out);
    if (c->chg_hist) cudaFree(c->chg_hist);
    if (c->chg_seed) cudaFree(c->chg_seed);
    if (c->chg_iters) cudaFree(c->chg_iters);
    if (c->grw_d) cudaFree(c->grw_d);
    if (c->ou_d) cudaFree(c->ou_d);
    if (c->grw_i) cudaFree(c->grw_i);
    if (c->grw_f) cudaFree(c->grw_f);
    for (void* p : {(void*)c->cdisk_d, c->cdisk_r, (void*)c->cdisk_tgt, c->cdisk_gs}) if (p) cudaFree(p);
    for (void* p : {(void*)c->mlp_blob, (void*)c->mlp_packed, (void*)c->mlp_grad, (void*)c->mlp_adam,
                    (void*)c->mlp_feat, (void*)c->mlp_train, (void*)c->mlp_count, (void*)c->mlp_perm,
                    (void*)c->mlp_scratch, (void*)c->mlp_err})
        if (p) cudaFree(p);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return SHARK_OK;
}

bool is_mixed(const shark_gpu_ctx* c) { return c->cfg.precision == SHARK_PREC_MIXED; }

// cuTensorMapEncodeTiled from the driver (through the runtime's entry-point query, so the library
// does not link libcuda itself).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
    return fn;
}

// Tensor maps of K1's TMA row staging for every FP32 state buffer of a 2D context: the gas planes
// as a 3D tensor (x over the row pitch, y over ny_max rows, the 5 gas variables) and the dust
// planes as a 4D tensor (x, y, species, component: plane 5 + c N + s), boxes of 64 columns x
// K1_TMA_ROWS rows x every variable of one species.  Out-of-range parts of a box read as zeros.
int32_t encode_k1_maps(shark_gpu_ctx* c) {
    shark::DeviceView& v = c->v;
    auto enc = tensor_map_encoder();
    if (!enc) return fail(SHARK_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t pitch = (cuuint64_t)v.pitch, rows = (cuuint64_t)v.ny_max, plane = (cuuint64_t)v.plane;
    const cuuint32_t R = (cuuint32_t)shark::K1_TMA_ROWS;
    for (int b = 0; b < v.nbuf; ++b) {
        float* base = static_cast<float*>(v.u[b]);
        {
            const cuuint64_t dim[3] = {pitch, rows, 5};
            const cuuint64_t stride[2] = {pitch * 4, plane * 4};
            const cuuint32_t box[3] = {64, R, 5};
            const cuuint32_t es[3] = {1, 1, 1};
            CUresult r = enc(&v.k1_gas[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dim, stride, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return fail(SHARK_ERR_CUDA, "cuTensorMapEncodeTiled (gas planes): error %d", (int)r);
        }
        if (v.ndust > 0) {
            const cuuint64_t N = (cuuint64_t)v.ndust;
            const cuuint64_t dim[4] = {pitch, rows, N, 4};
            const cuuint64_t stride[3] = {pitch * 4, plane * 4, N * plane * 4};
            const cuuint32_t box[4] = {64, R, 1, 4};
            const cuuint32_t es[4] = {1, 1, 1, 1};
            CUresult r = enc(&v.k1_dust[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base + 5 * plane, dim, stride, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return fail(SHARK_ERR_CUDA, "cuTensorMapEncodeTiled (dust planes): error %d", (int)r);
        }
    }
    return SHARK_OK;
}

cudaError_t do_step(shark_gpu_ctx* c, int slot) {
    return is_mixed(c) ? shark::launch_step<float>(c->v, slot) : shark::launch_step<double>(c->v, slot);
}

// queue the readback of dt slot `slot` and of the status word into the pinned ring
int32_t queue_readback(shark_gpu_ctx* c, int slot) {
    CUDA_TRY(cudaMemcpyAsync(c->host_ring + slot, c->dt_slots + slot, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<unsigned int*>(c->host_ring + 2 + slot), c->status, sizeof(unsigned int),
                             cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaEventRecord(c->ev_read[slot], c->stream));
    c->pending_read[slot] = true;
    return SHARK_OK;
}

int32_t wait_readback(shark_gpu_ctx* c, int slot, double* dt, unsigned int* st) {
    if (!c->pending_read[slot]) return fail(SHARK_ERR_STATE, "no dt readback queued for slot %d", slot);
    CUDA_TRY(cudaEventSynchronize(c->ev_read[slot]));
    c->pending_read[slot] = false;
    *dt = c->host_ring[slot];
    *st = *reinterpret_cast<unsigned int*>(c->host_ring + 2 + slot);
    c->status_seen |= *st;
    return SHARK_OK;
}

// ---- charging network (mlp.cu) ------------------------------------------------------------
namespace nn {
constexpr int F = SHARK_MLP_NFEAT, KIN = 16, H = 64;
constexpr int OFF_W1 = 0, OFF_B1 = H * KIN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H, OFF_W3 = OFF_B2 + H;
constexpr int OFF_B3 = OFF_W3 + H, OFF_XMU = SHARK_MLP_NPARAM, OFF_XSD = OFF_XMU + F, OFF_TMU = OFF_XSD + F;
constexpr int OFF_TSD = OFF_TMU + 1;
}  // namespace nn

int32_t mlp_alloc(shark_gpu_ctx* c) {
    if (c->mlp_blob) return SHARK_OK;
    CUDA_TRY(cudaMalloc(&c->mlp_blob, SHARK_MLP_NBLOB * sizeof(float)));
    CUDA_TRY(cudaMalloc(&c->mlp_packed, shark::mlp_packed_bytes()));
    CUDA_TRY(cudaMalloc(&c->mlp_grad, SHARK_MLP_NPARAM * sizeof(float)));
    CUDA_TRY(cudaMalloc(&c->mlp_adam, 2 * SHARK_MLP_NPARAM * sizeof(float)));
    CUDA_TRY(cudaMalloc(&c->mlp_count, sizeof(unsigned long long)));
    CUDA_TRY(cudaMalloc(&c->mlp_err, sizeof(unsigned int)));
    CUDA_TRY(cudaMemsetAsync(c->mlp_count, 0, sizeof(unsigned long long), c->stream));
    CUDA_TRY(cudaMemsetAsync(c->mlp_err, 0, sizeof(unsigned int), c->stream));
    // Glorot-uniform initial weights from a fixed seed, zero biases, identity normalisation
    std::vector<float> b(SHARK_MLP_NBLOB, 0.0f);
    std::mt19937 rng(12345u);
    auto uni = [&](float lim) { return std::uniform_real_distribution<float>(-lim, lim)(rng); };
    const float l1 = std::sqrt(6.0f / (nn::F + nn::H)), l2 = std::sqrt(6.0f / (2 * nn::H)), l3 = std::sqrt(6.0f / (nn::H + 1));
    for (int j = 0; j < nn::H; ++j)
        for (int i = 0; i < nn::F; ++i) b[nn::OFF_W1 + j * nn::KIN + i] = uni(l1);
    for (int e = 0; e < nn::H * nn::H; ++e) b[nn::OFF_W2 + e] = uni(l2);
    for (int j = 0; j < nn::H; ++j) b[nn::OFF_W3 + j] = uni(l3);
    for (int i = 0; i < nn::F; ++i) b[nn::OFF_XSD + i] = 1.0f;
    b[nn::OFF_TSD] = 1.0f;
    CUDA_TRY(cudaMemcpy(c->mlp_blob, b.data(), b.size() * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemsetAsync(c->mlp_adam, 0, 2 * SHARK_MLP_NPARAM * sizeof(float), c->stream));
    cudaError_t e = shark::mlp_pack(c->mlp_blob, c->mlp_packed, c->stream);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "mlp pack: %s", cudaGetErrorString(e));
    c->mlp_step = 0;
    return SHARK_OK;
}

int32_t mlp_scratch(shark_gpu_ctx* c, size_t n) {
    if (c->mlp_scratch_n >= n) return SHARK_OK;
    if (c->mlp_scratch) cudaFree(c->mlp_scratch);
    c->mlp_scratch = nullptr;
    c->mlp_scratch_n = 0;
    CUDA_TRY(cudaMalloc(&c->mlp_scratch, n * sizeof(float)));
    c->mlp_scratch_n = n;
    return SHARK_OK;
}

int32_t features(shark_gpu_ctx* c) {
    if (!c->mlp_feat) CUDA_TRY(cudaMalloc(&c->mlp_feat, (size_t)c->v.plane * SHARK_MLP_NFEAT * sizeof(float)));
    cudaError_t e = is_mixed(c) ? shark::launch_charge_features<float>(c->v, c->mlp_feat)
                                : shark::launch_charge_features<double>(c->v, c->mlp_feat);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "charge features: %s", cudaGetErrorString(e));
    return SHARK_OK;
}

// Network start points for the next charging call (SHARK_CHARGE_MLP_SEED on a cold start).
int32_t seed_charges(shark_gpu_ctx* c) {
    shark::ChargeView& cv = c->v.chg;
    cv.use_seed = 0;
    cv.seed = nullptr;
    if (!(c->cfg.chg_mode & SHARK_CHARGE_MLP_SEED) || !c->chg_cold) return SHARK_OK;
    if (!c->mlp_ready) return fail(SHARK_ERR_STATE, "SHARK_CHARGE_MLP_SEED without trained or loaded weights");
    int32_t rc = features(c);
    if (rc) return rc;
    if (!c->chg_seed) CUDA_TRY(cudaMalloc(&c->chg_seed, (size_t)c->v.plane * sizeof(float)));
    shark::MlpArgs a{};
    a.feat = c->mlp_feat;
    a.feat_stride = SHARK_MLP_NFEAT;
    a.n = (int)c->v.plane;
    a.blob = c->mlp_blob;
    a.packed = c->mlp_packed;
    a.seed = c->chg_seed;
    a.psi0 = cv.psi0;
    a.err = c->mlp_err;
    cudaError_t e = shark::mlp_forward(a, c->stream);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "mlp forward: %s", cudaGetErrorString(e));
    cv.use_seed = 1;
    cv.seed = c->chg_seed;
    return SHARK_OK;
}

}  // namespace

extern "C" {

int32_t shark_gpu_abi_version(void) { return SHARK_GPU_ABI_VERSION; }

const char* shark_gpu_last_error(void) { return g_last_error.c_str(); }

int32_t shark_gpu_config_defaults(shark_gpu_config* cfg) {
    if (!cfg) return fail(SHARK_ERR_INVALID_ARG, "cfg is NULL");
    std::memset(cfg, 0, sizeof *cfg);
    cfg->abi_version = SHARK_GPU_ABI_VERSION;
    cfg->nghost = 2;
    cfg->ny = 1;
    cfg->solver = 2;
    cfg->solverdust = 0;
    cfg->slope_type = 1;
    cfg->iso_cs = -1;
    cfg->precision = SHARK_PREC_FP64;
    cfg->flags = SHARK_FLAG_DRAG | SHARK_FLAG_BACK_REACTION;
    cfg->gamma = 1.66667;
    cfg->cfl = 0.5;
    cfg->smallr = 1e-27;
    cfg->smallc = 1e-27;
    cfg->smallp = cfg->smallr * cfg->smallc * cfg->smallc;
    cfg->box_l = 1.0;
    cfg->box_l_y = 1.0;
    cfg->dust_ratio_min = 1e-11;
    cfg->rhograin = 2.7;
    cfg->unit_l = cfg->unit_d = cfg->unit_t = 1.0;
    cfg->mu_gas = 2.31;                 // setup_commons.f90 of the setups
    cfg->T_cloud = 10.0;                // dustyTurb/setup_commons.f90:18
    cfg->chg_x = 5e-17;                 // ionisation_commons.f90:73-77
    cfg->chg_mu_ions = 25.0;
    cfg->chg_stick_el = 0.5;
    cfg->chg_eps = 1e-6;
    cfg->chg_nitermax = 1000;
    cfg->chg_B0 = 3e-5;
    cfg->chg_mode = SHARK_CHARGE_RESISTIVITIES;   // res_Marchand = .true.
    cfg->grw_sticking = 1.0;            // dust_commons.f90:17-63
    cfg->grw_clustered = 1.0;
    cfg->grw_cfl = 0.1;
    cfg->grw_eps_thr = 1e-10;
    cfg->grw_eps_thr_frag = 1e-10;
    cfg->grw_dtcontrol = -1.0;
    cfg->grw_delta_vambi = 1.0;
    cfg->grw_alpha_turb = 1.5;
    cfg->grw_size_mono = 1e-5;
    cfg->grw_slope_mono = 3.5;
    cfg->grw_Abr = 2.8e3;
    cfg->grw_gamma_grains = 25.0;
    cfg->grw_estar_grains = 2.8e11;
    cfg->disk_alpha_visc = 1e-2;        // disk_polar/setup_commons.f90:21
    cfg->kh_rho_dense = 1.0;            // KH/setup_commons.f90:8-19
    cfg->kh_rho_diffuse = 0.8;
    cfg->kh_T_dense = 10.0;
    cfg->kh_mach = 0.5;
    cfg->kh_vy0 = 0.1;
    cfg->kh_kx = 10.0;
    cfg->sedov_rho_ext = 1.0;           // sedov/setup_commons.f90:9-12
    cfg->sedov_P_ext = 1e-5;
    cfg->sedov_P_cen = 1.0;
    cfg->sedov_r_expl = (double)0.1f;   // `r_expl=0.1` is a default-REAL literal
    return SHARK_OK;
}

int32_t shark_gpu_init(const shark_gpu_config* cfg, shark_gpu_ctx** out) {
    if (!out) return fail(SHARK_ERR_INVALID_ARG, "ctx_out is NULL");
    *out = nullptr;
    int32_t rc = validate(cfg);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(SHARK_ERR_NO_DEVICE, "no CUDA device");
    if (cfg->device < 0 || cfg->device >= ndev) return fail(SHARK_ERR_NO_DEVICE, "device %d not present", cfg->device);
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, cfg->device));
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(SHARK_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a only", cfg->device,
                    prop.major, prop.minor);
    CUDA_TRY(cudaSetDevice(cfg->device));

    shark_gpu_ctx* c = new (std::nothrow) shark_gpu_ctx();
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "out of host memory");
    c->cfg = *cfg;
    // the caller's grid pointers are only read here
    c->cfg.dx = c->cfg.surf = c->cfg.vol = c->cfg.radii_c = c->cfg.position = c->cfg.cs = nullptr;
    shark::DeviceView& v = c->v;
    v.cfg = &c->cfg;
    v.nx = cfg->nx; v.ny = cfg->ny; v.ng = cfg->nghost;
    v.ndim = cfg->ny == 1 ? 1 : 2;
    v.nx_max = cfg->nx + 2 * cfg->nghost;
    v.ny_max = v.ndim == 1 ? 1 : cfg->ny + 2 * cfg->nghost;
    v.ndust = cfg->ndust;
    v.nvar = 5 + 4 * cfg->ndust;
    v.pitch = (v.nx_max + 31) / 32 * 32;
    v.plane = (long long)v.pitch * v.ny_max;
    if ((double)v.plane * v.nvar >= 2147483647.0) {
        delete c;
        return fail(SHARK_ERR_UNSUPPORTED, "state of %lld elements exceeds the 2^31 element indexing of the kernels",
                    (long long)v.plane * v.nvar);
    }
    c->elem = is_mixed(c) ? 4 : 8;
    c->state_bytes = (size_t)v.plane * v.nvar * c->elem;

    Columns col;
    if ((rc = build_columns(*cfg, v.nx_max, v.ny_max, col))) { release(c); return rc; }
    output_positions(*cfg, col, v.nx_max, v.ny_max, c->out_x, c->out_y);
    derive_tables(*cfg, col);
    v.uniform = cfg->geom == 0 && v.ndim == 2 && uniform_columns(col);
    v.cs_uniform = std::all_of(col.cs.begin(), col.cs.end(), [&](double x) { return x == col.cs[0]; });
    v.rho_ref = 0.0;

#define INIT_TRY(call)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            rc = fail(SHARK_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));                   \
            release(c);                                                                           \
            return rc;                                                                            \
        }                                                                                         \
    } while (0)
    INIT_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    INIT_TRY(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
    INIT_TRY(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    INIT_TRY(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    v.stream = c->stream;
    v.stream2 = c->stream2;
    v.fork = c->ev_fork;
    v.join = c->ev_join;
    for (auto& e : c->ev_read) INIT_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto& e : c->ev_time) INIT_TRY(cudaEventCreate(&e));
    v.nbuf = (cfg->flags & SHARK_FLAG_FARGO) ? 3 : 2;
    for (int b = 0; b < v.nbuf; ++b) {
        INIT_TRY(cudaMalloc(&c->ubuf[b], c->state_bytes));
        INIT_TRY(cudaMemsetAsync(c->ubuf[b], 0, c->state_bytes, c->stream));
        v.u[b] = c->ubuf[b];
    }
    v.u[2] = c->ubuf[2];
    v.cur = 0;
    if (is_mixed(c) && v.ndim == 2 && (rc = encode_k1_maps(c))) {
        release(c);
        return rc;
    }
    if (is_mixed(c) && v.ndim == 2) {
        int nsm = 0;
        INIT_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, cfg->device));
        v.k1_warps = shark::k1_resident_warps<float>(nsm);
    }
    if (cfg->setup == SHARK_SETUP_DISK_POLAR) {
        INIT_TRY(cudaMalloc(&c->uinit, c->state_bytes));
        INIT_TRY(cudaMemsetAsync(c->uinit, 0, c->state_bytes, c->stream));
    }
    v.u_init = c->uinit;
    const size_t ncol = (size_t)v.nx_max;
    INIT_TRY(cudaMalloc(&c->metrics, 14 * ncol * c->elem));
    INIT_TRY(cudaMalloc(&c->metrics_d, 9 * ncol * sizeof(double)));
    if (is_mixed(c)) {
        std::vector<float> h;
        upload_cols(h, col);
        INIT_TRY(cudaMemcpy(c->metrics, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        std::vector<double> h;
        upload_cols(h, col);
        INIT_TRY(cudaMemcpy(c->metrics, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    for (int a = 0; a < 14; ++a) v.m[a] = (const char*)c->metrics + a * ncol * c->elem;
    {
        std::vector<double> hd(9 * ncol);
        const std::vector<double>* src[9] = {&col.dx1, &col.dx2, &col.radc, &col.xpos, &col.cs,
                                             &col.fgrav, &col.trel, &col.hs, &col.vk};
        for (int a = 0; a < 9; ++a) std::memcpy(hd.data() + a * ncol, src[a]->data(), ncol * sizeof(double));
        INIT_TRY(cudaMemcpy(c->metrics_d, hd.data(), hd.size() * sizeof(double), cudaMemcpyHostToDevice));
        for (int a = 0; a < 9; ++a) v.md[a] = c->metrics_d + a * ncol;
    }
    INIT_TRY(cudaMalloc(&c->species, 5 * SHARK_MAX_DUST * sizeof(double)));
    float invf[SHARK_MAX_DUST] = {0};   // FP32 copy of 1/C_k for the mixed path's coefficients
    {
        // 1/C_k of the stopping times t_k = C_k / F_cell that K2's mixed path multiplies out:
        // dustyTurb C_k = St_0,k L rho_0 (F = c_s rho), polar disk (Epstein on the midplane density)
        // C_k = sqrt(pi gamma/8) rho_grain s_k (F = rho/hs c_s)
        double inv[SHARK_MAX_DUST] = {0};
        for (int k = 0; k < cfg->ndust; ++k) {
            const double C = cfg->setup == SHARK_SETUP_DUSTYTURB
                                 ? cfg->dust_stokes[k] * cfg->box_l * cfg->turb_rho0
                                 : std::sqrt(kPi * cfg->gamma / 8.0) * cfg->rhograin * cfg->dust_size[k];
            inv[k] = C != 0.0 ? 1.0 / C : 0.0;
            invf[k] = (float)inv[k];
        }
        INIT_TRY(cudaMemcpy(c->species + 4 * SHARK_MAX_DUST, inv, SHARK_MAX_DUST * sizeof(double), cudaMemcpyHostToDevice));
    }
    INIT_TRY(cudaMemcpy(c->species + 3 * SHARK_MAX_DUST, cfg->dust_stokes, SHARK_MAX_DUST * sizeof(double), cudaMemcpyHostToDevice));
    INIT_TRY(cudaMemcpy(c->species, cfg->dust_K, SHARK_MAX_DUST * sizeof(double), cudaMemcpyHostToDevice));
    INIT_TRY(cudaMemcpy(c->species + SHARK_MAX_DUST, cfg->dust_tstop, SHARK_MAX_DUST * sizeof(double), cudaMemcpyHostToDevice));
    INIT_TRY(cudaMemcpy(c->species + 2 * SHARK_MAX_DUST, cfg->dust_size, SHARK_MAX_DUST * sizeof(double), cudaMemcpyHostToDevice));
    v.dK = c->species;
    v.dtstop = c->species + SHARK_MAX_DUST;
    v.dsize = c->species + 2 * SHARK_MAX_DUST;
    v.dstokes = c->species + 3 * SHARK_MAX_DUST;
    v.dinvts = c->species + 4 * SHARK_MAX_DUST;
    INIT_TRY(cudaMalloc(&c->dt_slots, 2 * sizeof(double)));
    INIT_TRY(cudaMalloc(&c->status, sizeof(unsigned int)));
    INIT_TRY(cudaMemsetAsync(c->status, 0, sizeof(unsigned int), c->stream));
    INIT_TRY(cudaMalloc(&c->coef, shark::SHARK_COEF_FLOATS * sizeof(float)));
    INIT_TRY(cudaMemsetAsync(c->coef, 0, shark::SHARK_COEF_FLOATS * sizeof(float), c->stream));
    INIT_TRY(cudaMemcpyAsync(c->coef + shark::SHARK_COEF_INVTS, invf, SHARK_MAX_DUST * sizeof(float),
                             cudaMemcpyHostToDevice, c->stream));
    v.dt_slots = c->dt_slots;
    v.status = c->status;
    v.coef = c->coef;
    v.chg = shark::ChargeView{};
    if (cfg->flags & SHARK_FLAG_CHARGING) {
        std::vector<double> h;
        size_t off[11];
        build_charge_tables(*cfg, col, v.nx_max, h, v.chg, off);
        INIT_TRY(cudaMalloc(&c->chg_tables, h.size() * sizeof(double)));
        INIT_TRY(cudaMemcpy(c->chg_tables, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        v.chg.hs = c->chg_tables + off[0]; v.chg.trow = c->chg_tables + off[1]; v.chg.tau = c->chg_tables + off[2];
        v.chg.alpha = c->chg_tables + off[3]; v.chg.l2 = c->chg_tables + off[4]; v.chg.mkum = c->chg_tables + off[5];
        v.chg.ak = c->chg_tables + off[6];
        v.chg.rtau = c->chg_tables + off[7]; v.chg.nfac = c->chg_tables + off[8];
        v.chg.rmk = c->chg_tables + off[9]; v.chg.pl2 = c->chg_tables + off[10];
        {
            // FP32 copy for the mixed path, per temperature row and species: (alpha, 1/tau,
            // pi l^2/tau, tau), (unit_d/m, pi l^2, 1/m, sqrt(pi gamma/8) rhograin l)
            const int N = cfg->ndust, rows = v.chg.t_per_col ? v.nx_max : 1;
            std::vector<float> tf((size_t)rows * N * 8);
            for (int r = 0; r < rows; ++r)
                for (int k = 0; k < N; ++k) {
                    float* e = &tf[((size_t)r * N + k) * 8];
                    const double tau = h[off[2] + (size_t)r * N + k];
                    e[0] = (float)h[off[3] + (size_t)r * N + k];
                    e[1] = (float)h[off[7] + (size_t)r * N + k];
                    e[2] = (float)(h[off[10] + k] / tau);
                    e[3] = (float)tau;
                    e[4] = (float)h[off[8] + k];
                    e[5] = (float)h[off[10] + k];
                    e[6] = (float)h[off[9] + k];
                    e[7] = (float)h[off[6] + k];
                }
            INIT_TRY(cudaMalloc(&c->chg_tf, tf.size() * sizeof(float)));
            INIT_TRY(cudaMemcpy(c->chg_tf, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice));
            v.chg.tf = reinterpret_cast<const float4*>(c->chg_tf);
        }
        const size_t pl = (size_t)v.plane;
        INIT_TRY(cudaMalloc(&c->chg_psi, pl * sizeof(double)));
        INIT_TRY(cudaMemsetAsync(c->chg_psi, 0, pl * sizeof(double), c->stream));
        const size_t nplanes = 2 * (size_t)v.ndust + 5;   // zd N | ni | ne | eta 3 | gamma_d N
        INIT_TRY(cudaMalloc(&c->chg_out, nplanes * pl * c->elem));
        INIT_TRY(cudaMemsetAsync(c->chg_out, 0, nplanes * pl * c->elem, c->stream));
        char* b = (char*)c->chg_out;
        v.chg.zd = b;
        v.chg.ni = b + (size_t)v.ndust * pl * c->elem;
        v.chg.ne = b + ((size_t)v.ndust + 1) * pl * c->elem;
        v.chg.eta = b + ((size_t)v.ndust + 2) * pl * c->elem;
        v.chg.gamma_d = b + ((size_t)v.ndust + 5) * pl * c->elem;
        v.chg.psi_old = c->chg_psi;
        INIT_TRY(cudaMalloc(&c->chg_hist, (SHARK_CHARGE_HIST + 2) * sizeof(unsigned long long)));
        INIT_TRY(cudaMemsetAsync(c->chg_hist, 0, (SHARK_CHARGE_HIST + 2) * sizeof(unsigned long long), c->stream));
        v.chg.hist = c->chg_hist;
        INIT_TRY(cudaMalloc(&c->chg_iters, pl * sizeof(int32_t)));
        INIT_TRY(cudaMemsetAsync(c->chg_iters, 0, pl * sizeof(int32_t), c->stream));
        v.chg.iters = c->chg_iters;
        v.chg.on = true;
    }
    v.ou_nm = 0;
    v.ou = nullptr;
    v.ou_modes = nullptr;
    if (cfg->setup == SHARK_SETUP_DUSTYTURB && cfg->turb_mach > 0.0) {
        std::vector<double> modes;
        double sigma;
        build_forcing(*cfg, modes, c->ou_init, sigma);
        const int nm = (int)modes.size() / 3;
        INIT_TRY(cudaMalloc(&c->ou_d, (size_t)5 * nm * sizeof(double)));
        INIT_TRY(cudaMemcpy(c->ou_d, modes.data(), modes.size() * sizeof(double), cudaMemcpyHostToDevice));
        INIT_TRY(cudaMemcpy(c->ou_d + 3 * nm, c->ou_init.data(), c->ou_init.size() * sizeof(double), cudaMemcpyHostToDevice));
        v.ou_nm = nm;
        v.ou_modes = c->ou_d;
        v.ou = c->ou_d + 3 * nm;
        v.ou_sigma = sigma;
        v.ou_tcorr = cfg->turb_tcorr;
        v.ou_seed = (unsigned long long)cfg->turb_seed;
    }
    v.gw = shark::GrowthDev{};
    if (cfg->flags & SHARK_FLAG_GROWTH) {
        std::vector<double> hd;
        std::vector<int32_t> hi;
        std::vector<float> hf;
        size_t off[9];
        build_growth_tables(*cfg, col, v.nx_max, hd, hi, hf, v.gw, off);
        INIT_TRY(cudaMalloc(&c->grw_f, hf.size() * sizeof(float)));
        INIT_TRY(cudaMemcpy(c->grw_f, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice));
        INIT_TRY(cudaMalloc(&c->grw_d, hd.size() * sizeof(double)));
        INIT_TRY(cudaMemcpy(c->grw_d, hd.data(), hd.size() * sizeof(double), cudaMemcpyHostToDevice));
        INIT_TRY(cudaMalloc(&c->grw_i, hi.size() * sizeof(int32_t)));
        INIT_TRY(cudaMemcpy(c->grw_i, hi.data(), hi.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        v.gw.pA = c->grw_d + off[0]; v.gw.pS = c->grw_d + off[1]; v.gw.pD = c->grw_d + off[2];
        v.gw.peps = c->grw_d + off[3]; v.gw.mk = c->grw_d + off[4]; v.gw.sk = c->grw_d + off[5];
        v.gw.redis = c->grw_d + off[6]; v.gw.col = c->grw_d + off[7]; v.gw.pic = c->grw_i;
        {
            const size_t NN = (size_t)cfg->ndust * cfg->ndust, P = (size_t)v.gw.npair;
            v.gw.pair = c->grw_i + NN * 2;
            v.gw.gq = c->grw_i + NN * 2 + P;
            v.gw.pKf = c->grw_f;
            v.gw.pBf = c->grw_f + P;
            v.gw.gc = c->grw_f + 2 * P;
        }
    }
    if (cfg->setup == SHARK_SETUP_DISK_CART) {
        CdiskTables t;
        build_cdisk_tables(*cfg, v.nx_max, v.ny_max, v.pitch, v.plane, t);
        const size_t pl = (size_t)v.plane;
        std::vector<double> hd(2 * pl);
        std::memcpy(hd.data(), t.cs.data(), pl * sizeof(double));
        std::memcpy(hd.data() + pl, t.hs.data(), pl * sizeof(double));
        INIT_TRY(cudaMalloc(&c->cdisk_d, hd.size() * sizeof(double)));
        INIT_TRY(cudaMemcpy(c->cdisk_d, hd.data(), hd.size() * sizeof(double), cudaMemcpyHostToDevice));
        INIT_TRY(cudaMalloc(&c->cdisk_tgt, t.tgt.size() * sizeof(double)));
        INIT_TRY(cudaMemcpy(c->cdisk_tgt, t.tgt.data(), t.tgt.size() * sizeof(double), cudaMemcpyHostToDevice));
        std::vector<double> hr(4 * pl);
        const std::vector<double>* src[4] = {&t.cs, &t.fx, &t.fy, &t.eta};
        for (int a = 0; a < 4; ++a) std::memcpy(hr.data() + a * pl, src[a]->data(), pl * sizeof(double));
        INIT_TRY(cudaMalloc(&c->cdisk_r, 4 * pl * c->elem));
        if (is_mixed(c)) {
            std::vector<float> hf(hr.begin(), hr.end());
            INIT_TRY(cudaMemcpy(c->cdisk_r, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice));
        } else {
            INIT_TRY(cudaMemcpy(c->cdisk_r, hr.data(), hr.size() * sizeof(double), cudaMemcpyHostToDevice));
        }
        INIT_TRY(cudaMalloc(&c->cdisk_gs, 2 * (size_t)v.nvar * c->elem));
        INIT_TRY(cudaMemsetAsync(c->cdisk_gs, 0, 2 * (size_t)v.nvar * c->elem, c->stream));
        v.cdisk.csd = c->cdisk_d;
        v.cdisk.hsd = c->cdisk_d + pl;
        v.cdisk.tgt = c->cdisk_tgt;
        v.cdisk.r = c->cdisk_r;
        v.cdisk.gs = c->cdisk_gs;
        v.cdisk.on = true;
    }
    INIT_TRY(cudaHostAlloc(&c->host_ring, 4 * sizeof(double), cudaHostAllocDefault));
    std::memset(c->host_ring, 0, 4 * sizeof(double));
    const long long nact = (long long)v.nx * (v.ndim == 2 ? v.ny : 1);
    c->totals_blocks = (int)std::min<long long>(1024, std::max<long long>(1, nact / 256));
    INIT_TRY(cudaMalloc(&c->part, (size_t)c->totals_blocks * 4 * (v.ndust + 1) * 2 * sizeof(double)));
    INIT_TRY(cudaMalloc(&c->tot_out, 4 * (v.ndust + 1) * sizeof(double)));
    for (int a = 0; a < 4; ++a) v.ev[a] = c->ev_time[a];
    v.time_kernels = true;
    INIT_TRY(cudaStreamSynchronize(c->stream));
#undef INIT_TRY
    *out = c;
    return SHARK_OK;
}

// Pinned or registered host memory (cudaHostAlloc / cudaHostRegister) is read and written by the
// conversion kernels directly over the host link, which moves the bytes no slower than a copy
// engine and saves the staging pass; any other pointer goes through the FP64 staging buffer.
static const void* pinned_device_alias(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int32_t shark_gpu_upload(shark_gpu_ctx* c, const double* u_prim, int64_t ncells, int32_t nvar) {
    if (!c || !u_prim) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    const shark::DeviceView& v = c->v;
    if (ncells != (int64_t)v.nx_max * v.ny_max || nvar != v.nvar)
        return fail(SHARK_ERR_INVALID_ARG, "state is %lld x %d, context expects %lld x %d", (long long)ncells, nvar,
                    (long long)v.nx_max * v.ny_max, v.nvar);
    CUDA_TRY(cudaSetDevice(c->cfg.device));
    if (!c->rho_ref_set) {
        // reference density of the mixed fused flux kernel: the mean gas density of the active
        // cells of the first state (kept for the life of the context; any value is exact in
        // theory, one near the typical density keeps the pressure variations at FP32 precision)
        c->rho_ref_set = true;
        if (is_mixed(c) && v.ndim == 2 && v.uniform && c->cfg.iso_cs == 1 && v.cs_uniform) {
            double sum = 0.0;
            for (int iy = v.ng; iy < v.ng + v.ny; ++iy)
                for (int ix = v.ng; ix < v.ng + v.nx; ++ix) sum += u_prim[(long long)iy * v.nx_max + ix];
            const double mean = sum / ((double)v.nx * (double)v.ny);
            c->v.rho_ref = std::isfinite(mean) && mean > 0.0 ? mean : 0.0;
        }
    }
    // drain any readbacks still in flight: the new state starts a new dt sequence
    for (int s = 0; s < 2; ++s) if (c->pending_read[s]) { cudaEventSynchronize(c->ev_read[s]); c->pending_read[s] = false; }
    const size_t bytes = (size_t)ncells * nvar * sizeof(double);
    const double* src = static_cast<const double*>(pinned_device_alias(u_prim));
    if (!src) {
        if (!c->staging) CUDA_TRY(cudaMalloc(&c->staging, bytes));
        CUDA_TRY(cudaMemcpyAsync(c->staging, u_prim, bytes, cudaMemcpyHostToDevice, c->stream));
        src = c->staging;
    }
    c->v.cur = 0;
    {
        cudaError_t e = is_mixed(c) ? shark::launch_from_fortran<float>(c->v, src, c->ubuf[0])
                                    : shark::launch_from_fortran<double>(c->v, src, c->ubuf[0]);
        if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "upload conversion: %s", cudaGetErrorString(e));
    }
    const size_t sbytes = c->state_bytes;
    for (int b = 1; b < c->v.nbuf; ++b)
        CUDA_TRY(cudaMemcpyAsync(c->ubuf[b], c->ubuf[0], sbytes, cudaMemcpyDeviceToDevice, c->stream));
    if (c->uinit && !c->have_uinit) {
        // the first state uploaded is the disk's initial state (uprim_condinit, setup.f90:79-83)
        CUDA_TRY(cudaMemcpyAsync(c->uinit, c->ubuf[0], sbytes, cudaMemcpyDeviceToDevice, c->stream));
        c->have_uinit = true;
    }
    CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(unsigned int), c->stream));
    c->status_seen = 0;
    if (c->v.ou_nm > 0)   // the forcing restarts from its initial coefficients with the state
        CUDA_TRY(cudaMemcpyAsync(c->v.ou, c->ou_init.data(), c->ou_init.size() * sizeof(double), cudaMemcpyHostToDevice,
                                 c->stream));
    // apply_boundaries of the first step on every buffer (fixed SOD ghosts are only ever set here)
    for (int b = 0; b < c->v.nbuf; ++b) {
        c->v.cur = b;
        cudaError_t eb = is_mixed(c) ? shark::launch_boundaries<float>(c->v) : shark::launch_boundaries<double>(c->v);
        if (eb != cudaSuccess) return fail(SHARK_ERR_CUDA, "boundaries: %s", cudaGetErrorString(eb));
    }
    c->v.cur = 0;
    // first courant (src/solver/solve.f90:74) on the uploaded state -> dt slot 0
    cudaError_t e = is_mixed(c) ? shark::launch_courant<float>(c->v, 0) : shark::launch_courant<double>(c->v, 0);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "courant: %s", cudaGetErrorString(e));
    int32_t rc = queue_readback(c, 0);
    if (rc) return rc;
    c->nstep = 0;
    c->uploaded = true;
    return SHARK_OK;
}

int32_t shark_gpu_step(shark_gpu_ctx* c, double* dt_out, int32_t* status_out) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "ctx is NULL");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "step before upload");
    const int slot = (int)(c->nstep & 1);
    if (c->cfg.flags & SHARK_FLAG_STATIC) {
        // static: solve returns before doing anything; dt keeps its value
        double dt; unsigned st;
        int32_t rc = wait_readback(c, slot, &dt, &st);
        if (rc) return rc;
        if ((rc = queue_readback(c, slot))) return rc;
        if (dt_out) *dt_out = dt;
        if (status_out) *status_out = (int32_t)c->status_seen;
        return SHARK_OK;
    }
    if (c->v.chg.on) {
        int32_t rs = seed_charges(c);
        if (rs) return rs;
    }
    c->v.step = c->nstep + 1;
    cudaError_t e = do_step(c, slot);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    c->chg_cold = false;
    c->v.cur = shark::next_cur(c->v);
    c->nstep++;
    int32_t rc = queue_readback(c, 1 - slot);   // dt of the next step, written by k_finalize
    if (rc) return rc;
    double dt;
    unsigned st;
    if ((rc = wait_readback(c, slot, &dt, &st))) return rc;   // dt this step used (ready one step earlier)
    if (dt_out) *dt_out = dt;
    if (status_out) *status_out = (int32_t)c->status_seen;
    return SHARK_OK;
}

int32_t shark_gpu_run(shark_gpu_ctx* c, int64_t nsteps, double tend, double* time_io, int64_t* steps_done,
                      int32_t* status_out) {
    if (!c || !time_io) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    double time = *time_io;
    int64_t n = 0;
    int32_t st = 0;
    while (n < nsteps && !(time >= tend)) {
        double dt;
        int32_t rc = shark_gpu_step(c, &dt, &st);
        if (rc) { *time_io = time; if (steps_done) *steps_done = n; return rc; }
        time = time + dt;
        ++n;
    }
    *time_io = time;
    if (steps_done) *steps_done = n;
    if (status_out) *status_out = st;
    return SHARK_OK;
}

int32_t shark_gpu_sync(shark_gpu_ctx* c, int32_t* status_out) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "ctx is NULL");
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    unsigned int st = 0;
    CUDA_TRY(cudaMemcpy(&st, c->status, sizeof st, cudaMemcpyDeviceToHost));
    c->status_seen |= st;
    if (status_out) *status_out = (int32_t)c->status_seen;
    return SHARK_OK;
}

int32_t shark_gpu_download(shark_gpu_ctx* c, double* u_prim, double* q) {
    if (!c || (!u_prim && !q)) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "download before upload");
    const shark::DeviceView& v = c->v;
    const size_t n = (size_t)v.nx_max * v.ny_max * v.nvar;
    if (u_prim) {
        double* dst = static_cast<double*>(const_cast<void*>(pinned_device_alias(u_prim)));
        if (!dst) {
            if (!c->staging) CUDA_TRY(cudaMalloc(&c->staging, n * sizeof(double)));
            dst = c->staging;
        }
        cudaError_t e = is_mixed(c) ? shark::launch_to_fortran<float>(v, v.u[v.cur], dst)
                                    : shark::launch_to_fortran<double>(v, v.u[v.cur], dst);
        if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "download conversion: %s", cudaGetErrorString(e));
        if (dst == c->staging)
            CUDA_TRY(cudaMemcpyAsync(u_prim, c->staging, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    if (q) return shark_gpu_ctoprim(c, q, nullptr);
    return SHARK_OK;
}

int32_t shark_gpu_ctoprim(shark_gpu_ctx* c, double* q, double* cs) {
    if (!c || !q) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "ctoprim before upload");
    const shark::DeviceView& v = c->v;
    const size_t ncells = (size_t)v.nx_max * v.ny_max;
    const size_t n = ncells * v.nvar;
    double* tmp = nullptr;
    CUDA_TRY(cudaMalloc(&tmp, (n + ncells) * sizeof(double)));
    cudaError_t e = is_mixed(c) ? shark::launch_ctoprim<float>(v, tmp, tmp + n) : shark::launch_ctoprim<double>(v, tmp, tmp + n);
    if (e != cudaSuccess) { cudaFree(tmp); return fail(SHARK_ERR_CUDA, "ctoprim: %s", cudaGetErrorString(e)); }
    e = cudaMemcpyAsync(q, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && cs) e = cudaMemcpyAsync(cs, tmp + n, ncells * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "ctoprim copy: %s", cudaGetErrorString(e));
    return SHARK_OK;
}

// ---- output / restart (write_output.f90:2-300; the reference's read_output is a stub) --------
namespace {
std::string f_i11(long long v) {
    char b[64];
    std::snprintf(b, sizeof b, "%11lld", v);
    return b;
}
// Fortran E23.15: [sign]0.d1..d15 and E+ee (a signed three-digit exponent without the E),
// right-justified in 23 characters
std::string f_e23_15(double v) {
    std::string body;
    if (v == 0.0) {
        body = std::string(std::signbit(v) ? "-" : "") + "0.000000000000000E+00";
    } else {
        char m[64];
        std::snprintf(m, sizeof m, "%.14E", std::fabs(v));
        const std::string t(m);
        const size_t ep = t.find('E');
        const int e = std::atoi(t.c_str() + ep + 1) + 1;
        char ex[16];
        if (std::abs(e) <= 99) std::snprintf(ex, sizeof ex, "E%c%02d", e < 0 ? '-' : '+', std::abs(e));
        else std::snprintf(ex, sizeof ex, "%c%03d", e < 0 ? '-' : '+', std::abs(e));
        body = std::string(v < 0 ? "-" : "") + "0." + t.substr(0, 1) + t.substr(2, ep - 2) + ex;
    }
    return std::string(body.size() < 23 ? 23 - body.size() : 0, ' ') + body;
}
struct OutUnits {
    double ul, ud, ut, uv, uP, urho, uPe;
};
OutUnits out_units(const shark_gpu_config& c) {
    OutUnits u;
    u.ul = unit1(c.unit_l);
    u.ud = unit1(c.unit_d);
    u.ut = unit1(c.unit_t);
    u.uv = u.ul / u.ut;
    // unit_P = unit_v**2 (disk_polar/units.f90; 1 in SOD, DUSTYWAVE, SI, dustyTurb, sedov),
    // unit_d unit_v**2 in KH/units.f90
    u.uP = c.setup == SHARK_SETUP_KH ? u.ud * (u.uv * u.uv) : u.uv * u.uv;
    u.urho = c.geom == 2 ? u.ud * u.ul : u.ud;            // unit_dcol for GEOM 2
    u.uPe = c.geom == 2 ? u.uP * u.ul : u.uP;
    return u;
}
bool write_raw(const std::string& path, const double* p, size_t n) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(p, sizeof(double), n, f) == n;
    return (std::fclose(f) == 0) && ok;
}
bool read_raw(const std::string& path, std::vector<double>& v, size_t n) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    v.resize(n);
    const bool ok = std::fread(v.data(), sizeof(double), n, f) == n && std::fgetc(f) == EOF;
    std::fclose(f);
    return ok;
}
}  // namespace

int32_t shark_gpu_output(shark_gpu_ctx* c, int32_t iout, double time, const char* prefix) {
    if (!c || !prefix) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (iout < 0 || iout > 99999) return fail(SHARK_ERR_INVALID_ARG, "iout %d outside 0..99999", iout);
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "output before upload");
    const shark::DeviceView& v = c->v;
    const shark_gpu_config& cf = c->cfg;
    const OutUnits u = out_units(cf);
    const int N = v.ndust;
    const bool chg = v.chg.on;
    const size_t nact = (size_t)v.nx * (v.ndim == 2 ? v.ny : 1);
    const size_t nstreams = 5 + (N > 0 ? 1 + 5 * (size_t)N : 0) + (chg ? 5 + (size_t)N : 0);
    char nchar[8];
    std::snprintf(nchar, sizeof nchar, "%05d", iout);
    const std::string dir = std::string(prefix) + "output_" + nchar;
    if (mkdir(dir.c_str(), 0755) != 0 && errno != EEXIST) return fail(SHARK_ERR_INVALID_ARG, "cannot create %s", dir.c_str());
    // fields: ctoprim on the device, then the active cells packed into the streams' file order
    const size_t ncells = (size_t)v.nx_max * v.ny_max;
    double* q = nullptr;
    double* packed = nullptr;
    CUDA_TRY(cudaMalloc(&q, ncells * v.nvar * sizeof(double)));
    cudaError_t e = cudaMalloc(&packed, nstreams * nact * sizeof(double));
    if (e == cudaSuccess) e = is_mixed(c) ? shark::launch_ctoprim<float>(v, q, nullptr) : shark::launch_ctoprim<double>(v, q, nullptr);
    const shark::OutScale sc{u.urho, u.uv, u.uPe, u.ul};
    if (e == cudaSuccess)
        e = is_mixed(c) ? shark::launch_output_pack<float>(v, q, sc, packed) : shark::launch_output_pack<double>(v, q, sc, packed);
    std::vector<double> h(nstreams * nact);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), packed, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(q);
    cudaFree(packed);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "output: %s", cudaGetErrorString(e));
    {
        FILE* f = std::fopen((dir + "/info.dat").c_str(), "w");
        if (!f) return fail(SHARK_ERR_INVALID_ARG, "cannot write %s/info.dat", dir.c_str());
        std::fprintf(f, "nvar        =%s\n", f_i11(v.nvar).c_str());
        std::fprintf(f, "ndust        =%s\n", f_i11(N).c_str());
        std::fprintf(f, "ndustpscal   =%s\n", f_i11(0).c_str());
        std::fprintf(f, "NX        =%s\n", f_i11(cf.nx).c_str());
        std::fprintf(f, "NY        =%s\n", f_i11(cf.ny).c_str());
        std::fprintf(f, "MHD        =%s\n", f_i11(0).c_str());
        std::fprintf(f, "GEOM        =%s\n", f_i11(cf.geom).c_str());
        std::fprintf(f, "TURB        =%s\n", f_i11(0).c_str());
        std::fprintf(f, "GRIDSPACE       =%s\n", f_i11(cf.gridspace).c_str());
        std::fprintf(f, "time        =%s\n", f_e23_15(time).c_str());
        std::fprintf(f, "unit_t        =%s\n", f_e23_15(u.ut).c_str());
        std::fprintf(f, "unit_d        =%s\n", f_e23_15(u.ud).c_str());
        std::fprintf(f, "unit_l        =%s\n", f_e23_15(u.ul).c_str());
        std::fprintf(f, "unit_v        =%s\n", f_e23_15(u.uv).c_str());
        std::fprintf(f, "unit_p        =%s\n", f_e23_15(u.uP).c_str());
        std::fprintf(f, "charging       =%s\n", f_i11(chg ? 1 : 0).c_str());
        if (std::fclose(f) != 0) return fail(SHARK_ERR_INVALID_ARG, "cannot write %s/info.dat", dir.c_str());
    }
    const double* p = h.data();
    auto W = [&](const char* name, const double* src, size_t n) { return write_raw(dir + "/" + name, src, n); };
    bool ok = W("x", c->out_x.data(), nact);
    ok = ok && W("rho", p, nact);
    ok = ok && W("v", p + nact, nact);
    if (v.ndim == 2) ok = ok && W("y", c->out_y.data(), nact);
    ok = ok && W("vy", p + 2 * nact, nact);
    ok = ok && W("vz", p + 3 * nact, nact);
    ok = ok && W("P", p + 4 * nact, nact);
    size_t s = 5;
    if (N > 0) {
        ok = ok && W("rhod_tot", p + s * nact, nact); s += 1;
        for (const char* name : {"rhod", "sd", "vd", "vdy", "vdz"}) { ok = ok && W(name, p + s * nact, (size_t)N * nact); s += N; }
    }
    if (chg) {
        for (const char* name : {"eta_a", "eta_o", "eta_h", "ni", "ne"}) { ok = ok && W(name, p + s * nact, nact); s += 1; }
        if (N > 0) ok = ok && W("zd", p + s * nact, (size_t)N * nact);
    }
    if (!ok) return fail(SHARK_ERR_INVALID_ARG, "cannot write the field files of %s", dir.c_str());
    return SHARK_OK;
}

int32_t shark_gpu_read_output(shark_gpu_ctx* c, const char* dir, double* time_out) {
    if (!c || !dir) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    const shark::DeviceView& v = c->v;
    const shark_gpu_config& cf = c->cfg;
    const std::string d(dir);
    FILE* f = std::fopen((d + "/info.dat").c_str(), "r");
    if (!f) return fail(SHARK_ERR_INVALID_ARG, "cannot open %s/info.dat", dir);
    std::map<std::string, std::string> info;
    char line[256];
    while (std::fgets(line, sizeof line, f)) {
        std::string t(line);
        const size_t eq = t.find('=');
        if (eq == std::string::npos) continue;
        std::string k = t.substr(0, eq);
        k.erase(k.find_last_not_of(' ') + 1);
        info[k] = t.substr(eq + 1);
    }
    std::fclose(f);
    auto geti = [&](const char* k, long long& x) {
        auto it = info.find(k);
        if (it == info.end()) return false;
        x = std::atoll(it->second.c_str());
        return true;
    };
    // E23.15 values: a three-digit exponent has no E; insert it for strtod
    auto getd = [&](const char* k, double& x) {
        auto it = info.find(k);
        if (it == info.end()) return false;
        std::string t = it->second;
        t.erase(0, t.find_first_not_of(' '));
        t.erase(t.find_last_not_of(" \n\r") + 1);
        if (t.find('E') == std::string::npos) {
            const size_t pm = t.find_last_of("+-");
            if (pm != std::string::npos && pm > 0) t.insert(pm, "E");
        }
        x = std::strtod(t.c_str(), nullptr);
        return true;
    };
    long long nvar = 0, ndust = 0, nx = 0, ny = 0, geom = 0;
    double time = 0.0, ud = 0.0, ul = 0.0, uv = 0.0, up = 0.0;
    if (!(geti("nvar", nvar) && geti("ndust", ndust) && geti("NX", nx) && geti("NY", ny) && geti("GEOM", geom) &&
          getd("time", time) && getd("unit_d", ud) && getd("unit_l", ul) && getd("unit_v", uv) && getd("unit_p", up)))
        return fail(SHARK_ERR_INVALID_ARG, "%s/info.dat lacks a field", dir);
    if (nvar != v.nvar || ndust != v.ndust || nx != cf.nx || ny != cf.ny || geom != cf.geom)
        return fail(SHARK_ERR_INVALID_ARG, "%s holds nvar %lld ndust %lld %lldx%lld geom %lld, the context %dx%d", dir, nvar,
                    ndust, nx, ny, geom, cf.nx, cf.ny);
    const int N = v.ndust;
    const size_t nact = (size_t)v.nx * (v.ndim == 2 ? v.ny : 1);
    std::vector<double> rho, vx, vy, vz, P, rd, vdx, vdy, vdz;
    bool ok = read_raw(d + "/rho", rho, nact) && read_raw(d + "/v", vx, nact) && read_raw(d + "/vy", vy, nact) &&
              read_raw(d + "/vz", vz, nact) && read_raw(d + "/P", P, nact);
    if (N > 0)
        ok = ok && read_raw(d + "/rhod", rd, (size_t)N * nact) && read_raw(d + "/vd", vdx, (size_t)N * nact) &&
             read_raw(d + "/vdy", vdy, (size_t)N * nact) && read_raw(d + "/vdz", vdz, (size_t)N * nact);
    if (!ok) return fail(SHARK_ERR_INVALID_ARG, "%s: a field file is missing or has the wrong size", dir);
    const double urho = geom == 2 ? ud * ul : ud, uPe = geom == 2 ? up * ul : up;
    // primitives -> conserved with primtoc's operations (solve.f90:265-302); ghost cells are filled
    // by the upload's boundaries
    const size_t ncells = (size_t)v.nx_max * v.ny_max;
    std::vector<double> U(ncells * v.nvar, 0.0);
    const double g1 = cf.gamma - 1.0;
    for (size_t a = 0; a < nact; ++a) {
        const int ix = v.ng + (v.ndim == 2 ? (int)(a % v.nx) : (int)a);
        const int iy = v.ndim == 2 ? v.ng + (int)(a / v.nx) : 0;
        const size_t i = (size_t)iy * v.nx_max + ix;
        const double r = rho[a] / urho, ux = vx[a] / uv, uy = vy[a] / uv, uz = vz[a] / uv, p = P[a] / uPe;
        U[0 * ncells + i] = r;
        U[1 * ncells + i] = r * ux;
        U[2 * ncells + i] = r * uy;
        U[3 * ncells + i] = r * uz;
        U[4 * ncells + i] = p / g1 + 0.5 * r * (ux * ux) + 0.5 * r * (uy * uy) + 0.5 * r * (uz * uz);
        for (int k = 0; k < N; ++k) {
            const size_t j = (size_t)k * nact + a;
            const double d_k = rd[j] / urho;
            U[(5 + k) * ncells + i] = d_k;
            U[(5 + N + k) * ncells + i] = d_k * (vdx[j] / uv);
            U[(5 + 2 * N + k) * ncells + i] = d_k * (vdy[j] / uv);
            U[(5 + 3 * N + k) * ncells + i] = d_k * (vdz[j] / uv);
        }
    }
    int32_t rc = shark_gpu_upload(c, U.data(), (int64_t)ncells, v.nvar);
    if (rc) return rc;
    if (time_out) *time_out = time;
    return SHARK_OK;
}

int32_t shark_gpu_totals(shark_gpu_ctx* c, double* out) {
    if (!c || !out) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "totals before upload");
    cudaError_t e = is_mixed(c) ? shark::launch_totals<float>(c->v, c->part, c->totals_blocks, c->tot_out)
                                : shark::launch_totals<double>(c->v, c->part, c->totals_blocks, c->tot_out);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "totals: %s", cudaGetErrorString(e));
    CUDA_TRY(cudaMemcpyAsync(out, c->tot_out, 4 * (c->v.ndust + 1) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return SHARK_OK;
}

int32_t shark_gpu_last_step_ms(shark_gpu_ctx* c, float* ms_out) {
    if (!c || !ms_out) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (c->nstep == 0) return fail(SHARK_ERR_STATE, "no step run yet");
    CUDA_TRY(cudaEventSynchronize(c->ev_time[3]));
    CUDA_TRY(cudaEventElapsedTime(&ms_out[0], c->ev_time[0], c->ev_time[1]));   // dt slot reset
    CUDA_TRY(cudaEventElapsedTime(&ms_out[1], c->ev_time[1], c->ev_time[2]));   // flux/update
    CUDA_TRY(cudaEventElapsedTime(&ms_out[2], c->ev_time[2], c->ev_time[3]));   // drag + dt
    return SHARK_OK;
}

int32_t shark_gpu_timed_run(shark_gpu_ctx* c, int64_t nsteps, double* time_io, float* ms_out) {
    if (!c || !time_io || !ms_out) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "timed run before upload");
    if (nsteps < 0) return fail(SHARK_ERR_INVALID_ARG, "nsteps < 0");
    // The steps are queued back to back with no host wait between them (the dt of every step
    // lives on the device; the step's preparation kernel stores it into pinned host memory, read
    // through its unified address, and the host sums them afterwards), so host-side stalls cannot
    // leave the GPU idle inside the timed region and no copy-engine transfer sits between steps.
    const bool is_static = (c->cfg.flags & SHARK_FLAG_STATIC) != 0;
    double* dts = nullptr;
    CUDA_TRY(cudaHostAlloc(&dts, (size_t)(nsteps > 0 ? nsteps : 1) * sizeof(double), cudaHostAllocMapped));
    double* dts_dev = nullptr;   // the same memory as the kernels address it
    if (cudaHostGetDevicePointer(reinterpret_cast<void**>(&dts_dev), dts, 0) != cudaSuccess) {
        cudaFreeHost(dts);
        return fail(SHARK_ERR_CUDA, "timed run: no device address for the dt log");
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int32_t rc = SHARK_OK;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) rc = fail(SHARK_ERR_CUDA, "timed run: %s", cudaGetErrorString(e));
    double time = *time_io;
    const int slot0 = (int)(c->nstep & 1);
    double dt_first = 0.0;
    if (rc == SHARK_OK) {
        unsigned st0;
        rc = wait_readback(c, slot0, &dt_first, &st0);   // the readback the next step would wait on
    }
    if (rc == SHARK_OK && c->v.chg.on) rc = seed_charges(c);
    if (rc == SHARK_OK) {
        if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) rc = fail(SHARK_ERR_CUDA, "timed run: %s", cudaGetErrorString(e));
    }
    const bool tk = c->v.time_kernels;
    c->v.time_kernels = false;
    if (rc == SHARK_OK) cudaEventRecord(e0, c->stream);
    for (int64_t n = 0; n < nsteps && rc == SHARK_OK; ++n) {
        const int slot = (int)(c->nstep & 1);
        if (!is_static) {
            c->v.step = c->nstep + 1;
            c->v.dt_log = dts_dev + n;
            e = do_step(c, slot);
            c->v.dt_log = nullptr;
            if (e != cudaSuccess) { rc = fail(SHARK_ERR_CUDA, "step launch: %s", cudaGetErrorString(e)); break; }
            c->chg_cold = false;
            c->v.cur = shark::next_cur(c->v);
        } else if ((e = cudaMemcpyAsync(dts + n, c->dt_slots + slot, sizeof(double), cudaMemcpyDeviceToHost,
                                        c->stream)) != cudaSuccess) {
            rc = fail(SHARK_ERR_CUDA, "timed run: %s", cudaGetErrorString(e));
            break;
        }
        if (!is_static) c->nstep++;   // a static step keeps its dt slot, as shark_gpu_step does
    }
    c->v.time_kernels = tk;
    if (rc == SHARK_OK) {
        cudaEventRecord(e1, c->stream);
        rc = queue_readback(c, (int)(c->nstep & 1));   // what the next step waits on
    }
    if (rc == SHARK_OK) {
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms_out, e0, e1);
        if (e != cudaSuccess) rc = fail(SHARK_ERR_CUDA, "timed run: %s", cudaGetErrorString(e));
    }
    if (rc == SHARK_OK) {
        for (int64_t n = 0; n < nsteps; ++n) time = time + dts[n];
        unsigned int st = 0;
        if ((e = cudaMemcpy(&st, c->status, sizeof st, cudaMemcpyDeviceToHost)) != cudaSuccess)
            rc = fail(SHARK_ERR_CUDA, "timed run: %s", cudaGetErrorString(e));
        c->status_seen |= st;
    }
    (void)dt_first;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFreeHost(dts);
    *time_io = time;
    return rc;
}

int32_t shark_gpu_kernel_times(shark_gpu_ctx* c, int64_t nsteps, float* avg_ms) {
    if (!c || !avg_ms || nsteps <= 0) return fail(SHARK_ERR_INVALID_ARG, "bad argument");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "kernel timing before upload");
    std::vector<cudaEvent_t> ev((size_t)nsteps * 4, nullptr);
    for (auto& e : ev) CUDA_TRY(cudaEventCreate(&e));
    const bool tk = c->v.time_kernels;
    int32_t rc = SHARK_OK;
    for (int64_t n = 0; n < nsteps && rc == SHARK_OK; ++n) {
        for (int a = 0; a < 4; ++a) c->v.ev[a] = ev[(size_t)n * 4 + a];
        c->v.time_kernels = true;
        rc = shark_gpu_step(c, nullptr, nullptr);
    }
    for (int a = 0; a < 4; ++a) c->v.ev[a] = c->ev_time[a];
    c->v.time_kernels = tk;
    double sum[4] = {0, 0, 0, 0};
    if (rc == SHARK_OK) {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        for (int64_t n = 0; n < nsteps && e == cudaSuccess; ++n) {
            float t;
            cudaEvent_t* E = &ev[(size_t)n * 4];
            for (int a = 0; a < 3 && e == cudaSuccess; ++a) {
                e = cudaEventElapsedTime(&t, E[a], E[a + 1]);
                sum[a] += t;
            }
            if (e == cudaSuccess) { e = cudaEventElapsedTime(&t, E[0], E[3]); sum[3] += t; }
        }
        if (e != cudaSuccess) rc = fail(SHARK_ERR_CUDA, "kernel times: %s", cudaGetErrorString(e));
    }
    for (auto& e : ev) cudaEventDestroy(e);
    for (int a = 0; a < 4; ++a) avg_ms[a] = (float)(sum[a] / (double)nsteps);
    return rc;
}

int32_t shark_gpu_charge(shark_gpu_ctx* c) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "ctx is NULL");
    if (!c->v.chg.on) return fail(SHARK_ERR_STATE, "charging is not enabled in this context");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "charge before upload");
    int32_t rc = seed_charges(c);
    if (rc) return rc;
    cudaError_t e = is_mixed(c) ? shark::launch_charge<float>(c->v) : shark::launch_charge<double>(c->v);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "charge: %s", cudaGetErrorString(e));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->chg_cold = false;
    return SHARK_OK;
}

int32_t shark_gpu_charge_reset(shark_gpu_ctx* c) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "ctx is NULL");
    if (!c->v.chg.on) return fail(SHARK_ERR_STATE, "charging is not enabled in this context");
    CUDA_TRY(cudaMemsetAsync(c->chg_psi, 0, (size_t)c->v.plane * sizeof(double), c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->chg_cold = true;
    return SHARK_OK;
}

int32_t shark_gpu_mlp_load(shark_gpu_ctx* c, const float* blob, int64_t n) {
    if (!c || !blob) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (n != SHARK_MLP_NBLOB) return fail(SHARK_ERR_INVALID_ARG, "blob has %lld floats, expected %d", (long long)n, SHARK_MLP_NBLOB);
    int32_t rc = mlp_alloc(c);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->mlp_blob, blob, SHARK_MLP_NBLOB * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    cudaError_t e = shark::mlp_pack(c->mlp_blob, c->mlp_packed, c->stream);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "mlp pack: %s", cudaGetErrorString(e));
    CUDA_TRY(cudaMemsetAsync(c->mlp_adam, 0, 2 * SHARK_MLP_NPARAM * sizeof(float), c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->mlp_step = 0;
    c->mlp_ready = true;
    return SHARK_OK;
}

int32_t shark_gpu_mlp_save(shark_gpu_ctx* c, float* blob, int64_t n) {
    if (!c || !blob) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (n != SHARK_MLP_NBLOB) return fail(SHARK_ERR_INVALID_ARG, "blob has %lld floats, expected %d", (long long)n, SHARK_MLP_NBLOB);
    int32_t rc = mlp_alloc(c);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(blob, c->mlp_blob, SHARK_MLP_NBLOB * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return SHARK_OK;
}

int32_t shark_gpu_mlp_collect(shark_gpu_ctx* c, int64_t capacity, int64_t* count) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "ctx is NULL");
    if (!c->v.chg.on) return fail(SHARK_ERR_STATE, "charging is not enabled in this context");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "collect before upload");
    int32_t rc = mlp_alloc(c);
    if (rc) return rc;
    if (!c->mlp_train) {
        if (capacity <= 0) return fail(SHARK_ERR_INVALID_ARG, "capacity must be > 0");
        CUDA_TRY(cudaMalloc(&c->mlp_train, (size_t)capacity * (SHARK_MLP_NFEAT + 1) * sizeof(float)));
        CUDA_TRY(cudaMalloc(&c->mlp_perm, (size_t)capacity * sizeof(int32_t)));
        c->mlp_cap = capacity;
    }
    // the plain Newton from the reference's cold start gives the converged solutions
    CUDA_TRY(cudaMemsetAsync(c->chg_psi, 0, (size_t)c->v.plane * sizeof(double), c->stream));
    shark::ChargeView& cv = c->v.chg;
    cv.use_seed = 0;
    cv.seed = nullptr;
    cudaError_t e = is_mixed(c) ? shark::launch_charge<float>(c->v) : shark::launch_charge<double>(c->v);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "charge: %s", cudaGetErrorString(e));
    c->chg_cold = false;
    if ((rc = features(c))) return rc;
    e = is_mixed(c) ? shark::launch_charge_collect<float>(c->v, c->mlp_feat, c->mlp_train, c->mlp_count, c->mlp_cap)
                    : shark::launch_charge_collect<double>(c->v, c->mlp_feat, c->mlp_train, c->mlp_count, c->mlp_cap);
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "collect: %s", cudaGetErrorString(e));
    unsigned long long n = 0;
    CUDA_TRY(cudaMemcpyAsync(&n, c->mlp_count, sizeof n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if ((long long)n > c->mlp_cap) {
        n = (unsigned long long)c->mlp_cap;
        CUDA_TRY(cudaMemcpy(c->mlp_count, &n, sizeof n, cudaMemcpyHostToDevice));
    }
    if (count) *count = (int64_t)n;
    return SHARK_OK;
}

int32_t shark_gpu_mlp_train(shark_gpu_ctx* c, int32_t steps, int32_t batch, float lr, uint64_t seed, float* loss_curve) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "ctx is NULL");
    if (steps <= 0 || batch <= 0 || !(lr > 0.0f)) return fail(SHARK_ERR_INVALID_ARG, "steps, batch and lr must be > 0");
    if (!c->mlp_train) return fail(SHARK_ERR_STATE, "no training samples: call shark_gpu_mlp_collect first");
    unsigned long long n = 0;
    CUDA_TRY(cudaMemcpy(&n, c->mlp_count, sizeof n, cudaMemcpyDeviceToHost));
    if (n < (unsigned long long)batch) return fail(SHARK_ERR_STATE, "%llu samples < batch %d", n, batch);
    const int F = SHARK_MLP_NFEAT;
    // normalisation of the features and of the target from the training set (first training only)
    std::vector<float> h((size_t)n * (F + 1));
    CUDA_TRY(cudaMemcpy(h.data(), c->mlp_train, h.size() * sizeof(float), cudaMemcpyDeviceToHost));
    if (!c->mlp_ready) {
        std::vector<float> nb(F * 2 + 2);
        for (int i = 0; i <= F; ++i) {
            double s = 0.0, s2 = 0.0;
            for (size_t r = 0; r < n; ++r) { const double x = h[r * (F + 1) + i]; s += x; s2 += x * x; }
            const double mu = s / (double)n, var = std::max(s2 / (double)n - mu * mu, 0.0);
            const double sd = std::sqrt(var) > 1e-12 ? std::sqrt(var) : 1.0;
            if (i < F) { nb[i] = (float)mu; nb[F + i] = (float)sd; }
            else { nb[2 * F] = (float)mu; nb[2 * F + 1] = (float)sd; }
        }
        CUDA_TRY(cudaMemcpy(c->mlp_blob + nn::OFF_XMU, nb.data(), nb.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    int32_t rc = mlp_scratch(c, (size_t)steps);
    if (rc) return rc;
    CUDA_TRY(cudaMemsetAsync(c->mlp_scratch, 0, (size_t)steps * sizeof(float), c->stream));
    std::mt19937_64 rng(seed);
    std::vector<int32_t> perm(n);
    for (size_t i = 0; i < n; ++i) perm[i] = (int32_t)i;
    size_t pos = n;
    shark::MlpArgs a{};
    a.feat = c->mlp_train;
    a.target = c->mlp_train;
    a.feat_stride = F + 1;
    a.n = batch;
    a.blob = c->mlp_blob;
    a.packed = c->mlp_packed;
    a.grad = c->mlp_grad;
    a.inv_n = 1.0f / (float)batch;
    a.err = c->mlp_err;
    for (int s = 0; s < steps; ++s) {
        if (pos + (size_t)batch > n) {
            std::shuffle(perm.begin(), perm.end(), rng);
            CUDA_TRY(cudaMemcpyAsync(c->mlp_perm, perm.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
            CUDA_TRY(cudaStreamSynchronize(c->stream));
            pos = 0;
        }
        a.index = c->mlp_perm + pos;
        a.loss = c->mlp_scratch + s;
        pos += (size_t)batch;
        CUDA_TRY(cudaMemsetAsync(c->mlp_grad, 0, SHARK_MLP_NPARAM * sizeof(float), c->stream));
        cudaError_t e = shark::mlp_backward(a, c->stream);
        if (e == cudaSuccess) e = shark::mlp_adam(c->mlp_blob, c->mlp_grad, c->mlp_adam, c->mlp_adam + SHARK_MLP_NPARAM, lr,
                                                  ++c->mlp_step, c->stream);
        if (e == cudaSuccess) e = shark::mlp_pack(c->mlp_blob, c->mlp_packed, c->stream);
        if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "mlp training step: %s", cudaGetErrorString(e));
    }
    unsigned int err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, c->mlp_err, sizeof err, cudaMemcpyDeviceToHost, c->stream));
    if (loss_curve) CUDA_TRY(cudaMemcpyAsync(loss_curve, c->mlp_scratch, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (err) return fail(SHARK_ERR_CUDA, "a tensor-core completion wait of the network gave up");
    if (loss_curve) for (int s = 0; s < steps; ++s) loss_curve[s] /= (float)batch;
    c->mlp_ready = true;
    return SHARK_OK;
}

int32_t shark_gpu_mlp_eval(shark_gpu_ctx* c, const float* feat, const float* target, int64_t n, float* out, float* grad,
                           float* loss) {
    if (!c || !feat || n <= 0 || n > (1 << 30)) return fail(SHARK_ERR_INVALID_ARG, "bad argument");
    int32_t rc = mlp_alloc(c);
    if (rc) return rc;
    const int F = SHARK_MLP_NFEAT;
    if ((rc = mlp_scratch(c, (size_t)n * (F + 1) + (size_t)n + 1))) return rc;
    std::vector<float> h((size_t)n * (F + 1), 0.0f);
    for (int64_t r = 0; r < n; ++r) {
        for (int i = 0; i < F; ++i) h[r * (F + 1) + i] = feat[r * F + i];
        if (target) h[r * (F + 1) + F] = target[r];
    }
    float* d_in = c->mlp_scratch;
    float* d_out = c->mlp_scratch + (size_t)n * (F + 1);
    float* d_loss = d_out + n;
    CUDA_TRY(cudaMemcpyAsync(d_in, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    shark::MlpArgs a{};
    a.feat = d_in;
    a.target = d_in;
    a.feat_stride = F + 1;
    a.n = (int)n;
    a.blob = c->mlp_blob;
    a.packed = c->mlp_packed;
    a.err = c->mlp_err;
    a.out = d_out;
    cudaError_t e = shark::mlp_forward(a, c->stream);
    if (e == cudaSuccess && target && grad) {
        a.out = nullptr;
        a.grad = c->mlp_grad;
        a.loss = d_loss;
        a.inv_n = 1.0f / (float)n;
        e = cudaMemsetAsync(c->mlp_grad, 0, SHARK_MLP_NPARAM * sizeof(float), c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(d_loss, 0, sizeof(float), c->stream);
        if (e == cudaSuccess) e = shark::mlp_backward(a, c->stream);
    }
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "mlp eval: %s", cudaGetErrorString(e));
    if (out) CUDA_TRY(cudaMemcpyAsync(out, d_out, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (target && grad) {
        CUDA_TRY(cudaMemcpyAsync(grad, c->mlp_grad, SHARK_MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
        if (loss) CUDA_TRY(cudaMemcpyAsync(loss, d_loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    }
    unsigned int err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, c->mlp_err, sizeof err, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (err) return fail(SHARK_ERR_CUDA, "a tensor-core completion wait of the network gave up");
    return SHARK_OK;
}

int32_t shark_gpu_mlp_features(shark_gpu_ctx* c, float* feat) {
    if (!c || !feat) return fail(SHARK_ERR_INVALID_ARG, "NULL argument");
    if (!c->v.chg.on) return fail(SHARK_ERR_STATE, "charging is not enabled in this context");
    if (!c->uploaded) return fail(SHARK_ERR_STATE, "features before upload");
    int32_t rc = features(c);
    if (rc) return rc;
    const shark::DeviceView& v = c->v;
    std::vector<float> h((size_t)v.plane * SHARK_MLP_NFEAT);
    CUDA_TRY(cudaMemcpyAsync(h.data(), c->mlp_feat, h.size() * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (int iy = 0; iy < v.ny_max; ++iy)
        for (int ix = 0; ix < v.nx_max; ++ix)
            for (int i = 0; i < SHARK_MLP_NFEAT; ++i)
                feat[((size_t)iy * v.nx_max + ix) * SHARK_MLP_NFEAT + i] = h[((size_t)iy * v.pitch + ix) * SHARK_MLP_NFEAT + i];
    return SHARK_OK;
}

int32_t shark_gpu_charge_stats(shark_gpu_ctx* c, int64_t* hist, int64_t* nonconv, int64_t* total_iters) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "ctx is NULL");
    if (!c->v.chg.on) return fail(SHARK_ERR_STATE, "charging is not enabled in this context");
    unsigned long long h[SHARK_CHARGE_HIST + 2];
    CUDA_TRY(cudaMemcpyAsync(h, c->chg_hist, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (hist) for (int b = 0; b < SHARK_CHARGE_HIST; ++b) hist[b] = (int64_t)h[b];
    if (nonconv) *nonconv = (int64_t)h[SHARK_CHARGE_HIST];
    if (total_iters) *total_iters = (int64_t)h[SHARK_CHARGE_HIST + 1];
    return SHARK_OK;
}

int32_t shark_gpu_download_charge(shark_gpu_ctx* c, double* zd, double* ni, double* ne, double* psi, double* eta,
                                  double* gamma_d, int32_t* iters) {
    if (!c) return fail(SHARK_ERR_INVALID_ARG, "ctx is NULL");
    if (!c->v.chg.on) return fail(SHARK_ERR_STATE, "charging is not enabled in this context");
    const shark::DeviceView& v = c->v;
    const size_t nc = (size_t)v.nx_max * v.ny_max;
    const int N = v.ndust;
    double* tmp = nullptr;
    CUDA_TRY(cudaMalloc(&tmp, nc * (size_t)N * sizeof(double)));
    struct Part { double* dst; const void* src; int count; bool fp64; };
    const Part parts[6] = {{zd, v.chg.zd, N, false}, {ni, v.chg.ni, 1, false}, {ne, v.chg.ne, 1, false},
                           {psi, v.chg.psi_old, 1, true}, {eta, v.chg.eta, 3, false}, {gamma_d, v.chg.gamma_d, N, false}};
    cudaError_t e = cudaSuccess;
    for (const Part& q : parts) {
        if (!q.dst || e != cudaSuccess) continue;
        if (q.fp64 || !is_mixed(c)) e = shark::launch_planes_to_fortran<double>(v, q.src, q.count, tmp);
        else e = shark::launch_planes_to_fortran<float>(v, q.src, q.count, tmp);
        if (e == cudaSuccess) e = cudaMemcpyAsync(q.dst, tmp, nc * q.count * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
    cudaFree(tmp);
    if (e == cudaSuccess && iters) {
        std::vector<int32_t> h((size_t)v.plane);
        e = cudaMemcpyAsync(h.data(), c->chg_iters, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e == cudaSuccess)
            for (int iy = 0; iy < v.ny_max; ++iy)
                for (int ix = 0; ix < v.nx_max; ++ix)
                    iters[(size_t)iy * v.nx_max + ix] = h[(size_t)iy * v.pitch + ix];
    }
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, "download_charge: %s", cudaGetErrorString(e));
    return SHARK_OK;
}

int32_t shark_gpu_free(shark_gpu_ctx* c) { return release(c); }

}  // extern "C"
