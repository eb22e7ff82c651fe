// shark_oracle.cpp -- TEST INFRASTRUCTURE ONLY (see shark_oracle.h).
//
// Line-faithful FP64 restatement of SHARK's per-step update.  Each routine cites the Fortran it
// follows; operation order inside expressions follows Fortran's left-to-right evaluation so the
// FP64 GPU path (same order, no FMA contraction) can be compared at round-off level.  Built with
// -O2 -ffp-contract=off (gfortran -O3 on x86-64/aarch64 without -ffast-math keeps IEEE order).
//
// Array layout mirrors the Fortran module arrays: u(i,ivar) -> u[ivar*ncells + i] (0-based),
// qm/qp/flux(i,ivar,idim) -> [(idim*nvar + ivar)*ncells + i], force(i,1:3) -> [c*ncells + i],
// force_dust(i,1:3,idust) -> [(idust*3 + c)*ncells + i], tstop(i,idust) -> [idust*ncells + i].
#include "shark_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <sys/stat.h>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double half = 0.5;
constexpr double pi = 3.141592653589793238462643383279;   // src/commons/phys_const.f90:14

// gfortran evaluates x**n (integer n) with __builtin_powi; x**2 / x**2.0 fold to x*x.
inline double sq(double x) { return x * x; }
inline double powi(double x, int n) { return __builtin_powi(x, n); }
// Fortran SIGN(1.0d0, x): +1 for +0 and positive, -1 for -0 and negative.
inline double fsign1(double x) { return std::signbit(x) ? -1.0 : 1.0; }
inline double fmax2(double a, double b) { return a > b ? a : b; }   // gfortran MAX for non-NaN
inline double fmin2(double a, double b) { return a < b ? a : b; }

}  // namespace

struct oracle_state {
    shark_gpu_config cfg;
    int nx, ny, nghost, ndust, nvar, ndim;
    int nx_max, ny_max;
    int64_t ncells;
    int first_active, last_active, first_active_y, last_active_y;  // 0-based inclusive
    // variable indices (src/commons/allocate_init.f90:225-262), 0-based
    int irho = 0, ivx = 1, ivy = 2, ivz = 3, iP = 4;
    std::vector<int> irhod, ivdx, ivdy, ivdz;
    int index_vn[2], index_vt[2];
    std::vector<int> index_vdn, index_vdt;   // [idust*2 + idim]

    std::vector<double> u, q, qm, qp, flux, cs;
    std::vector<double> dx, surf, vol, position, radii_c;
    std::vector<uint8_t> active, active_pred;
    std::vector<double> force, force_dust, tstop, sdust, epsilondust;
    std::vector<double> u_init;     // disk_polar: uprim_condinit (state of the first upload / setup)
    std::vector<double> fargo_v;    // fargo_velocity(ncells)
    // charging (ionisation_commons.f90): per cell psi_old, ni, ne, resistivities, Newton
    // iteration count; per cell and species zd, gamma_d (species-major like sdust)
    std::vector<double> psi_old, ni, ne, eta_o, eta_h, eta_a, zd, gamma_d;
    std::vector<int32_t> chg_iters;
    std::vector<double> chg_seed;   // optional Newton start per cell (0 = none)
    // dustyTurb Ornstein-Uhlenbeck forcing: modes (kx', ky', |k'|) and coefficients (a_m, b_m)
    std::vector<double> ou_modes, ou_coef;
    std::vector<double> eta_visc;   // kinematic viscosity per cell (disk: alpha H cs)
    int64_t ou_step = 0;
    double dt = 0.0, time = 0.0;

    // setup-derived scalars
    double box_l = 1.0, box_l_y = 1.0;

    double& U(int64_t i, int v) { return u[(int64_t)v * ncells + i]; }
    double& Q(int64_t i, int v) { return q[(int64_t)v * ncells + i]; }
    double& QM(int64_t i, int v, int d) { return qm[((int64_t)d * nvar + v) * ncells + i]; }
    double& QP(int64_t i, int v, int d) { return qp[((int64_t)d * nvar + v) * ncells + i]; }
    double& FLX(int64_t i, int v, int d) { return flux[((int64_t)d * nvar + v) * ncells + i]; }
    double& DX(int64_t i, int d) { return dx[(int64_t)d * ncells + i]; }
    double& SURF(int64_t i, int d) { return surf[(int64_t)d * ncells + i]; }
    double& POS(int64_t i, int d) { return position[(int64_t)d * ncells + i]; }
    double& FORCE(int64_t i, int c) { return force[(int64_t)c * ncells + i]; }
    double& FDUST(int64_t i, int c, int k) { return force_dust[((int64_t)k * 3 + c) * ncells + i]; }
    double& TSTOP(int64_t i, int k) { return tstop[(int64_t)k * ncells + i]; }
    double& SDUST(int64_t i, int k) { return sdust[(int64_t)k * ncells + i]; }
    double& EPSD(int64_t i, int k) { return epsilondust[(int64_t)k * ncells + i]; }

    int64_t icell(int ix, int iy) const { return (ny == 1) ? ix : (int64_t)ix + (int64_t)iy * nx_max; }
    int ixx(int64_t i) const { return (ny == 1) ? (int)i : (int)(i % nx_max); }
    int iyy(int64_t i) const { return (ny == 1) ? 0 : (int)(i / nx_max); }

    bool flag(int f) const { return (cfg.flags & f) != 0; }
};

namespace {

// ---------------------------------------------------------------------------------------------
// slope_limit  (src/solver/slope_limiters.f90:5-37)
// ---------------------------------------------------------------------------------------------
inline double slope_limit(int slope_type, double slope_lft, double slope_rgt) {
    double r;
    if (slope_type == 1) {
        r = slope_lft;
        if (std::fabs(slope_rgt) < std::fabs(slope_lft)) r = slope_rgt;
        if (slope_rgt * slope_lft < 0.0) r = 0.0;
    } else if (slope_type == 2) {
        r = 2.0 * slope_lft * slope_rgt / (slope_lft + slope_rgt);
        if (slope_rgt * slope_lft <= 0.0) r = 0.0;
    } else {  // 3: MC with factor 1.5 (other values rejected at create time)
        double dcen = half * (slope_lft + slope_rgt);
        double dsgn = fsign1(dcen);
        double slop = fmin2(1.5 * std::fabs(slope_lft), 1.5 * std::fabs(slope_rgt));
        double dlim = slop;
        if ((slope_lft * slope_rgt) <= 0.0) dlim = 0.0;
        r = dsgn * fmin2(dlim, std::fabs(dcen));
    }
    return r;
}

// ---------------------------------------------------------------------------------------------
// get_active_cells (src/grid/grid.f90:57-99)
// ---------------------------------------------------------------------------------------------
void get_active_cells(oracle_state& s) {
    s.active.assign(s.ncells, 0);
    s.active_pred.assign(s.ncells, 0);
    if (s.ndim == 1) {
        for (int ix = 0; ix < s.nx_max; ++ix) {
            if (ix >= s.first_active && ix <= s.last_active) s.active[ix] = 1;
            if (ix >= 1 && ix <= s.nx_max - 2) s.active_pred[ix] = 1;
        }
    } else {
        for (int ix = 0; ix < s.nx_max; ++ix)
            for (int iy = 0; iy < s.ny_max; ++iy) {
                int64_t ii = s.icell(ix, iy);
                if (ix >= s.first_active && ix <= s.last_active && iy >= s.first_active_y &&
                    iy <= s.last_active_y)
                    s.active[ii] = 1;
                if (ix >= 1 && ix <= s.nx_max - 2 && iy >= 1 && iy <= s.ny_max - 2) s.active_pred[ii] = 1;
            }
    }
}

// ---------------------------------------------------------------------------------------------
// gridinit (src/grid/grid.f90:104-173) and gridinit_disk_log (src/grid/grid.f90:180-240)
// float(n) is default REAL in gfortran: exact for the integers involved.
// ---------------------------------------------------------------------------------------------
void gridinit(oracle_state& s) {
    const double rmax_x = s.box_l, rmax_y = s.box_l_y;
    const int nx = s.nx, ny = s.ny;
    std::fill(s.radii_c.begin(), s.radii_c.end(), 1.0);   // allocate_init.f90:27-30
    if (s.cfg.geom == 0) {
        if (s.ndim == 1) {
            for (int ix = 0; ix < s.ncells; ++ix) {
                s.DX(ix, 0) = rmax_x / (double)(float)nx;
                s.vol[ix] = s.DX(ix, 0);
                s.SURF(ix, 0) = 1.0;
                // 1D positions are right cell edges, accumulated (grid.f90:131)
                if (s.active[ix]) s.POS(ix, 0) = s.POS(ix - 1, 0) + s.DX(ix, 0);
            }
        } else {
            for (int ix = 0; ix < s.nx_max; ++ix)
                for (int iy = 0; iy < s.ny_max; ++iy) {
                    int64_t c = s.icell(ix, iy);
                    s.DX(c, 0) = rmax_x / (double)(float)nx;
                    s.DX(c, 1) = rmax_y / (double)(float)ny;
                    s.SURF(c, 0) = s.DX(c, 0);
                    s.SURF(c, 1) = s.DX(c, 1);
                    s.vol[c] = s.DX(c, 0) * s.DX(c, 1);
                    s.POS(c, 0) = ((double)(float)(ix - s.first_active) + half) * rmax_x / (double)(float)nx;
                    s.POS(c, 1) = ((double)(float)(iy - s.first_active_y) + half) * rmax_y / (double)(float)ny;
                }
        }
    } else {  // geom 2, polar face-on, 2D only (validated at create)
        const double inner_r = s.cfg.inner_r;
        if (s.cfg.gridspace == 0) {
            for (int ix = 0; ix < s.nx_max; ++ix)
                for (int iy = 0; iy < s.ny_max; ++iy) {
                    int64_t c = s.icell(ix, iy);
                    s.DX(c, 0) = rmax_x / (double)(float)nx;
                    s.DX(c, 1) = 2.0 * pi / (double)(float)ny;
                    s.radii_c[c] = inner_r + ((double)(float)(ix - s.first_active) + half) * rmax_x / (double)(float)nx;
                    double phi = ((double)(float)(iy - s.first_active_y) + half) * 2.0 * pi / (double)(float)ny;
                    s.POS(c, 0) = s.radii_c[c] * std::cos(phi);
                    s.POS(c, 1) = s.radii_c[c] * std::sin(phi);
                    s.SURF(c, 0) = (s.radii_c[c] - half * s.DX(c, 0)) * (s.DX(c, 1));
                    s.SURF(c, 1) = s.DX(c, 0);
                    s.vol[c] = s.radii_c[c] * s.DX(c, 0) * s.DX(c, 1);
                }
        } else {
            const double zeta_r = std::pow(rmax_x / inner_r, 1.0 / (double)(nx - 1));
            for (int iy = 0; iy < s.ny_max; ++iy) {
                for (int ix = 0; ix < s.nx_max; ++ix) {
                    int64_t c = s.icell(ix, iy);
                    int k = ix - s.first_active;
                    s.radii_c[c] = inner_r * half * (powi(zeta_r, k) + powi(zeta_r, k + 1));
                    s.DX(c, 0) = inner_r * (powi(zeta_r, k + 1) - powi(zeta_r, k));
                    s.DX(c, 1) = 2.0 * pi / (double)(float)ny;
                    double phi = ((double)(float)(iy - s.first_active_y) + half) * 2.0 * pi / (double)(float)ny;
                    s.POS(c, 0) = s.radii_c[c] * std::cos(phi);
                    s.POS(c, 1) = s.radii_c[c] * std::sin(phi);
                    s.SURF(c, 0) = inner_r * (powi(zeta_r, k)) * (s.DX(c, 1));
                    s.SURF(c, 1) = s.DX(c, 0);
                    s.vol[c] = s.radii_c[c] * s.DX(c, 0) * s.DX(c, 1);
                }
                for (int g = 0; g < s.nghost; ++g) {
                    int64_t cl = s.icell(g, iy), cr = s.icell(s.nx_max - 1 - g, iy);
                    s.radii_c[cl] = inner_r * 0.5;
                    s.radii_c[cr] = rmax_x + 0.5 * s.DX(s.icell(s.last_active, iy), 0);
                    s.DX(cl, 0) = s.DX(s.icell(s.first_active, iy), 0);
                    s.DX(cr, 0) = s.DX(s.icell(s.last_active, iy), 0);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// ctoprim (src/solver/solve.f90:195-253); non_standard_eos is not used by the in-scope setups.
// ---------------------------------------------------------------------------------------------
void ctoprim(oracle_state& s) {
    const double gamma = s.cfg.gamma, smallr = s.cfg.smallr, smallp = s.cfg.smallp;
    const int N = s.ndust;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < s.ncells; ++i) {
        double rho = s.U(i, s.irho);
        s.Q(i, s.irho) = fmax2(rho, smallr);
        s.Q(i, s.ivx) = s.U(i, s.ivx) / rho;
        s.Q(i, s.ivy) = s.U(i, s.ivy) / rho;
        s.Q(i, s.ivz) = s.U(i, s.ivz) / rho;
        double ekin = half * rho * sq(s.U(i, s.ivx) / rho) + half * rho * sq(s.U(i, s.ivy) / rho) +
                      half * rho * sq(s.U(i, s.ivz) / rho);
        double emag = 0.0;
        s.Q(i, s.iP) = fmax2((gamma - 1.0) * (s.U(i, s.iP) - ekin - emag), smallp);
        if (s.cfg.iso_cs < 1) s.cs[i] = std::sqrt(gamma * s.Q(i, s.iP) / s.Q(i, s.irho));
        if (s.cfg.iso_cs == 1) s.Q(i, s.iP) = s.U(i, s.irho) * sq(s.cs[i]);
        for (int k = 0; k < N; ++k) {
            double rd = s.U(i, s.irhod[k]);
            s.Q(i, s.irhod[k]) = rd;
            s.Q(i, s.ivdx[k]) = s.U(i, s.ivdx[k]) / rd;
            s.Q(i, s.ivdy[k]) = s.U(i, s.ivdy[k]) / rd;
            s.Q(i, s.ivdz[k]) = s.U(i, s.ivdz[k]) / rd;
        }
    }
}

// primtoc (src/solver/solve.f90:265-302)
void primtoc(oracle_state& s) {
    const double gamma = s.cfg.gamma;
    for (int64_t i = 0; i < s.ncells; ++i) {
        double r = s.Q(i, s.irho);
        s.U(i, s.irho) = r;
        s.U(i, s.ivx) = r * s.Q(i, s.ivx);
        s.U(i, s.ivy) = r * s.Q(i, s.ivy);
        s.U(i, s.ivz) = r * s.Q(i, s.ivz);
        s.U(i, s.iP) = s.Q(i, s.iP) / (gamma - 1.0) + half * r * sq(s.Q(i, s.ivx)) +
                       half * r * sq(s.Q(i, s.ivy)) + half * r * sq(s.Q(i, s.ivz));
        for (int k = 0; k < s.ndust; ++k) {
            double rd = s.Q(i, s.irhod[k]);
            s.U(i, s.irhod[k]) = rd;
            s.U(i, s.ivdx[k]) = rd * s.Q(i, s.ivdx[k]);
            s.U(i, s.ivdy[k]) = rd * s.Q(i, s.ivdy[k]);
            s.U(i, s.ivdz[k]) = rd * s.Q(i, s.ivdz[k]);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Boundaries
// ---------------------------------------------------------------------------------------------
// periodic_boundaries (src/grid/boundary_types.f90:149-186): y rows first (active x only),
// then x columns over all y (which fills the corners).
void periodic_boundaries(oracle_state& s) {
    const int ng = s.nghost;
    if (s.ndim == 2) {
        for (int ix = s.first_active; ix <= s.last_active; ++ix)
            for (int g = 0; g < ng; ++g) {
                int64_t bl = s.icell(ix, g), br = s.icell(ix, s.ny_max - 1 - g);
                int64_t al = s.icell(ix, s.last_active_y - ng + 1 + g), ar = s.icell(ix, s.first_active_y + ng - 1 - g);
                for (int v = 0; v < s.nvar; ++v) {
                    s.U(bl, v) = s.U(al, v);
                    s.U(br, v) = s.U(ar, v);
                }
            }
    }
    for (int g = 0; g < ng; ++g)
        for (int iy = 0; iy < s.ny_max; ++iy) {
            int64_t bl = s.icell(g, iy), br = s.icell(s.nx_max - 1 - g, iy);
            int64_t al = s.icell(s.last_active - ng + 1 + g, iy), ar = s.icell(s.first_active + ng - 1 - g, iy);
            for (int v = 0; v < s.nvar; ++v) {
                s.U(bl, v) = s.U(al, v);
                s.U(br, v) = s.U(ar, v);
            }
        }
}

// SOD apply_boundaries (src/setups/SOD/boundaries.f90:49-77): fixed left/right states along the
// shock direction, periodic along the other one.
void sod_boundaries(oracle_state& s) {
    const int ng = s.nghost;
    const double g1 = s.cfg.gamma - 1.0;
    auto fix = [&](int64_t bl, int64_t br) {
        s.U(bl, s.irho) = s.cfg.sod_rho_l;
        s.U(br, s.irho) = s.cfg.sod_rho_r;
        s.U(bl, s.iP) = s.cfg.sod_P_l / g1;
        s.U(br, s.iP) = s.cfg.sod_P_r / g1;
        s.U(bl, s.ivx) = 0.0; s.U(br, s.ivx) = 0.0;
        s.U(bl, s.ivy) = 0.0; s.U(br, s.ivy) = 0.0;
        s.U(bl, s.ivz) = 0.0; s.U(br, s.ivz) = 0.0;
    };
    if (s.ndim == 2) {
        for (int ix = s.first_active; ix <= s.last_active; ++ix)
            for (int g = 0; g < ng; ++g) {
                int64_t bl = s.icell(ix, g), br = s.icell(ix, s.ny_max - 1 - g);
                int64_t al = s.icell(ix, s.last_active_y - ng + 1 + g), ar = s.icell(ix, s.first_active_y + ng - 1 - g);
                if (s.cfg.sod_direction == 1) fix(bl, br);
                else for (int v = 0; v < s.nvar; ++v) { s.U(bl, v) = s.U(al, v); s.U(br, v) = s.U(ar, v); }
            }
    }
    for (int g = 0; g < ng; ++g)
        for (int iy = 0; iy < s.ny_max; ++iy) {
            int64_t bl = s.icell(g, iy), br = s.icell(s.nx_max - 1 - g, iy);
            int64_t al = s.icell(s.last_active - ng + 1 + g, iy), ar = s.icell(s.first_active + ng - 1 - g, iy);
            if (s.cfg.sod_direction == 0) fix(bl, br);
            else for (int v = 0; v < s.nvar; ++v) { s.U(bl, v) = s.U(al, v); s.U(br, v) = s.U(ar, v); }
        }
}

// SI apply_boundaries (src/setups/SI/boundaries.f90:1-81): periodic along y; shear-periodic along
// x with the azimuthal (vz) momentum shifted by -/+ rho q Omega L.  The first loop's `mom_new`
// lines have no effect in the reference (values computed and discarded) and are omitted.
void si_boundaries(oracle_state& s) {
    const int ng = s.nghost;
    const double qs = s.cfg.si_q_shear, om = s.cfg.si_omega, L = s.box_l;
    for (int ix = s.first_active; ix <= s.last_active; ++ix)
        for (int g = 0; g < ng; ++g) {
            int64_t bl = s.icell(ix, g), br = s.icell(ix, s.ny_max - 1 - g);
            int64_t al = s.icell(ix, s.last_active_y - ng + 1 + g), ar = s.icell(ix, s.first_active_y + ng - 1 - g);
            for (int v = 0; v < s.nvar; ++v) { s.U(bl, v) = s.U(al, v); s.U(br, v) = s.U(ar, v); }
        }
    for (int g = 0; g < ng; ++g)
        for (int iy = 0; iy < s.ny_max; ++iy) {
            int64_t bl = s.icell(g, iy), br = s.icell(s.nx_max - 1 - g, iy);
            int64_t al = s.icell(s.last_active - ng + 1 + g, iy), ar = s.icell(s.first_active + ng - 1 - g, iy);
            for (int v = 0; v < s.nvar; ++v) { s.U(bl, v) = s.U(al, v); s.U(br, v) = s.U(ar, v); }
            s.U(bl, s.ivz) = s.U(al, s.ivz) - s.U(al, s.irho) * qs * om * L;
            s.U(br, s.ivz) = s.U(ar, s.ivz) + s.U(ar, s.irho) * qs * om * L;
            for (int k = 0; k < s.ndust; ++k) {
                s.U(bl, s.ivdz[k]) = s.U(al, s.ivdz[k]) - s.U(al, s.irhod[k]) * qs * om * L;
                s.U(br, s.ivdz[k]) = s.U(ar, s.ivdz[k]) + s.U(ar, s.irhod[k]) * qs * om * L;
            }
        }
}

// disk_polar profile: aspect ratio h(r) = disk_hoverr r^((T slope + 1)/2), H = h r,
// Omega = sqrt(Mstar/r^3), cs = Omega H (disk_polar/setup.f90:27-32 with constant h for slope -1)
double disk_h(const shark_gpu_config& c, double r) { return c.disk_hoverr * std::pow(r, 0.5 * (c.disk_temp_slope + 1.0)); }
double disk_cs(const shark_gpu_config& c, double r) {
    return std::sqrt(c.disk_mstar / (r * r * r)) * (disk_h(c, r) * r);
}

// disk_polar apply_boundaries (disk_polar/boundaries.f90:1-70): periodic in phi over the active
// radii, outflow in r with the radial velocities clipped to point out of the domain.  The
// reference copies u_prim(first_active) / u_prim(last_active), i.e. one cell of the first row,
// into every radial ghost (the cell index is used without icell); this restatement copies the
// first/last active cell of the same row, the evident intent.  Accretion (off) is not restated.
void disk_boundaries(oracle_state& s) {
    const int ng = s.nghost;
    for (int ix = s.first_active; ix <= s.last_active; ++ix)
        for (int g = 0; g < ng; ++g) {
            int64_t bl = s.icell(ix, g), br = s.icell(ix, s.ny_max - 1 - g);
            int64_t al = s.icell(ix, s.last_active_y - ng + 1 + g), ar = s.icell(ix, s.first_active_y + ng - 1 - g);
            for (int v = 0; v < s.nvar; ++v) { s.U(bl, v) = s.U(al, v); s.U(br, v) = s.U(ar, v); }
        }
    for (int g = 0; g < ng; ++g)
        for (int iy = 0; iy < s.ny_max; ++iy) {
            int64_t bl = s.icell(g, iy), br = s.icell(s.nx_max - 1 - g, iy);
            int64_t al = s.icell(s.first_active, iy), ar = s.icell(s.last_active, iy);
            for (int v = 0; v < s.nvar; ++v) { s.U(bl, v) = s.U(al, v); s.U(br, v) = s.U(ar, v); }
            s.U(br, s.ivx) = fmin2(s.U(br, s.ivx), 0.0);
            s.U(bl, s.ivx) = fmax2(s.U(bl, s.ivx), 0.0);
            for (int k = 0; k < s.ndust; ++k) {
                s.U(br, s.ivdx[k]) = fmin2(s.U(br, s.ivdx[k]), 0.0);
                s.U(bl, s.ivdx[k]) = fmax2(s.U(bl, s.ivdx[k]), 0.0);
            }
        }
}

// Cartesian disk apply_boundaries = zero_gradients (disk/boundaries.f90, boundary_types.f90:48-100)
// as written: in 2D the source of every ghost is u_prim(first_active_y), u_prim(last_active_y),
// u_prim(first_active) or u_prim(last_active) -- cell indices of the first (ghost) row, since the
// row numbers are used as cell numbers -- so the ghosts take the values of cells of that row,
// in the order of the loops: y ghosts of the active columns first (column by column, bottom
// before top), then the x ghosts of every row.
void disk_cart_boundaries(oracle_state& s) {
    const int ng = s.nghost;
    // Fortran cell numbers first_active_y, last_active_y, first_active, last_active (1-based)
    // as 0-based linear indices
    const int64_t sy_l = s.first_active_y, sy_r = s.last_active_y, sx_l = s.first_active, sx_r = s.last_active;
    for (int ix = s.first_active; ix <= s.last_active; ++ix)
        for (int g = 0; g < ng; ++g) {
            int64_t bl = s.icell(ix, g), br = s.icell(ix, s.ny_max - 1 - g);
            for (int v = 0; v < s.nvar; ++v) {
                s.U(bl, v) = s.U(sy_l, v);
                s.U(br, v) = s.U(sy_r, v);
            }
        }
    for (int g = 0; g < ng; ++g)
        for (int iy = 0; iy < s.ny_max; ++iy) {
            int64_t bl = s.icell(g, iy), br = s.icell(s.nx_max - 1 - g, iy);
            for (int v = 0; v < s.nvar; ++v) {
                s.U(bl, v) = s.U(sx_l, v);
                s.U(br, v) = s.U(sx_r, v);
            }
        }
}

void apply_boundaries(oracle_state& s) {
    switch (s.cfg.setup) {
        case SHARK_SETUP_SOD: sod_boundaries(s); break;
        case SHARK_SETUP_SI: si_boundaries(s); break;
        case SHARK_SETUP_DISK_POLAR: disk_boundaries(s); break;
        case SHARK_SETUP_DISK_CART: disk_cart_boundaries(s); break;
        default: periodic_boundaries(s); break;   // DUSTYWAVE, dustyTurb, KH, sedov (*/boundaries.f90)
    }
}

// Cartesian disk geometry of cell i (disk/setup.f90): offsets from the box centre, softened
// radius rr = sqrt(xx^2 + yy^2 + smooth_r^2), H = HoverR rr
struct CdiskCell {
    double xx, yy, rr, r_cyl;
};
CdiskCell cdisk_cell(const oracle_state& s, int64_t i) {
    CdiskCell c;
    c.xx = s.position[i] - half * s.box_l;
    c.yy = s.position[(size_t)s.ncells + i] - half * s.box_l_y;
    c.r_cyl = std::sqrt(sq(c.xx) + sq(c.yy));
    c.rr = std::sqrt(sq(c.xx) + sq(c.yy) + sq(s.cfg.cdisk_smooth_r));
    return c;
}
double cdisk_H(const oracle_state& s, int64_t i) { return s.cfg.disk_hoverr * cdisk_cell(s, i).rr; }

// ---------------------------------------------------------------------------------------------
// compute_tstop per setup
// ---------------------------------------------------------------------------------------------
void compute_tstop(oracle_state& s) {
    const int N = s.ndust;
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        for (int k = 0; k < N; ++k) {
            double ts;
            switch (s.cfg.setup) {
                case SHARK_SETUP_DUSTYWAVE:   // DUSTYWAVE/setup.f90:212-221
                    ts = s.Q(i, s.irhod[k]) * s.Q(i, s.irho) / s.cfg.dust_K[k] / (s.Q(i, s.irho));
                    break;
                case SHARK_SETUP_SI:          // SI/setup.f90:389-397 (constant, precomputed on host)
                    ts = s.cfg.dust_tstop[k];
                    break;
                case SHARK_SETUP_DUSTYTURB:   // dustyTurb/setup.f90:456
                    ts = s.cfg.dust_stokes[k] * s.box_l * s.cfg.turb_rho0 / s.cs[i] / s.Q(i, s.irho);
                    break;
                case SHARK_SETUP_DISK_CART: {    // disk/setup.f90 compute_tstop: Epstein with Sigma/sqrt(2 pi H)
                    ts = std::sqrt(pi * s.cfg.gamma / 8.0) * (s.cfg.rhograin) * s.SDUST(i, k) /
                         (s.Q(i, s.irho) / (std::sqrt(2.0 * pi * cdisk_H(s, i))) * s.cs[i]);
                    break;
                }
                case SHARK_SETUP_DISK_POLAR: {   // disk_polar/setup.f90:425-451, Epstein with Sigma/(sqrt(2 pi) H)
                    const double H = disk_h(s.cfg, s.radii_c[i]) * s.radii_c[i];
                    ts = std::sqrt(pi * s.cfg.gamma / 8.0) * (s.cfg.rhograin) * s.SDUST(i, k) /
                         (s.Q(i, s.irho) / (std::sqrt(2.0 * pi) * H) * s.cs[i]);
                    break;
                }
                default:                      // SOD/setup.f90:179-185, KH/setup.f90:218-239, Epstein
                    ts = std::sqrt(pi * s.cfg.gamma / 8.0) * (s.cfg.rhograin) * s.SDUST(i, k) /
                         (s.Q(i, s.irho) * s.cs[i]);
                    break;
            }
            s.TSTOP(i, k) = ts;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Charging: Marchand et al. (2021) Newton on the reduced grain potential psi
// (src/chemistry/ionisation.f90:4-214).  Constants of src/commons/phys_const.f90:5-13.
// Fortran x**2., x**2.0 and x**3. are evaluated as products, x**4.0 as (x*x)*(x*x); SUM() in
// index order.  The state -> (nH, T, zeta, n_k, a_k) map is per setup:
//   dustyTurb (cgs code units): nH = rho unit_d/(mu_gas mH), T = T_cloud, zeta = chg_x,
//     n_k = rho_k unit_d/(m_k unit_m), m_k = 4/3 pi rhograin s_k^3 (mrn_distri, dust_init.f90:192);
//   polar disk (2D surface densities): the same on the midplane densities Sigma/(sqrt(2 pi) H),
//     T from the isothermal sound speed through cs_eos (disk_polar/eos.f90), zeta =
//     chg_x exp(-Sigma unit_d unit_l/chg_sigma_att).  The reference's disk has no temperature
//     (its barotrop is empty) and a unit_nH without mu_gas mH; this is the re-specified form.
// ---------------------------------------------------------------------------------------------
namespace phys {
constexpr double e_el = 4.8e-10, m_el = 9.109e-28, clight = 3e10, mH = 1.67e-24, kB = 1.38e-16;
}
double unit_or_1(double u) { return u != 0.0 ? u : 1.0; }
double F43() { return (double)(4.0f / 3.0f); }   // Fortran 4./3. is a default-REAL quotient

// Start point of the reference (ionisation.f90:33-52): Newton on the dust-free balance, from -2.5.
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

struct ChargeCell {
    double nH, T, x, rho_cgs;
    std::vector<double> nk, lk, mk_cgs;
};

void charge_inputs(oracle_state& s, int64_t i, ChargeCell& c) {
    const shark_gpu_config& g = s.cfg;
    const double ul = unit_or_1(g.unit_l), ud = unit_or_1(g.unit_d), ut = unit_or_1(g.unit_t);
    const double um = ul * ul * ul * ud, uv = ul / ut, unH = ud / (g.mu_gas * phys::mH);
    const int N = s.ndust;
    double hs = 1.0;                                    // column-to-midplane factor
    if (g.setup == SHARK_SETUP_DISK_POLAR) hs = std::sqrt(2.0 * pi) * (disk_h(g, s.radii_c[i]) * s.radii_c[i]);
    const double rho = s.U(i, s.irho) / hs;
    c.rho_cgs = rho * ud;
    c.nH = rho * unH;
    if (g.setup == SHARK_SETUP_DISK_POLAR) {
        const double csc = s.cs[i] * uv;
        c.T = g.mu_gas * phys::mH * (csc * csc) / (g.gamma * phys::kB);
        c.x = g.chg_sigma_att > 0.0 ? g.chg_x * std::exp(-(s.U(i, s.irho) * ud * ul) / g.chg_sigma_att) : g.chg_x;
    } else {
        c.T = g.T_cloud;
        c.x = g.chg_x;
    }
    c.nk.resize(N); c.lk.resize(N); c.mk_cgs.resize(N);
    for (int k = 0; k < N; ++k) {
        const double sk = s.cfg.dust_size[k];
        const double mk = F43() * pi * g.rhograin * (sk * sk * sk);   // code mass (mrn_distri)
        c.lk[k] = sk * ul;
        c.mk_cgs[k] = mk * um;
        c.nk[k] = (s.U(i, s.irhod[k]) / hs) * ud / (mk * um);
    }
}

// One cell of `charge` (ionisation.f90:60-206).  psi_start: psi_old(i) or 0.  Returns the
// iteration count; writes zd (N), ni, ne, psi_old and, with res, eta_o/h/a and gamma_d (N).
int charge_cell(const shark_gpu_config& g, const ChargeCell& c, double psi0, double psi_start,
                double* zd, double& ni_o, double& ne_o, double& psi_out, bool res,
                double& eta_o, double& eta_h, double& eta_a, double* gamma_d) {
    const int N = (int)c.nk.size();
    const double mH = phys::mH, kB = phys::kB, e_el = phys::e_el, m_el = phys::m_el;
    const double thetai = g.chg_stick_el * std::sqrt(g.chg_mu_ions * mH / m_el);
    const double epsone = 0.99999, T = c.T, x = c.x, nH = c.nH;
    std::vector<double> tau(N), alpha(N), l2(N);
    const double sigmav_ie = (2e-7) / std::sqrt(T / 300.0);
    for (int k = 0; k < N; ++k) {
        tau[k] = c.lk[k] * kB * T / (e_el * e_el);
        alpha[k] = std::sqrt(8.0 / (pi * tau[k]));
        l2[k] = c.lk[k] * c.lk[k];
    }
    const double vi = std::sqrt(8.0 * kB * T / (pi * g.chg_mu_ions * mH));
    const double th2 = thetai * thetai, th3 = thetai * thetai * thetai;
    double conv = 1e4, psi = psi0;
    int niter = 0;
    if (psi_start != 0.0) psi = psi_start;
    int lowT = 0;
    double eps_psi, n_i = 0.0, fpsi;
    while (conv > g.chg_eps && niter < g.chg_nitermax) {
        eps_psi = (1.0 - psi) / thetai * std::exp(-psi);
        const double et = eps_psi * thetai;
        const double et2 = et * et;
        n_i = 0.0;
        for (int k = 0; k < N; ++k)
            n_i = n_i + (-(psi * tau[k] + (1.0 - et2) / (1.0 + et * alpha[k] + et2)) * c.nk[k] / (1.0 - eps_psi));
        double S1 = 0.0;
        for (int k = 0; k < N; ++k)
            S1 = S1 + c.nk[k] * pi * l2[k] * ((1.0 - psi) + (2.0 / tau[k]) * (et2 + et) / (1.0 + et * alpha[k] + et2));
        fpsi = sigmav_ie * eps_psi * (n_i * n_i) / (x * nH) + n_i * vi / (x * nH) * (S1) - 1.0;
        const double D = (-eps_psi * (2.0 - psi) / (1.0 - psi));
        double S2 = 0.0, S3 = 0.0, S4 = 0.0, S5 = 0.0, S6 = 0.0;
        for (int k = 0; k < N; ++k) {
            const double den = 1.0 + et * alpha[k] + et2;
            S2 = S2 + c.nk[k] * (-(et2 * et2) + (4.0 * th2 - th3 * alpha[k]) * (eps_psi * eps_psi) +
                                 (2.0 * thetai * alpha[k] - 4.0 * th2) * eps_psi + 1.0 - thetai * alpha[k]) / (den * den);
            S3 = S3 + c.nk[k] * tau[k];
            S4 = S4 + c.nk[k] * pi * l2[k] / (tau[k] * den);
            S5 = S5 + c.nk[k] * pi * l2[k] * (2.0 * eps_psi * th2 + thetai * alpha[k]) / (tau[k] * (den * den));
            S6 = S6 + c.nk[k] * pi * l2[k];
        }
        const double om = 1.0 - eps_psi;
        const double dni = -1.0 / (om * om) * (D) * (S2) - (psi / om * (D) + 1.0) * S3 / om;
        const double dfdpsi =
            sigmav_ie * n_i / (x * nH) * (n_i * (D) + 2.0 * eps_psi * dni) +
            2.0 * n_i * vi / (x * nH) * (et2 + et) *
                ((dni / n_i + (D) * (2.0 * et + 1.0) / (eps_psi * (1.0 + et))) * (S4) + ((D) * S5)) +
            n_i * vi / (x * nH) * (dni / n_i * (1.0 - psi) - 1.0) * (S6);
        const double prev = psi;
        psi = psi - fpsi / dfdpsi;
        if (psi < psi0) {
            psi = psi0 * 0.9999999;
            lowT = 1;
        } else if (psi > 0.0) {
            psi = -1e-5;
        }
        conv = std::fabs(fpsi);   // the reference's interim values of conv are overwritten here
        niter = niter + 1;
        // an update that leaves psi unchanged with the residual above the tolerance repeats
        // itself until nitermax (e.g. the psi0 clamp): go there directly, same final state
        if (psi == prev && conv > g.chg_eps) niter = g.chg_nitermax;
    }
    eps_psi = (1.0 - psi) / thetai * std::exp(-psi);
    if (lowT > 0) eps_psi = epsone;
    double nsum = 0.0;
    for (int k = 0; k < N; ++k) {
        zd[k] = psi * tau[k] + (1.0 - (eps_psi * eps_psi) * th2) / (1.0 + eps_psi * thetai * alpha[k] + (eps_psi * eps_psi) * th2);
        nsum = nsum - zd[k] * c.nk[k] / (1.0 - eps_psi);
        if (lowT > 0) nsum = std::sqrt(eps_psi * x * nH / sigmav_ie);
    }
    ni_o = nsum;
    ne_o = eps_psi * ni_o;
    psi_out = lowT > 0 ? psi0 : psi;
    if (res) {
        // resistivities (ionisation.f90:163-206); the grain stopping time uses the gas density
        // and cs_eos(T) in cgs (the reference multiplies cs_eos, already cgs, by unit_v)
        const double B = g.chg_B0 * std::sqrt(nH / 1e4);
        const double cs_T = std::sqrt(g.gamma * kB * T / (g.mu_gas * mH));
        const double mu_i = 2.0 * mH * g.chg_mu_ions * mH / (2.0 * mH + g.chg_mu_ions * mH);
        const double mu_e = 2.0 * mH * m_el / (m_el + 2.0 * mH);
        const double vrms_i = std::sqrt(8.0 * kB * T / (pi * mu_i)) * 1e-5;
        const double vrms_el = std::sqrt(8.0 * kB * T / (pi * mu_e)) * 1e-5;
        const double sigmav_el = 3.16e-11 * std::pow(vrms_el, 1.3);
        const double sigmav_ions = 2.4e-9 * std::pow(vrms_i, 0.6);
        const double as_He_ions = (double)1.14f, as_He_el = (double)1.16f;   // REAL*4 literals
        const double t_sel = 1.0 / as_He_el * ((m_el + 2.0 * mH) / (2.0 * mH)) / sigmav_el / nH;
        const double t_sions = 1.0 / as_He_ions * ((g.chg_mu_ions * mH + 2.0 * mH) / (2.0 * mH)) / sigmav_ions / nH;
        const double sig_el = (ne_o) * (e_el * e_el) * t_sel / m_el;
        const double sig_i = (ni_o) * (e_el * e_el) * t_sions / (g.chg_mu_ions * mH);
        const double om_el = -e_el * B / phys::clight / m_el;
        const double om_i = e_el * B / phys::clight / (g.chg_mu_ions * mH);
        double so = 0.0, sp = 0.0, sh = 0.0;
        for (int k = 0; k < N; ++k) {
            const double t_sd = std::sqrt(pi * g.gamma / 8.0) * (g.rhograin * unit_or_1(g.unit_d)) * (c.lk[k]) / (c.rho_cgs * cs_T);
            const double sd = c.nk[k] * ((zd[k] * e_el) * (zd[k] * e_el)) * t_sd / (c.mk_cgs[k]);
            const double omd = zd[k] * e_el * B / phys::clight / (c.mk_cgs[k]);
            so = so + sd;
            sp = sp + sd / (1.0 + (omd * t_sd) * (omd * t_sd));
            sh = sh + sd * (omd * t_sd) / (1.0 + (omd * t_sd) * (omd * t_sd));
            gamma_d[k] = t_sd * omd;
        }
        const double sigma_o = so + sig_i + sig_el;
        const double sigma_p = sig_i / (1.0 + (om_i * t_sions) * (om_i * t_sions)) +
                               sig_el / (1.0 + (om_el * t_sel) * (om_el * t_sel)) + sp;
        const double sigma_h = -sig_i * (om_i * t_sions) / (1.0 + (om_i * t_sions) * (om_i * t_sions)) -
                               sig_el * (om_el * t_sel) / (1.0 + (om_el * t_sel) * (om_el * t_sel)) - sh;
        eta_o = 1.0 / sigma_o;
        eta_h = sigma_h / (sigma_p * 2. + sigma_h * sigma_h);   // as written in ionisation.f90:200
        eta_a = sigma_p / (sigma_p * sigma_p + sigma_h * sigma_h) - 1.0 / sigma_o;
    }
    return niter;
}

// analytical_charge (ionisation.f90:809-922, functions_NR.f90:15-128, newton_raphson.f90:7-97):
// per cell and species, Newton on the grain charge Z from -1 until |f| < 1e-14 (at most 1e5
// iterations) of the Fujii et al. (2011) balance; n_i, n_e of the cell are those of the last
// species (the reference overwrites them in the species loop).  Cell inputs in cgs through the
// setup map of charge_inputs (q(irho) is the floored density, as in the reference).
double fujii_f(double y, double zeta, double rho, double m_d, double rho_d, double s_d, double T, double mu_gas,
               double mu_ions, double* fp) {
    const double mH = phys::mH, kB = phys::kB, e = phys::e_el;
    const double m_i = mu_ions * mH, m_e = phys::m_el;
    const double k_e = pi * (s_d * s_d) * std::sqrt(8 * kB * T / (pi * m_e)) * std::exp((e * e) * y / (s_d * kB * T));
    const double k_i = pi * (s_d * s_d) * std::sqrt(8 * kB * T / (pi * m_i)) * (1 - (e * e) * y / (s_d * kB * T));
    const double a = m_d * rho / (rho_d * mu_gas * mH);
    const double f = mu_gas * mH * zeta / rho * (a * a) * ((1 / k_i) - (1 / k_e)) - y;
    if (fp) {
        const double kp_e = pi * s_d * std::sqrt(8 * kB * T / pi / m_e) * (e * e) / kB / T * std::exp((e * e) * (y) / s_d / kB / T);
        const double kp_i = -pi * s_d * std::sqrt(8 * kB * T / pi / m_i) * (e * e) / kB / T;
        const double b = m_d * rho / rho_d / mu_gas / mH;
        *fp = mu_gas * mH * zeta / rho * (b * b) * (kp_e / (k_e * k_e) - kp_i / (k_i * k_i)) - 1;
    }
    return f;
}

int fujii_solve(double zeta, double rho, double m_d, double rho_d, double s_d, double T, double mu_gas, double mu_ions,
                double& y, bool& converged) {
    y = -1.0;
    int k;
    converged = false;
    for (k = 1; k <= 100000; ++k) {
        double fp;
        const double fy = fujii_f(y, zeta, rho, m_d, rho_d, s_d, T, mu_gas, mu_ions, &fp);
        if (std::fabs(fy) < 1.e-14) { converged = true; break; }
        const double dy = fy / fp;
        y = y - dy;
    }
    if (!converged) {
        const double fy = fujii_f(y, zeta, rho, m_d, rho_d, s_d, T, mu_gas, mu_ions, nullptr);
        converged = std::fabs(fy) <= 1.e-14;
    }
    return k - 1;
}

void analytical_charge(oracle_state& s) {
    const shark_gpu_config& g = s.cfg;
    const int N = s.ndust;
    const size_t nc = (size_t)s.ncells;
    const double ul = unit_or_1(g.unit_l), ud = unit_or_1(g.unit_d), um = ul * ul * ul * ud;
    const double mH = phys::mH, kB = phys::kB, e = phys::e_el;
#pragma omp parallel
    {
        ChargeCell c;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < s.ncells; ++i) {
            charge_inputs(s, i, c);
            double hs = 1.0;
            if (g.setup == SHARK_SETUP_DISK_POLAR) hs = std::sqrt(2.0 * pi) * (disk_h(g, s.radii_c[i]) * s.radii_c[i]);
            const double rho = s.Q(i, s.irho) / hs * ud;
            int total = 0;
            for (int k = 0; k < N; ++k) {
                const double m_d = F43() * pi * g.rhograin * (g.dust_size[k] * g.dust_size[k] * g.dust_size[k]) * um;
                const double rho_d = s.Q(i, s.irhod[k]) / hs * ud;
                const double s_d = g.dust_size[k] * ul;
                double y;
                bool conv;
                total += fujii_solve(c.x, rho, m_d, rho_d, s_d, c.T, g.mu_gas, g.chg_mu_ions, y, conv);
                s.zd[(size_t)k * nc + i] = y;
                const double m_i = g.chg_mu_ions * mH, m_e = phys::m_el;
                const double k_e = pi * (s_d * s_d) * std::sqrt(8 * kB * c.T / (pi * m_e)) * std::exp((e * e) * y / (s_d * kB * c.T));
                const double k_i = pi * (s_d * s_d) * std::sqrt(8 * kB * c.T / (pi * m_i)) * (1 - (e * e) * y / (s_d * kB * c.T));
                s.ni[i] = c.x * rho * m_d / (k_i * g.mu_gas * mH * rho_d);
                s.ne[i] = c.x * rho * m_d / (k_e * g.mu_gas * mH * rho_d);
            }
            s.chg_iters[i] = total;
        }
    }
}

// charge over every cell, ghosts included (the reference's active-cell test is commented out)
void charge(oracle_state& s) {
    const shark_gpu_config& g = s.cfg;
    const int N = s.ndust;
    const double thetai = g.chg_stick_el * std::sqrt(g.chg_mu_ions * phys::mH / phys::m_el);
    const double psi0 = charge_psi0(thetai);
    const bool res = (g.chg_mode & SHARK_CHARGE_RESISTIVITIES) != 0;
    const size_t nc = (size_t)s.ncells;
    if (s.psi_old.size() != nc) {
        s.psi_old.assign(nc, 0.0); s.ni.assign(nc, 0.0); s.ne.assign(nc, 0.0);
        s.eta_o.assign(nc, 0.0); s.eta_h.assign(nc, 0.0); s.eta_a.assign(nc, 0.0);
        s.zd.assign(nc * N, 0.0); s.gamma_d.assign(nc * N, 0.0); s.chg_iters.assign(nc, 0);
    }
    if (g.chg_mode & SHARK_CHARGE_ANALYTICAL) { analytical_charge(s); return; }
#pragma omp parallel
    {
        ChargeCell c;
        std::vector<double> zd(N), gd(N);
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < s.ncells; ++i) {
            charge_inputs(s, i, c);
            double start = s.psi_old[i];
            if (!s.chg_seed.empty() && s.chg_seed[i] != 0.0) start = s.chg_seed[i];
            double psi;
            s.chg_iters[i] = charge_cell(g, c, psi0, start, zd.data(), s.ni[i], s.ne[i], psi, res,
                                         s.eta_o[i], s.eta_h[i], s.eta_a[i], gd.data());
            s.psi_old[i] = psi;
            for (int k = 0; k < N; ++k) {
                s.zd[(size_t)k * nc + i] = zd[k];
                if (res) s.gamma_d[(size_t)k * nc + i] = gd[k];
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Dust growth (src/dust/dust_growth.f90:3-256): Smoluchowski coagulation (and fragmentation) on
// the mass grid of dust_init.f90:11-45, sub-cycled per cell with dt_growth = CFL_growth
// rho_k/|drho_k/dt|.  Re-specified where the reference has no definition, with the reason:
//   temperature: dustyTurb T_cloud, polar disk T(r) from its isothermal cs (the reference calls
//     the empty barotrop of these setups);
//   polar disk: densities, Reynolds number and Jeans length on the midplane Sigma/(sqrt(2 pi) H),
//     the large-eddy time 1/Omega(r), and the surface-density rate K Sigma_i Sigma_j/(sqrt(2 pi) H
//     m_i m_j) (the reference's disk branch is empty);
//   velocities: cs_eos(T) is cgs and is divided by unit_v where a code velocity is meant.
// x**3. and zeta**3. are evaluated as products; the REAL*4 literals 3.2, 1./2.6, 1.6 of the
// Stokes function keep their single-precision values.  A cell that needs more than 100000
// sub-steps stops there (the reference loops on).
// ---------------------------------------------------------------------------------------------
namespace phys_g { constexpr double grav = 6.67e-8; }

struct GrowthGrid {
    double zeta, eta, massmin, m_mono, Ebr_mono;
    std::vector<double> aminus, aplus, mk, sk, redis;   // redis[ifrag * N + k]: share of bin k
};

GrowthGrid growth_grid(const shark_gpu_config& g) {
    const int N = g.ndust;
    const double ul = unit_or_1(g.unit_l), ud = unit_or_1(g.unit_d), ut = unit_or_1(g.unit_t);
    const double um = ul * ul * ul * ud, uv = ul / ut;
    const double rg_cgs = g.rhograin * ud;
    GrowthGrid G;
    G.zeta = std::pow(g.grw_smax / g.grw_smin, 1.0 / N);
    G.eta = G.zeta * G.zeta * G.zeta;
    G.massmin = (g.grw_kernel == 0) ? F43() * pi * rg_cgs * (g.grw_smin * g.grw_smin * g.grw_smin) / um
                                    : g.grw_smin * g.grw_smin * g.grw_smin;
    const double a_mu = g.grw_size_mono / 2.0;
    G.Ebr_mono = g.grw_Abr * std::pow(g.grw_gamma_grains, 5.0 / 3.0) * std::pow(a_mu, 4.0 / 3.0) /
                 std::pow(g.grw_estar_grains, 2.0 / 3.0) / (uv * uv * um);
    G.m_mono = 4.0 / 3.0 * pi * rg_cgs * (g.grw_size_mono * g.grw_size_mono * g.grw_size_mono) / um;
    G.aminus.resize(N); G.aplus.resize(N); G.mk.resize(N); G.sk.resize(N);
    for (int k = 0; k < N; ++k) {
        G.aminus[k] = g.grw_smin * powi(G.zeta, k) / ul;
        G.aplus[k] = g.grw_smin * powi(G.zeta, k + 1) / ul;
        const double s = g.dust_size[k];
        G.sk[k] = s;
        G.mk[k] = (g.grw_kernel == 0) ? F43() * pi * g.rhograin * (s * s * s) : s * s * s;
    }
    const double e4 = 4.0 - g.grw_slope_mono;
    G.redis.assign((size_t)N * N, 0.0);
    for (int i = 0; i < N; ++i) {
        double sum = 0.0;
        for (int j = 0; j <= i; ++j) {
            const double r = (std::pow(G.aplus[j], e4) - std::pow(G.aminus[j], e4)) /
                             (std::pow(G.aplus[i], e4) - std::pow(G.aminus[0], e4));
            G.redis[(size_t)i * N + j] = r;
        }
        for (int j = 0; j < N; ++j) sum += G.redis[(size_t)i * N + j];
        for (int j = 0; j < N; ++j) G.redis[(size_t)i * N + j] = G.redis[(size_t)i * N + j] / sum;
    }
    return G;
}

// x_stokes-dependent factor of the turbulent relative velocity (dust_growth.f90:94)
double growth_f_stokes(double x) {
    return (double)3.2f - 1.0 - x + 2.0 / (1. + x) * ((double)(1.0f / 2.6f) + (x * x * x) / ((double)1.6f + x));
}

// pairwise relative velocity dv(k, j) of one cell (dust_growth.f90:88-114)
struct GrowthCell {
    double T, rho, rho_cgs, cs_v, t_L, t_eta, Re, vambi, hs;
};

double growth_dv(const shark_gpu_config& g, const GrowthGrid& G, const GrowthCell& c, const double* ts,
                 const double* vx, const double* vy, const double* vz, const double* gam, int k, int j) {
    const double ul = unit_or_1(g.unit_l), ud = unit_or_1(g.unit_d), ut = unit_or_1(g.unit_t);
    const double um = ul * ul * ul * ud, uv = ul / ut;
    const double x_stokes = ts[j] / ts[k];
    const double f_Stokes = growth_f_stokes(x_stokes);
    const double St1 = ts[k] / c.t_L, St2 = ts[j] / c.t_L;
    const double a = g.grw_alpha_turb;
    const double rm = std::pow(c.Re, -0.5);
    const double vclass1 = a * c.cs_v * std::sqrt((St1 - St2) / (St1 + St2)) *
                           std::sqrt(St1 * St1 / (St1 + rm) - St2 * St2 / (St2 + rm));
    const double vclass2 = a * c.cs_v * std::sqrt(f_Stokes * St1);
    const double vclass3 = a * c.cs_v * std::sqrt(1.0 / (1.0 + St1) + 1.0 / (1.0 + St2));
    double vturb = vclass2;
    if (ts[k] < c.t_eta) vturb = vclass1;
    if (ts[k] > c.t_L) vturb = vclass3;
    const double X = (8.0 * phys::kB * c.T / pi) * (G.mk[k] * um + G.mk[j] * um) / (G.mk[k] * G.mk[j] * (um * um)) / (uv * uv);
    const double sX = std::sqrt(X);
    const double vbrow = std::sqrt(sX * sX);
    const double dxv = vx[k] - vx[j], dyv = vy[k] - vy[j], dzv = vz[k] - vz[j];
    const double vhydro = std::sqrt(dxv * dxv + dyv * dyv + dzv * dzv);
    double vad = 0.0;
    if (gam) {
        const double d = c.vambi / uv * (std::fabs(gam[k]) / std::sqrt(1.0 + gam[k] * gam[k]) -
                                         std::fabs(gam[j]) / std::sqrt(1.0 + gam[j] * gam[j]));
        vad = std::sqrt(d * d);
    }
    double dv = 0.0;
    if (g.grw_mode & SHARK_GROWTH_TURB) dv = vturb;
    if (g.grw_mode & SHARK_GROWTH_BROWNIAN) dv = std::sqrt(dv * dv + vbrow * vbrow);
    if (g.grw_mode & SHARK_GROWTH_DRIFT) dv = std::sqrt(dv * dv + vhydro * vhydro);
    if (g.grw_mode & SHARK_GROWTH_AMBIPOLAR) dv = std::sqrt(dv * dv + vad * vad);
    return dv;
}

int growth_bin(double m, double massmin, double eta, int cap) {
    const int b = (int)std::floor(std::log(m / massmin) / std::log(eta) + 1);
    return std::max(std::min(b, cap), 1);
}

// One cell's sub-cycled update of rho_k (1-based bin numbers as in the reference); returns the
// number of sub-steps.
int growth_cell(const shark_gpu_config& g, const GrowthGrid& G, const GrowthCell& c, double dt, double rho_gas,
                double* rd, const double* ts, const double* vx, const double* vy, const double* vz,
                const double* gam, std::vector<double>& drhodt) {
    const int N = g.ndust;
    const bool frag = (g.grw_mode & SHARK_GROWTH_FRAGMENTATION) != 0;
    const double ut = unit_or_1(g.unit_t);
    double time_growth = 0.0;
    int niter = 0;
    while (time_growth < dt && niter < 100000) {
        std::fill(drhodt.begin(), drhodt.end(), 0.0);
        niter = niter + 1;
        for (int k = 0; k < N; ++k) {
            const double m1 = G.mk[k], s1 = G.sk[k];
            for (int j = 0; j <= k; ++j) {
                const double m2 = G.mk[j], s2 = G.sk[j];
                const double dv = g.grw_kernel == 0 ? growth_dv(g, G, c, ts, vx, vy, vz, gam, k, j) : 0.0;
                double f_frag = 0.0, p_coag = 1.0;
                if (frag) {
                    const double Ecol = 0.5 * (m1 * m2) / (m1 + m2) * (dv * dv);
                    const double Ebr = (m1 + m2) / G.m_mono * G.Ebr_mono;
                    f_frag = fmax2(fmin2((Ecol - 0.1 * Ebr) / (4.9 * Ebr), 1.0), 0.0);
                }
                double dndt = (g.grw_clustered * g.grw_clustered) * pi * ((s1 + s2) * (s1 + s2)) * dv * rd[k] * rd[j] / m1 / m2;
                if (g.grw_kernel == 1) { p_coag = 1.0; f_frag = 0.0; dndt = rd[k] * rd[j] / m1 / m2; }
                else if (g.grw_kernel == 2) { p_coag = 1.0; f_frag = 0.0; dndt = (m1 + m2) * rd[k] * rd[j] / m1 / m2; }
                dndt = dndt / c.hs;
                if (k == j) dndt = dndt / 2.0;
                if (g.grw_kernel == 0) {
                    if (g.grw_eps_thr > 0.0 && (rd[k] < g.grw_eps_thr * rho_gas)) p_coag = 0.0;
                    if (g.grw_eps_thr > 0.0 && (rd[j] < g.grw_eps_thr * rho_gas)) p_coag = 0.0;
                    if (g.grw_eps_thr_frag > 0.0 && (rd[k] < g.grw_eps_thr_frag * rho_gas)) f_frag = 0.0;
                    if (g.grw_eps_thr_frag > 0.0 && (rd[j] < g.grw_eps_thr_frag * rho_gas)) f_frag = 0.0;
                }
                const double mc = (1.0 - f_frag) * (m1 + m2);
                const int ic1 = growth_bin(mc, G.massmin, G.eta, N);
                const int ic2 = std::max(std::min((int)std::floor(std::log(mc / G.massmin) / std::log(G.eta) + 1) + 1, N), 1);
                double eps_m = 1.0;
                if (ic1 < ic2) eps_m = fmin2((G.mk[ic2 - 1] - (1.0 - f_frag) * (m1 + m2)) / (G.mk[ic2 - 1] - G.mk[ic1 - 1]), 1.0);
                if (p_coag >= 0.0) {
                    const double st = g.grw_sticking;
                    drhodt[k] = drhodt[k] - p_coag * (1.0 - f_frag) * m1 * dndt * st - p_coag * f_frag * m1 * dndt;
                    drhodt[j] = drhodt[j] - p_coag * (1.0 - f_frag) * m2 * dndt * st - p_coag * f_frag * m2 * dndt;
                    if (f_frag < 1.0) {
                        drhodt[ic1 - 1] = drhodt[ic1 - 1] + eps_m * p_coag * (1.0 - f_frag) * (m1 + m2) * dndt * st;
                        drhodt[ic2 - 1] = drhodt[ic2 - 1] + (1. - eps_m) * p_coag * (1.0 - f_frag) * (m1 + m2) * dndt * st;
                    }
                }
                if ((frag && f_frag > 0.0) && p_coag > 0.) {
                    const int ifrag2 = std::max(std::min((int)std::floor(std::log(0.1 * f_frag * (m1 + m2) / G.massmin) /
                                                                         std::log(G.eta) + 1), ic1), 1);
                    for (int kd = 0; kd < ifrag2; ++kd)
                        drhodt[kd] = drhodt[kd] + p_coag * f_frag * (m1 + m2) * dndt * G.redis[(size_t)(ifrag2 - 1) * N + kd];
                }
            }
        }
        double dtg = 1e32;
        for (int k = 0; k < N; ++k)
            if (std::fabs(drhodt[k]) != 0.0) dtg = fmin2(dtg, rd[k] / std::fabs(drhodt[k]) * g.grw_cfl);
        dtg = fmin2(dtg, dt - time_growth);
        if (g.grw_dtcontrol > 0.0) dtg = fmin2(g.grw_dtcontrol * (double)365.25f * 3600 * 24 / ut, dt - time_growth);
        for (int k = 0; k < N; ++k) rd[k] = fmax2(rd[k] + drhodt[k] * dtg, rho_gas * g.dust_ratio_min);
        time_growth = time_growth + dtg;
    }
    return niter;
}

// per-cell inputs of the growth kernel for the setup (see the header comment)
void growth_inputs(oracle_state& s, int64_t i, GrowthCell& c) {
    const shark_gpu_config& g = s.cfg;
    const double ud = unit_or_1(g.unit_d), ut = unit_or_1(g.unit_t), ul = unit_or_1(g.unit_l);
    const double uv = ul / ut;
    c.hs = 1.0;
    if (g.setup == SHARK_SETUP_DISK_POLAR) {
        c.hs = std::sqrt(2.0 * pi) * (disk_h(g, s.radii_c[i]) * s.radii_c[i]);
        const double csc = s.cs[i] * uv;
        c.T = g.mu_gas * phys::mH * (csc * csc) / (g.gamma * phys::kB);
    } else {
        c.T = g.T_cloud;
    }
    c.rho = s.Q(i, s.irho) / c.hs;
    c.rho_cgs = c.rho * ud;
    const double cs_T = std::sqrt(g.gamma * phys::kB * c.T / (g.mu_gas * phys::mH));
    c.cs_v = cs_T / uv;
    const double lambJ = std::sqrt(3. * pi / (32. * phys_g::grav * c.rho_cgs)) * cs_T;
    c.vambi = 0.0;
    if (!s.eta_a.empty()) c.vambi = g.grw_delta_vambi * (phys::clight * phys::clight) * s.eta_a[i] / lambJ / (4.0 * pi);
    c.Re = 6.2e7 * std::sqrt(c.rho_cgs / (g.mu_gas * phys::mH) / 1e5) * std::sqrt(c.T / 10.0);
    if (g.setup == SHARK_SETUP_DISK_POLAR) c.t_L = 1.0 / std::sqrt(g.disk_mstar / powi(s.radii_c[i], 3));
    else c.t_L = std::sqrt(3. * pi / (32. * phys_g::grav * c.rho_cgs)) / ut;
    c.t_eta = c.t_L / std::sqrt(c.Re);
}

std::vector<int32_t> g_growth_iters;   // sub-steps per cell of the last growth call

void dust_growth(oracle_state& s) {
    const int N = s.ndust;
    const shark_gpu_config& g = s.cfg;
    const GrowthGrid G = growth_grid(g);
    const bool ambi = (g.grw_mode & SHARK_GROWTH_AMBIPOLAR) && !s.gamma_d.empty();
    if ((int64_t)g_growth_iters.size() != s.ncells) g_growth_iters.assign(s.ncells, 0);
#pragma omp parallel
    {
        std::vector<double> rd(N), ts(N), vx(N), vy(N), vz(N), gam(N), drhodt(N);
        GrowthCell c;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < s.ncells; ++i) {
            if (!s.active[i]) continue;
            growth_inputs(s, i, c);
            for (int k = 0; k < N; ++k) {
                rd[k] = s.U(i, s.irhod[k]);
                ts[k] = s.TSTOP(i, k);
                vx[k] = s.Q(i, s.ivdx[k]); vy[k] = s.Q(i, s.ivdy[k]); vz[k] = s.Q(i, s.ivdz[k]);
                if (ambi) gam[k] = s.gamma_d[(size_t)k * s.ncells + i];
            }
            g_growth_iters[i] = growth_cell(g, G, c, s.dt, s.U(i, s.irho), rd.data(), ts.data(), vx.data(), vy.data(),
                                            vz.data(), ambi ? gam.data() : nullptr, drhodt);
            for (int k = 0; k < N; ++k) s.U(i, s.irhod[k]) = rd[k];
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Driven turbulence of the dustyTurb box, 2D (the reference drives 1D modes only:
// src/turb/turb.f90:227-324 and solve.f90:129-146).  Solenoidal acceleration
//   a(x) = sum_m e_m [a_m cos(k_m.x) + b_m sin(k_m.x)],  e_m = (k_y, -k_x)/|k|,
// over the integer wave vectors kmin <= |k| L/(2 pi) <= kmax of one half plane; the coefficients
// follow an Ornstein-Uhlenbeck process with correlation time tcorr, advanced exactly each step,
//   c <- f c + s sqrt(1 - f^2) xi,  f = exp(-dt/tcorr),  xi ~ N(0,1),
// from the stationary law at t = 0; s = mach^(3/2) cs^2/(L sqrt(Nm)) (energy injection of the
// order of the dissipation (mach cs)^3/L at tcorr = L/cs).  Normal deviates by Box-Muller from
// the counter-based uniform of the ICs, counter ((step Nm + m) 2 + component) 2 + {0, 1}.  The
// kick is the reference's: gas momentum += rho a dt on the active cells, after dust growth.
// ---------------------------------------------------------------------------------------------
inline double hash_uniform(uint64_t seed, uint64_t counter);

void turb_modes(const shark_gpu_config& c, std::vector<double>& modes) {
    modes.clear();
    const int kmax = c.turb_kmax, kmin = c.turb_kmin;
    for (int kx = 0; kx <= kmax; ++kx)
        for (int ky = -kmax; ky <= kmax; ++ky) {
            if (kx == 0 && ky <= 0) continue;
            const double kk = std::sqrt((double)(kx * kx + ky * ky));
            if (kk < kmin || kk > kmax) continue;
            const double kxp = 2.0 * pi * kx / c.box_l, kyp = 2.0 * pi * ky / c.box_l_y;
            modes.push_back(kxp);
            modes.push_back(kyp);
            modes.push_back(std::sqrt(kxp * kxp + kyp * kyp));
        }
}

double ou_normal(uint64_t seed, uint64_t counter) {
    const double u1 = hash_uniform(seed, 2 * counter), u2 = hash_uniform(seed, 2 * counter + 1);
    return std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(2.0 * pi * u2);
}

double ou_sigma(const shark_gpu_config& c, int nm) {
    return std::pow(c.turb_mach, 1.5) * (c.cs0 * c.cs0) / c.box_l / std::sqrt((double)nm);
}

void turb_init(oracle_state& s) {
    turb_modes(s.cfg, s.ou_modes);
    const int nm = (int)s.ou_modes.size() / 3;
    const double sg = ou_sigma(s.cfg, nm);
    s.ou_coef.assign(2 * nm, 0.0);
    for (int m = 0; m < nm; ++m)
        for (int q = 0; q < 2; ++q) s.ou_coef[2 * m + q] = sg * ou_normal(s.cfg.turb_seed, (uint64_t)(m * 2 + q));
    s.ou_step = 0;
}

void turb_kick(oracle_state& s) {
    const int nm = (int)s.ou_modes.size() / 3;
    if (nm == 0) return;
    s.ou_step = s.ou_step + 1;
    const double f = std::exp(-s.dt / s.cfg.turb_tcorr);
    const double sg = ou_sigma(s.cfg, nm) * std::sqrt(1.0 - f * f);
    for (int m = 0; m < nm; ++m)
        for (int q = 0; q < 2; ++q)
            s.ou_coef[2 * m + q] = f * s.ou_coef[2 * m + q] +
                                   sg * ou_normal(s.cfg.turb_seed, (uint64_t)((s.ou_step * nm + m) * 2 + q));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        const double x = s.POS(i, 0), y = s.POS(i, 1);
        double ax = 0.0, ay = 0.0;
        for (int m = 0; m < nm; ++m) {
            const double kxp = s.ou_modes[3 * m], kyp = s.ou_modes[3 * m + 1], kk = s.ou_modes[3 * m + 2];
            const double ph = kxp * x + kyp * y;
            const double w = s.ou_coef[2 * m] * std::cos(ph) + s.ou_coef[2 * m + 1] * std::sin(ph);
            ax = ax + kyp / kk * w;
            ay = ay - kxp / kk * w;
        }
        const double rho = s.U(i, s.irho);
        s.U(i, s.ivx) = s.U(i, s.ivx) + rho * ax * s.dt;
        s.U(i, s.ivy) = s.U(i, s.ivy) + rho * ay * s.dt;
    }
}

// update_force_setup of disk_polar (disk_polar/setup.f90:364-398) without planet/self-gravity:
// point-mass gravity -Mstar/r^2 on gas and dust.
void disk_force(oracle_state& s) {
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        const double g = -s.cfg.disk_mstar / sq(s.radii_c[i]);
        s.FORCE(i, 0) = g; s.FORCE(i, 1) = 0.0; s.FORCE(i, 2) = 0.0;
        for (int k = 0; k < s.ndust; ++k) { s.FDUST(i, 0, k) = g; s.FDUST(i, 1, k) = 0.0; s.FDUST(i, 2, k) = 0.0; }
    }
}

// update_force_setup of the Cartesian disk (disk/setup.f90) without a planet: the star's
// softened gravity -Mstar (xx, yy)/rr^3 on gas and dust (active cells; the ghosts keep 0).
void disk_cart_force(oracle_state& s) {
    const double M = s.cfg.disk_mstar;
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        const CdiskCell c = cdisk_cell(s, i);
        const double fx = -M * c.xx / powi(c.rr, 3), fy = -M * c.yy / powi(c.rr, 3);
        s.FORCE(i, 0) = fx; s.FORCE(i, 1) = fy; s.FORCE(i, 2) = 0.0;
        for (int k = 0; k < s.ndust; ++k) { s.FDUST(i, 0, k) = fx; s.FDUST(i, 1, k) = fy; s.FDUST(i, 2, k) = 0.0; }
    }
}

// update_force_setup (SI/setup.f90:335-368); SOD and DUSTYWAVE leave force at zero.
void update_force_setup(oracle_state& s) {
    if (s.cfg.setup == SHARK_SETUP_DISK_POLAR) { disk_force(s); return; }
    if (s.cfg.setup == SHARK_SETUP_DISK_CART) { disk_cart_force(s); return; }
    if (s.cfg.setup != SHARK_SETUP_SI) return;
    const double qs = s.cfg.si_q_shear, om = s.cfg.si_omega, r0 = s.cfg.si_rad0, eta = s.cfg.si_eta_stream;
    const bool drag = s.flag(SHARK_FLAG_DRAG);
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        double xc = s.POS(i, 0) - half * s.box_l;
        s.FORCE(i, 0) = 2.0 * qs * sq(om) * xc - 2.0 * om * s.Q(i, s.ivz) - 2.0 * r0 * om * eta;
        s.FORCE(i, 1) = 0.0;
        s.FORCE(i, 2) = 2.0 * om * s.Q(i, s.ivx);
        for (int k = 0; k < s.ndust; ++k) {
            s.FDUST(i, 0, k) = 2.0 * qs * sq(om) * xc - 2.0 * om * s.Q(i, s.ivdz[k]);
            s.FDUST(i, 1, k) = 0.0;
            s.FDUST(i, 2, k) = 2.0 * om * s.Q(i, s.ivdx[k]);
            if (!drag) {
                double ts = s.TSTOP(i, k), rr = s.Q(i, s.irhod[k]) / s.Q(i, s.irho);
                s.FORCE(i, 0) = s.FORCE(i, 0) - rr * (s.Q(i, s.ivx) - s.Q(i, s.ivdx[k])) / ts;
                s.FORCE(i, 1) = s.FORCE(i, 1) - rr * (s.Q(i, s.ivy) - s.Q(i, s.ivdy[k])) / ts;
                s.FORCE(i, 2) = s.FORCE(i, 2) - rr * (s.Q(i, s.ivz) - s.Q(i, s.ivdz[k])) / ts;
                s.FDUST(i, 0, k) = s.FDUST(i, 0, k) + (s.Q(i, s.ivx) - s.Q(i, s.ivdx[k])) / ts;
                s.FDUST(i, 1, k) = s.FDUST(i, 1, k) + (s.Q(i, s.ivy) - s.Q(i, s.ivdy[k])) / ts;
                s.FDUST(i, 2, k) = s.FDUST(i, 2, k) + (s.Q(i, s.ivz) - s.Q(i, s.ivdz[k])) / ts;
            }
        }
    }
}

// setup_inloop of disk_polar (disk_polar/setup.f90:206-284): relax density and in-plane velocities
// of gas and dust towards the initial state inside r_relax with t_rel = n_rel orbits (measured
// from the inner radius), then reset the radial ghosts and the first active column to the
// initial state of the first active column.
void disk_inloop(oracle_state& s) {
    const double Mstar = s.cfg.disk_mstar, n_rel = s.cfg.disk_n_rel, r_relax = s.cfg.disk_r_relax;
    const double sm = s.cfg.inner_r;
    auto UI = [&](int64_t i, int v) { return s.u_init[(size_t)v * s.ncells + i]; };
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        const double rc = s.radii_c[i];
        if (!(rc < r_relax)) continue;
        const double t_rel = n_rel * 2.0 * pi / (std::sqrt(Mstar / powi(rc, 3))) - n_rel * 2.0 * pi / (std::sqrt(Mstar / powi(sm, 3)));
        const double e = std::exp(-s.dt / t_rel);
        auto relax = [&](int ir, int ivx_, int ivy_) {
            const double rho_init = UI(i, ir), vx_init = UI(i, ivx_) / rho_init, vy_init = UI(i, ivy_) / rho_init;
            const double rho_old = s.U(i, ir), vx_old = s.U(i, ivx_) / rho_old, vy_old = s.U(i, ivy_) / rho_old;
            const double rho_new = (rho_init) * (1.0 - e) + rho_old * e;
            const double vx_new = (vx_init) * (1.0 - e) + vx_old * e;
            const double vy_new = (vy_init) * (1.0 - e) + vy_old * e;
            s.U(i, ir) = rho_new;
            s.U(i, ivx_) = rho_new * vx_new;
            s.U(i, ivy_) = rho_new * vy_new;
        };
        relax(s.irho, s.ivx, s.ivy);
        for (int k = 0; k < s.ndust; ++k) relax(s.irhod[k], s.ivdx[k], s.ivdy[k]);
    }
    for (int ix = 0; ix <= s.first_active; ++ix)
        for (int iy = s.first_active_y; iy <= s.last_active_y; ++iy)
            for (int v = 0; v < s.nvar; ++v) s.U(s.icell(ix, iy), v) = UI(s.icell(s.first_active, iy), v);
}

// setup_inloop of the Cartesian disk (disk/setup.f90) as written, with its relaxation rate 0:
// the cells with rr < buffer_in box_l or rr > buffer_out box_l are reset to rho_ana =
// Sigma_0 R_0/rr (1/100 of the edge value beyond R_out = frac_R_disk box_l), the momenta
// (-y_soft, x_soft) v_ana with v_ana = -Omega rho_ana, the energy slot rho_ana cs0^2, and every
// dust species to dust2gas times that with (-yy, xx) in place of the softened offsets.  (With
// v_ana = -Omega rho_ana the buffers turn the other way round from the initial rotation; the
// vz momenta are not touched.)  dust_to is the first species' initial dust-to-gas ratio.
void disk_cart_inloop(oracle_state& s) {
    const double M = s.cfg.disk_mstar, hr = s.cfg.disk_hoverr;
    const double R_out = s.cfg.cdisk_frac_r_disk * s.box_l;
    const double bin = s.cfg.cdisk_buffer_in * s.box_l, bout = s.cfg.cdisk_buffer_out * s.box_l;
    const double rate = 0.0;
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        const CdiskCell c = cdisk_cell(s, i);
        const double rr = c.rr;
        if (!(rr < bin || rr > bout)) continue;
        const double x_soft = c.xx * rr / c.r_cyl, y_soft = c.yy * rr / c.r_cyl;
        const double H = hr * rr;
        const double Omega = std::sqrt(M / powi(rr, 3));
        const double cs0 = H * Omega;
        double rho_ana = s.cfg.disk_sigma0 * (s.cfg.disk_r0 / rr);
        if (rr > R_out) rho_ana = s.cfg.disk_sigma0 * (s.cfg.disk_r0 / R_out) / 100.0;
        const double v_ana = -Omega * rho_ana;
        s.U(i, s.irho) = rho_ana + (s.U(i, s.irho) - rho_ana) * rate;
        s.U(i, s.ivx) = -y_soft * v_ana + (s.U(i, s.ivx) + c.yy * v_ana) * rate;
        s.U(i, s.ivy) = x_soft * v_ana + (s.U(i, s.ivy) - c.xx * v_ana) * rate;
        s.U(i, s.iP) = (rho_ana + (s.U(i, s.irho) - rho_ana) * rate) * sq(cs0);
        for (int k = 0; k < s.ndust; ++k) {
            const double dust_to = s.cfg.dust_eps[0];
            s.U(i, s.irhod[k]) = dust_to * rho_ana + (s.U(i, s.irhod[k]) - rho_ana * dust_to) * rate;
            s.U(i, s.ivdx[k]) = -c.yy * v_ana * dust_to + (s.U(i, s.ivdx[k]) + dust_to * c.yy * v_ana) * rate;
            s.U(i, s.ivdy[k]) = c.xx * v_ana * dust_to + (s.U(i, s.ivdy[k]) - dust_to * c.xx * v_ana) * rate;
        }
    }
}

// setup_inloop (SI/setup.f90:299-332): Crank-Nicolson rotation, only without force_kick.
void setup_inloop(oracle_state& s) {
    if (s.cfg.setup == SHARK_SETUP_DISK_POLAR) { disk_inloop(s); return; }
    if (s.cfg.setup == SHARK_SETUP_DISK_CART) { disk_cart_inloop(s); return; }
    if (s.cfg.setup != SHARK_SETUP_SI) return;
    if (s.flag(SHARK_FLAG_FORCE_KICK)) return;
    const double qs = s.cfg.si_q_shear, om = s.cfg.si_omega, r0 = s.cfg.si_rad0, eta = s.cfg.si_eta_stream;
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        double u = s.U(i, s.ivz) / s.U(i, s.irho);
        double v = s.U(i, s.ivx) / s.U(i, s.irho);
        double d = s.U(i, s.irho);
        double Ohmdt = om * s.dt;
        double AA = 2.0 * qs * om * (s.POS(i, 0) - half * s.box_l) - 2.0 * r0 * eta;
        s.U(i, s.ivz) = d * (u * (1. - sq(Ohmdt)) + 2. * v * Ohmdt + AA * sq(Ohmdt)) / (1. + sq(Ohmdt));
        s.U(i, s.ivx) = d * (v * (1. - sq(Ohmdt)) - 2. * u * Ohmdt + AA * Ohmdt) / (1. + sq(Ohmdt));
        AA = 2.0 * qs * om * (s.POS(i, 0) - half * s.box_l);
        for (int k = 0; k < s.ndust; ++k) {
            u = s.U(i, s.ivdz[k]) / s.U(i, s.irhod[k]);
            v = s.U(i, s.ivdx[k]) / s.U(i, s.irhod[k]);
            d = s.U(i, s.irhod[k]);
            s.U(i, s.ivdz[k]) = d * (u * (1. - sq(Ohmdt)) + 2. * v * Ohmdt + AA * sq(Ohmdt)) / (1. + sq(Ohmdt));
            s.U(i, s.ivdx[k]) = d * (v * (1. - sq(Ohmdt)) - 2. * u * Ohmdt + AA * Ohmdt) / (1. + sq(Ohmdt));
        }
    }
}

// ---------------------------------------------------------------------------------------------
// courant (src/solver/courant.f90:11-124), non-MHD, no gravity.  Serial like the reference.
// Note `vv` in the force limiter is the LAST species' velocity sum (overwritten in the dust loop).
// ---------------------------------------------------------------------------------------------
void courant(oracle_state& s) {
    const double CFL = s.cfg.cfl;
    const bool fk = s.flag(SHARK_FLAG_FORCE_KICK);
    double dt = 2e44;
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        double dxx;
        if (s.ndim == 1) dxx = s.DX(i, 0);
        else if (s.cfg.geom == 2) dxx = fmin2(s.DX(i, 0), s.radii_c[i] * s.DX(i, 1));
        else dxx = fmin2(s.DX(i, 0), s.DX(i, 1));
        double vv = std::fabs(s.Q(i, s.ivx)) + std::fabs(s.Q(i, s.ivy)) + std::fabs(s.Q(i, s.ivz));
        double vmax = s.cs[i] + vv;
        double ca = 0.0;
        for (int k = 0; k < s.ndust; ++k) {
            vv = std::fabs(s.Q(i, s.ivdx[k])) + std::fabs(s.Q(i, s.ivdy[k])) + std::fabs(s.Q(i, s.ivdz[k]));
            vmax = fmax2(vmax, ca + vv);
        }
        dt = fmin2(dt, CFL * dxx / std::fabs(vmax));
        if (fk) {
            double force_max = std::sqrt(sq(s.FORCE(i, 0)) + sq(s.FORCE(i, 1)) + sq(s.FORCE(i, 2)));
            for (int k = 0; k < s.ndust; ++k)
                force_max = fmax2(force_max, std::sqrt(sq(s.FDUST(i, 0, k)) + sq(s.FDUST(i, 1, k)) + sq(s.FDUST(i, 2, k))));
            if (vv != 0.0) {
                double fratio = fmax2(force_max * dxx / sq(vv), 1e-3);
                dt = fmin2(dt, CFL * dxx / vv * (std::sqrt(1.0 + 2.0 * CFL * fratio) - 1.0) / fratio);
            }
        }
    }
    s.dt = dt;
}

// kick (src/solver/force_kicks.f90:2-41); the energy fix-up condition is always true in practice
// (iso_cs.ne.1 .or. non_standard_eos.ne.1 with non_standard_eos = -1).
void kick(oracle_state& s, double coeffdt) {
    const double dt = s.dt;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        double rho = s.U(i, s.irho);
        double energy_old = half * sq(s.U(i, s.ivx)) / rho + half * sq(s.U(i, s.ivy)) / rho + half * sq(s.U(i, s.ivz)) / rho;
        s.U(i, s.ivx) = s.U(i, s.ivx) + rho * coeffdt * dt * s.FORCE(i, 0);
        s.U(i, s.ivy) = s.U(i, s.ivy) + rho * coeffdt * dt * s.FORCE(i, 1);
        s.U(i, s.ivz) = s.U(i, s.ivz) + rho * coeffdt * dt * s.FORCE(i, 2);
        double energy_new = half * sq(s.U(i, s.ivx)) / rho + half * sq(s.U(i, s.ivy)) / rho + half * sq(s.U(i, s.ivz)) / rho;
        s.U(i, s.iP) = s.U(i, s.iP) + (energy_new - energy_old);
        for (int k = 0; k < s.ndust; ++k) {
            double rd = s.U(i, s.irhod[k]);
            s.U(i, s.ivdx[k]) = s.U(i, s.ivdx[k]) + rd * coeffdt * dt * s.FDUST(i, 0, k);
            s.U(i, s.ivdy[k]) = s.U(i, s.ivdy[k]) + rd * coeffdt * dt * s.FDUST(i, 1, k);
            s.U(i, s.ivdz[k]) = s.U(i, s.ivdz[k]) + rd * coeffdt * dt * s.FDUST(i, 2, k);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// predictor (src/solver/godunov.f90:7-629), non-MHD, no gravity, no dust passive scalars.
// In the reference, drx..dwy are OMP-private and zeroed once per thread; in 1D the y-slopes are
// never assigned so they stay 0 for gas and dust alike.  The Cartesian source block
// (`#if GE0M==0`, a typo that is always true) is evaluated first and, for GEOM==2, overwritten.
// ---------------------------------------------------------------------------------------------
void predictor(oracle_state& s) {
    const double gamma = s.cfg.gamma, smallP = s.cfg.smallp, dt = s.dt;
    const int N = s.ndust, nvar = s.nvar, st = s.cfg.slope_type;
    const bool fk = s.flag(SHARK_FLAG_FORCE_KICK), polar = (s.cfg.geom == 2), two_d = (s.ndim == 2);
    std::fill(s.qm.begin(), s.qm.end(), 0.0);
    std::fill(s.qp.begin(), s.qp.end(), 0.0);
#pragma omp parallel
    {
        std::vector<double> dq((size_t)nvar * 2, 0.0);  // dq(i,:,:) of the current cell
#pragma omp for schedule(static)
        for (int64_t i = 0; i < s.ncells; ++i) {
            if (!s.active_pred[i]) continue;
            const int ix = s.ixx(i), iy = s.iyy(i);
            const double radius_polar = polar ? s.radii_c[i] : 1.0;
            std::fill(dq.begin(), dq.end(), 0.0);
            if (st > 0) {
                for (int v = 0; v < nvar; ++v) {
                    int64_t il = s.icell(ix - 1, iy), ir = s.icell(ix + 1, iy);
                    dq[v] = slope_limit(st, 2.0 * (s.Q(i, v) - s.Q(il, v)) / (s.DX(i, 0) + s.DX(il, 0)),
                                        2.0 * (s.Q(ir, v) - s.Q(i, v)) / (s.DX(ir, 0) + s.DX(i, 0)));
                    if (two_d) {
                        il = s.icell(ix, iy - 1);
                        ir = s.icell(ix, iy + 1);
                        dq[nvar + v] = slope_limit(st, 2.0 * (s.Q(i, v) - s.Q(il, v)) / (s.DX(i, 1) + s.DX(il, 1)),
                                                   2.0 * (s.Q(ir, v) - s.Q(i, v)) / (s.DX(ir, 1) + s.DX(i, 1))) /
                                       radius_polar;
                    }
                }
            }
            double drx, dry = 0, dpx, dpy = 0, dux, duy = 0, dvx, dvy = 0, dwx, dwy = 0;
            double r_rho = s.Q(i, s.irho);
            double u = s.Q(i, s.ivx);
            dux = dq[s.ivx];
            drx = dq[s.irho];
            double w = s.Q(i, s.ivz);
            dwx = dq[s.ivz];
            double v = s.Q(i, s.ivy);
            dvx = dq[s.ivy];
            double p = s.Q(i, s.iP);
            dpx = dq[s.iP];
            const double csi = s.cs[i];
            if (s.cfg.iso_cs == 1) {
                p = s.Q(i, s.irho) * sq(csi);
                dpx = dq[s.irho] * sq(csi);
            }
            if (two_d) {
                duy = dq[nvar + s.ivx];
                dry = dq[nvar + s.irho];
                dvy = dq[nvar + s.ivy];
                dpy = dq[nvar + s.iP];
                dwy = dq[nvar + s.ivz];
                if (s.cfg.iso_cs == 1) dpy = dq[nvar + s.irho] * sq(csi);
            }
            if (fk) {
                u = u + s.FORCE(i, 0) * half * dt;
                v = v + s.FORCE(i, 1) * half * dt;
                w = w + s.FORCE(i, 2) * half * dt;
            }
            double sr0 = -u * drx - v * dry - (dux + dvy) * r_rho;
            double sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma * p;
            double su0 = -u * dux - v * duy - (dpx) / r_rho;
            double sv0 = -u * dvx - v * dvy - (dpy) / r_rho;
            double sw0 = -u * dwx - v * dwy;
            if (polar) {
                sr0 = -u * drx - v * dry - (dux + dvy) * r_rho - r_rho * u / radius_polar;
                sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma * p - gamma * p * u / radius_polar;
                su0 = -u * dux - v * duy - (dpx) / r_rho + (sq(v)) / radius_polar;
                sv0 = -u * dvx - v * dvy - (dpy) / r_rho - u * v / radius_polar;
                sw0 = -u * dwx - v * dwy;
            }
            double dx_loc = s.DX(i, 0);
            s.QM(i, s.irho, 0) = r_rho + half * dt * sr0 + half * drx * dx_loc;
            s.QM(i, s.ivx, 0) = u + half * dt * su0 + half * dux * dx_loc;
            s.QM(i, s.iP, 0) = fmax2(p + half * dt * sp0 + half * dpx * dx_loc, smallP);
            s.QM(i, s.ivy, 0) = v + half * dt * sv0 + half * dvx * dx_loc;
            s.QM(i, s.ivz, 0) = w + half * dt * sw0 + half * dwx * dx_loc;
            s.QP(i, s.irho, 0) = r_rho + half * dt * sr0 - half * drx * dx_loc;
            s.QP(i, s.ivx, 0) = u + half * dt * su0 - half * dux * dx_loc;
            s.QP(i, s.iP, 0) = fmax2(p + half * dt * sp0 - half * dpx * dx_loc, smallP);
            s.QP(i, s.ivy, 0) = v + half * dt * sv0 - half * dvx * dx_loc;
            s.QP(i, s.ivz, 0) = w + half * dt * sw0 - half * dwx * dx_loc;
            if (two_d) {
                dx_loc = radius_polar * s.DX(i, 1);
                s.QM(i, s.irho, 1) = r_rho + half * dt * sr0 + half * dry * dx_loc;
                s.QM(i, s.ivx, 1) = u + half * dt * su0 + half * duy * dx_loc;
                s.QM(i, s.iP, 1) = fmax2(p + half * dt * sp0 + half * dpy * dx_loc, smallP);
                s.QM(i, s.ivy, 1) = v + half * dt * sv0 + half * dvy * dx_loc;
                s.QM(i, s.ivz, 1) = w + half * dt * sw0 + half * dwy * dx_loc;
                s.QP(i, s.irho, 1) = r_rho + half * dt * sr0 - half * dry * dx_loc;
                s.QP(i, s.ivx, 1) = u + half * dt * su0 - half * duy * dx_loc;
                s.QP(i, s.iP, 1) = fmax2(p + half * dt * sp0 - half * dpy * dx_loc, smallP);
                s.QP(i, s.ivy, 1) = v + half * dt * sv0 - half * dvy * dx_loc;
                s.QP(i, s.ivz, 1) = w + half * dt * sw0 - half * dwy * dx_loc;
            }
            // dust (godunov.f90:359-510)
            for (int k = 0; k < N; ++k) {
                const int irs = s.irhod[k], ivxs = s.ivdx[k], ivys = s.ivdy[k], ivzs = s.ivdz[k];
                r_rho = s.Q(i, irs);
                u = s.Q(i, ivxs);
                dux = dq[ivxs];
                drx = dq[irs];
                v = s.Q(i, ivys);
                dvx = dq[ivys];
                w = s.Q(i, ivzs);
                dwx = dq[ivzs];
                if (two_d) {
                    dry = dq[nvar + irs];
                    duy = dq[nvar + ivxs];
                    dvy = dq[nvar + ivys];
                    dwy = dq[nvar + ivzs];
                }
                if (fk) {
                    u = u + s.FDUST(i, 0, k) * half * dt;
                    v = v + s.FDUST(i, 1, k) * half * dt;
                    w = w + s.FDUST(i, 2, k) * half * dt;
                }
                sr0 = -u * drx - v * dry - (dux + dvy) * r_rho;
                su0 = -u * dux - v * duy;
                sv0 = -u * dvx - v * dvy;
                sw0 = -u * dwx - v * dwy;
                if (polar) {
                    sr0 = sr0 - r_rho * u / radius_polar;
                    su0 = su0 + sq(v) / radius_polar;
                    sv0 = sv0 - u * v / radius_polar;
                }
                dx_loc = s.DX(i, 0);
                s.QM(i, irs, 0) = r_rho + half * dt * sr0 + half * drx * dx_loc;
                s.QM(i, ivxs, 0) = u + half * dt * su0 + half * dux * dx_loc;
                s.QM(i, ivys, 0) = v + half * dt * sv0 + half * dvx * dx_loc;
                s.QM(i, ivzs, 0) = w + half * dt * sw0 + half * dwx * dx_loc;
                s.QP(i, irs, 0) = r_rho + half * dt * sr0 - half * drx * dx_loc;
                s.QP(i, ivxs, 0) = u + half * dt * su0 - half * dux * dx_loc;
                s.QP(i, ivys, 0) = v + half * dt * sv0 - half * dvx * dx_loc;
                s.QP(i, ivzs, 0) = w + half * dt * sw0 - half * dwx * dx_loc;
                if (two_d) {
                    dx_loc = radius_polar * s.DX(i, 1);
                    s.QM(i, irs, 1) = r_rho + half * dt * sr0 + half * dry * dx_loc;
                    s.QM(i, ivxs, 1) = u + half * dt * su0 + half * duy * dx_loc;
                    s.QM(i, ivys, 1) = v + half * dt * sv0 + half * dvy * dx_loc;
                    s.QM(i, ivzs, 1) = w + half * dt * sw0 + half * dwy * dx_loc;
                    s.QP(i, irs, 1) = r_rho + half * dt * sr0 - half * dry * dx_loc;
                    s.QP(i, ivxs, 1) = u + half * dt * su0 - half * duy * dx_loc;
                    s.QP(i, ivys, 1) = v + half * dt * sv0 - half * dvy * dx_loc;
                    s.QP(i, ivzs, 1) = w + half * dt * sw0 - half * dwy * dx_loc;
                }
            }
            // isothermal pressure on the faces (godunov.f90:606-611)
            if (s.cfg.iso_cs == 1) {
                for (int d = 0; d < s.ndim; ++d) {
                    s.QP(i, s.iP, d) = sq(csi) * s.QP(i, s.irho, d);
                    s.QM(i, s.iP, d) = sq(csi) * s.QM(i, s.irho, d);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Riemann solvers (src/solver/solvers.f90), non-MHD branches.
// ---------------------------------------------------------------------------------------------
struct GasFace {  // the five gas fluxes in (rho, normal mom, transverse mom, z mom, energy) order
    double rho, mn, mt, mz, e;
};

// solver_llf (solvers.f90:4-155)
GasFace solver_llf(double gamma, double rho_lft, double u_lft, double v_lft, double w_lft, double P_lft,
                   double rho_rgt, double u_rgt, double v_rgt, double w_rgt, double P_rgt, double csl, double csr) {
    double mom_u_rgt = rho_rgt * u_rgt, mom_u_lft = rho_lft * u_lft;
    double E_rgt = P_rgt / (gamma - 1.0) + half * rho_rgt * sq(u_rgt);
    double E_lft = P_lft / (gamma - 1.0) + half * rho_lft * sq(u_lft);
    double mom_v_rgt = rho_rgt * v_rgt, mom_v_lft = rho_lft * v_lft;
    E_rgt = E_rgt + half * rho_rgt * sq(v_rgt);
    E_lft = E_lft + half * rho_lft * sq(v_lft);
    double mom_w_rgt = rho_rgt * w_rgt, mom_w_lft = rho_lft * w_lft;
    E_rgt = E_rgt + half * rho_rgt * sq(w_rgt);
    E_lft = E_lft + half * rho_lft * sq(w_lft);
    double flx_rho_rgt = rho_rgt * u_rgt, flx_rho_lft = rho_lft * u_lft;
    double flx_mom_u_rgt = (rho_rgt * sq(u_rgt) + P_rgt), flx_mom_u_lft = (rho_lft * sq(u_lft) + P_lft);
    double flx_mom_v_rgt = rho_rgt * u_rgt * v_rgt, flx_mom_v_lft = rho_lft * u_lft * v_lft;
    double flx_mom_w_rgt = rho_rgt * u_rgt * w_rgt, flx_mom_w_lft = rho_lft * u_lft * w_lft;
    double flx_P_rgt = (E_rgt + P_rgt) * u_rgt, flx_P_lft = (E_lft + P_lft) * u_lft;
    double lam = fmax2(std::fabs(u_lft) + csl, std::fabs(u_rgt) + csr);
    GasFace f;
    f.rho = half * (flx_rho_lft + flx_rho_rgt) - half * lam * (rho_rgt - rho_lft);
    f.mn = half * (flx_mom_u_lft + flx_mom_u_rgt) - half * lam * (mom_u_rgt - mom_u_lft);
    f.mt = half * (flx_mom_v_lft + flx_mom_v_rgt) - half * lam * (mom_v_rgt - mom_v_lft);
    f.mz = half * (flx_mom_w_lft + flx_mom_w_rgt) - half * lam * (mom_w_rgt - mom_w_lft);
    f.e = half * (flx_P_lft + flx_P_rgt) - half * lam * (E_rgt - E_lft);
    return f;
}

// solver_hll (solvers.f90:157-306)
GasFace solver_hll(double gamma, double rho_lft, double u_lft, double v_lft, double w_lft, double P_lft,
                   double rho_rgt, double u_rgt, double v_rgt, double w_rgt, double P_rgt, double csl, double csr) {
    double mom_u_rgt = rho_rgt * u_rgt, mom_u_lft = rho_lft * u_lft;
    double E_rgt = P_rgt / (gamma - 1.0) + half * rho_rgt * sq(u_rgt);
    double E_lft = P_lft / (gamma - 1.0) + half * rho_lft * sq(u_lft);
    double mom_v_rgt = rho_rgt * v_rgt, mom_v_lft = rho_lft * v_lft;
    E_rgt = E_rgt + half * rho_rgt * sq(v_rgt);
    E_lft = E_lft + half * rho_lft * sq(v_lft);
    double mom_w_rgt = rho_rgt * w_rgt, mom_w_lft = rho_lft * w_lft;
    E_rgt = E_rgt + half * rho_rgt * sq(w_rgt);
    E_lft = E_lft + half * rho_lft * sq(w_lft);
    double flx_rho_rgt = rho_rgt * u_rgt, flx_rho_lft = rho_lft * u_lft;
    double flx_mom_u_rgt = (rho_rgt * sq(u_rgt) + P_rgt), flx_mom_u_lft = (rho_lft * sq(u_lft) + P_lft);
    double flx_mom_v_rgt = rho_rgt * u_rgt * v_rgt, flx_mom_v_lft = rho_lft * u_lft * v_lft;
    double flx_mom_w_rgt = rho_rgt * u_rgt * w_rgt, flx_mom_w_lft = rho_lft * u_lft * w_lft;
    double flx_P_rgt = (E_rgt + P_rgt) * u_rgt, flx_P_lft = (E_lft + P_lft) * u_lft;
    double S_lft = fmin2(fmin2(u_lft, u_rgt) - fmax2(csl, csr), 0.0);
    double S_rgt = fmax2(fmax2(u_lft, u_rgt) + fmax2(csl, csr), 0.0);
    GasFace f;
    f.rho = (S_rgt * flx_rho_lft - S_lft * flx_rho_rgt + S_rgt * S_lft * (rho_rgt - rho_lft)) / (S_rgt - S_lft);
    f.mn = (S_rgt * flx_mom_u_lft - S_lft * flx_mom_u_rgt + S_rgt * S_lft * (mom_u_rgt - mom_u_lft)) / (S_rgt - S_lft);
    f.mt = (S_rgt * flx_mom_v_lft - S_lft * flx_mom_v_rgt + S_rgt * S_lft * (mom_v_rgt - mom_v_lft)) / (S_rgt - S_lft);
    f.mz = (S_rgt * flx_mom_w_lft - S_lft * flx_mom_w_rgt + S_rgt * S_lft * (mom_w_rgt - mom_w_lft)) / (S_rgt - S_lft);
    f.e = (S_rgt * flx_P_lft - S_lft * flx_P_rgt + S_rgt * S_lft * (E_rgt - E_lft)) / (S_rgt - S_lft);
    return f;
}

// solver_hllc (solvers.f90:308-500)
GasFace solver_hllc(double gamma, double rho_lft, double u_lft, double v_lft, double w_lft, double P_lft,
                    double rho_rgt, double u_rgt, double v_rgt, double w_rgt, double P_rgt, double csl, double csr) {
    double E_rgt = P_rgt / (gamma - 1.0) + half * rho_rgt * sq(u_rgt) + half * rho_rgt * sq(v_rgt) + half * rho_rgt * sq(w_rgt);
    double E_lft = P_lft / (gamma - 1.0) + half * rho_lft * sq(u_lft) + half * rho_lft * sq(v_lft) + half * rho_lft * sq(w_lft);
    double S_lft = fmin2(fmin2(u_lft, u_rgt) - fmax2(csl, csr), 0.0);
    double S_rgt = fmax2(fmax2(u_lft, u_rgt) + fmax2(csl, csr), 0.0);
    double hllc_l = rho_lft * (u_lft - S_lft);
    double hllc_r = rho_rgt * (S_rgt - u_rgt);
    double ustar = (hllc_r * u_rgt + hllc_l * u_lft + (P_lft - P_rgt)) / (hllc_r + hllc_l);
    double Pstar = (hllc_r * P_lft + hllc_l * P_rgt + hllc_l * hllc_r * (u_lft - u_rgt)) / (hllc_r + hllc_l);
    double rhostarleft = rho_lft * (S_lft - u_lft) / (S_lft - ustar);
    double estarleft = ((S_lft - u_lft) * E_lft - P_lft * u_lft + Pstar * ustar) / (S_lft - ustar);
    double rhostarright = rho_rgt * (S_rgt - u_rgt) / (S_rgt - ustar);
    double estarright = ((S_rgt - u_rgt) * E_rgt - P_rgt * u_rgt + Pstar * ustar) / (S_rgt - ustar);
    double r_o, u_o, P_o, e_o;
    if (S_lft > 0.0) { r_o = rho_lft; u_o = u_lft; P_o = P_lft; e_o = E_lft; }
    else if (ustar > 0.0) { r_o = rhostarleft; u_o = ustar; P_o = Pstar; e_o = estarleft; }
    else if (S_rgt > 0.0) { r_o = rhostarright; u_o = ustar; P_o = Pstar; e_o = estarright; }
    else { r_o = rho_rgt; u_o = u_rgt; P_o = P_rgt; e_o = E_rgt; }
    GasFace f;
    f.rho = r_o * u_o;
    f.mn = r_o * u_o * u_o + P_o;
    f.e = (e_o + P_o) * u_o;
    if (ustar > 0.0) { f.mt = r_o * u_o * v_lft; f.mz = r_o * u_o * w_lft; }
    else { f.mt = r_o * u_o * v_rgt; f.mz = r_o * u_o * w_rgt; }
    return f;
}

struct DustFace { double rho, mn, mt, mz; };

// solver_dust_Huang_Bai (solvers.f90:506-698), one species.
DustFace solver_dust_hb(double rho_lft, double u_lft, double v_lft, double w_lft,
                        double rho_rgt, double u_rgt, double v_rgt, double w_rgt) {
    double flx_rho_rgt = rho_rgt * u_rgt, flx_rho_lft = rho_lft * u_lft;
    double flx_mom_u_rgt = rho_rgt * sq(u_rgt), flx_mom_u_lft = rho_lft * sq(u_lft);
    double flx_mom_v_rgt = rho_rgt * u_rgt * v_rgt, flx_mom_v_lft = rho_lft * u_lft * v_lft;
    double flx_mom_w_rgt = rho_rgt * u_rgt * w_rgt, flx_mom_w_lft = rho_lft * u_lft * w_lft;
    DustFace f{0.0, 0.0, 0.0, 0.0};
    if (u_rgt > 0.0 && u_lft > 0.0) {
        f = {flx_rho_lft, flx_mom_u_lft, flx_mom_v_lft, flx_mom_w_lft};
    } else if (u_lft < 0.0 && u_rgt < 0.0) {
        f = {flx_rho_rgt, flx_mom_u_rgt, flx_mom_v_rgt, flx_mom_w_rgt};
    } else if (u_lft < 0.0 && u_rgt > 0.0) {
        f = {0.0, 0.0, 0.0, 0.0};
    } else if (u_lft > 0.0 && u_rgt < 0.0) {
        f = {flx_rho_lft + flx_rho_rgt, flx_mom_u_lft + flx_mom_u_rgt, flx_mom_v_lft + flx_mom_v_rgt,
             flx_mom_w_lft + flx_mom_w_rgt};
    }
    return f;
}

// solver_dust_llf (solvers.f90:840-1001), non-MHD, one species.
DustFace solver_dust_llf(double rho_lft, double u_lft, double v_lft, double w_lft,
                         double rho_rgt, double u_rgt, double v_rgt, double w_rgt) {
    double mom_u_rgt = rho_rgt * u_rgt, mom_u_lft = rho_lft * u_lft;
    double mom_v_rgt = rho_rgt * v_rgt, mom_v_lft = rho_lft * v_lft;
    double mom_w_rgt = rho_rgt * w_rgt, mom_w_lft = rho_lft * w_lft;
    double flx_rho_rgt = rho_rgt * u_rgt, flx_rho_lft = rho_lft * u_lft;
    double flx_mom_u_rgt = rho_rgt * sq(u_rgt), flx_mom_u_lft = rho_lft * sq(u_lft);
    double flx_mom_v_rgt = rho_rgt * u_rgt * v_rgt, flx_mom_v_lft = rho_lft * u_lft * v_lft;
    double flx_mom_w_rgt = rho_rgt * u_rgt * w_rgt, flx_mom_w_lft = rho_lft * u_lft * w_lft;
    double lam = fmax2(std::fabs(u_lft), std::fabs(u_rgt));
    DustFace f;
    f.rho = half * (flx_rho_lft + flx_rho_rgt) - half * lam * (rho_rgt - rho_lft);
    f.mn = half * (flx_mom_u_lft + flx_mom_u_rgt) - half * lam * (mom_u_rgt - mom_u_lft);
    f.mt = half * (flx_mom_v_lft + flx_mom_v_rgt) - half * lam * (mom_v_rgt - mom_v_lft);
    f.mz = half * (flx_mom_w_lft + flx_mom_w_rgt) - half * lam * (mom_w_rgt - mom_w_lft);
    return f;
}

// solver_dust_hll (solvers.f90:1010-1194), non-MHD, one species.
DustFace solver_dust_hll(double rho_lft, double u_lft, double v_lft, double w_lft,
                         double rho_rgt, double u_rgt, double v_rgt, double w_rgt) {
    double mom_u_rgt = rho_rgt * u_rgt, mom_u_lft = rho_lft * u_lft;
    double mom_v_rgt = rho_rgt * v_rgt, mom_v_lft = rho_lft * v_lft;
    double mom_w_rgt = rho_rgt * w_rgt, mom_w_lft = rho_lft * w_lft;
    double flx_rho_rgt = rho_rgt * u_rgt, flx_rho_lft = rho_lft * u_lft;
    double flx_mom_u_rgt = rho_rgt * sq(u_rgt), flx_mom_u_lft = rho_lft * sq(u_lft);
    double flx_mom_v_rgt = rho_rgt * u_rgt * v_rgt, flx_mom_v_lft = rho_lft * u_lft * v_lft;
    double flx_mom_w_rgt = rho_rgt * u_rgt * w_rgt, flx_mom_w_lft = rho_lft * u_lft * w_lft;
    double S_lft = fmin2(fmin2(u_lft, u_rgt), 0.0);
    double S_rgt = fmax2(fmax2(u_lft, u_rgt), 0.0);
    DustFace f{0.0, 0.0, 0.0, 0.0};
    if (S_rgt - S_lft != 0.0) {
        f.rho = (S_rgt * flx_rho_lft - S_lft * flx_rho_rgt + S_rgt * S_lft * (rho_rgt - rho_lft)) / (S_rgt - S_lft);
        f.mn = (S_rgt * flx_mom_u_lft - S_lft * flx_mom_u_rgt + S_rgt * S_lft * (mom_u_rgt - mom_u_lft)) / (S_rgt - S_lft);
        f.mt = (S_rgt * flx_mom_v_lft - S_lft * flx_mom_v_rgt + S_rgt * S_lft * (mom_v_rgt - mom_v_lft)) / (S_rgt - S_lft);
        f.mz = (S_rgt * flx_mom_w_lft - S_lft * flx_mom_w_rgt + S_rgt * S_lft * (mom_w_rgt - mom_w_lft)) / (S_rgt - S_lft);
    }
    return f;
}

// solver_hllc_dust (solvers.f90:704-836), one species: the gas HLLC of the reference with zero
// pressure, bounded by the gas sound speeds csl, csr of the face; the star "pressure" comes from
// the Lagrangian speeds.  The energies the reference forms are not used by the flux and are left
// out.
DustFace solver_dust_hllc(double rho_lft, double u_lft, double v_lft, double w_lft, double rho_rgt, double u_rgt,
                          double v_rgt, double w_rgt, double csl, double csr) {
    const double P_rgt = 0.0, P_lft = 0.0;
    double S_lft = fmin2(fmin2(u_lft, u_rgt) - fmax2(csl, csr), 0.0);
    double S_rgt = fmax2(fmax2(u_lft, u_rgt) + fmax2(csl, csr), 0.0);
    double hllc_l = rho_lft * (u_lft - S_lft);
    double hllc_r = rho_rgt * (S_rgt - u_rgt);
    double ustar = (hllc_r * u_rgt + hllc_l * u_lft + (P_lft - P_rgt)) / (hllc_r + hllc_l);
    double Pstar = (hllc_r * P_lft + hllc_l * P_rgt + hllc_l * hllc_r * (u_lft - u_rgt)) / (hllc_r + hllc_l);
    double rhostarleft = rho_lft * (S_lft - u_lft) / (S_lft - ustar);
    double rhostarright = rho_rgt * (S_rgt - u_rgt) / (S_rgt - ustar);
    double r_o, u_o, P_o;
    if (S_lft > 0.0) { r_o = rho_lft; u_o = u_lft; P_o = P_lft; }
    else if (ustar > 0.0) { r_o = rhostarleft; u_o = ustar; P_o = Pstar; }
    else if (S_rgt > 0.0) { r_o = rhostarright; u_o = ustar; P_o = Pstar; }
    else { r_o = rho_rgt; u_o = u_rgt; P_o = P_rgt; }
    DustFace f;
    f.rho = r_o * u_o;
    f.mn = r_o * u_o * u_o + P_o;
    if (ustar > 0.0) { f.mt = r_o * u_o * v_lft; f.mz = r_o * u_o * w_lft; }
    else { f.mt = r_o * u_o * v_rgt; f.mz = r_o * u_o * w_rgt; }
    return f;
}

// solve_wrapper (godunov.f90:768-833): gas solver then each dust species, flx in nvar order.
void solve_wrapper(const oracle_state& s, const double* ql, const double* qr, double* flx, double csl,
                   double csr, int idim) {
    const int ivn = s.index_vn[idim], ivt = s.index_vt[idim];
    GasFace g;
    const double gamma = s.cfg.gamma;
    if (s.cfg.solver == 0)
        g = solver_llf(gamma, ql[0], ql[ivn], ql[ivt], ql[3], ql[4], qr[0], qr[ivn], qr[ivt], qr[3], qr[4], csl, csr);
    else if (s.cfg.solver == 1)
        g = solver_hll(gamma, ql[0], ql[ivn], ql[ivt], ql[3], ql[4], qr[0], qr[ivn], qr[ivt], qr[3], qr[4], csl, csr);
    else
        g = solver_hllc(gamma, ql[0], ql[ivn], ql[ivt], ql[3], ql[4], qr[0], qr[ivn], qr[ivt], qr[3], qr[4], csl, csr);
    flx[0] = g.rho;
    flx[ivn] = g.mn;
    flx[ivt] = g.mt;
    flx[3] = g.mz;
    flx[4] = g.e;
    for (int k = 0; k < s.ndust; ++k) {
        const int ir = s.irhod[k], iu = s.index_vdn[k * 2 + idim], iv = s.index_vdt[k * 2 + idim], iw = s.ivdz[k];
        DustFace d;
        if (s.cfg.solverdust == 0) d = solver_dust_hb(ql[ir], ql[iu], ql[iv], ql[iw], qr[ir], qr[iu], qr[iv], qr[iw]);
        else if (s.cfg.solverdust == 1) d = solver_dust_llf(ql[ir], ql[iu], ql[iv], ql[iw], qr[ir], qr[iu], qr[iv], qr[iw]);
        else if (s.cfg.solverdust == 2) d = solver_dust_hll(ql[ir], ql[iu], ql[iv], ql[iw], qr[ir], qr[iu], qr[iv], qr[iw]);
        else d = solver_dust_hllc(ql[ir], ql[iu], ql[iv], ql[iw], qr[ir], qr[iu], qr[iv], qr[iw], csl, csr);
        flx[ir] = d.rho;
        flx[iu] = d.mn;
        flx[iv] = d.mt;
        flx[iw] = d.mz;
    }
}

// add_delta_u (godunov.f90:633-760)
void add_delta_u(oracle_state& s) {
    const int nvar = s.nvar;
    const double gamma = s.cfg.gamma, dt = s.dt;
    const bool iso = (s.cfg.iso_cs == 1), two_d = (s.ndim == 2);
    std::fill(s.flux.begin(), s.flux.end(), 0.0);
#pragma omp parallel
    {
        std::vector<double> ql(nvar), qr(nvar), flx(nvar);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < s.ncells; ++i) {
            if (!s.active_pred[i]) continue;
            const int ix = s.ixx(i), iy = s.iyy(i);
            for (int d = 0; d < (two_d ? 2 : 1); ++d) {
                int64_t il = (d == 0) ? s.icell(ix - 1, iy) : s.icell(ix, iy - 1);
                for (int v = 0; v < nvar; ++v) {
                    ql[v] = s.QM(il, v, d);
                    qr[v] = s.QP(i, v, d);
                    flx[v] = 0.0;
                }
                double csl, csr;
                if (iso) {
                    csl = s.cs[il];
                    csr = s.cs[i];
                } else {
                    csl = std::sqrt(gamma * ql[s.iP] / ql[s.irho]);
                    csr = std::sqrt(gamma * qr[s.iP] / qr[s.irho]);
                }
                solve_wrapper(s, ql.data(), qr.data(), flx.data(), csl, csr, d);
                for (int v = 0; v < nvar; ++v) s.FLX(i, v, d) = flx[v];
            }
        }
#pragma omp for schedule(static)
        for (int64_t i = 0; i < s.ncells; ++i) {
            if (!s.active[i]) continue;
            const int ix = s.ixx(i), iy = s.iyy(i);
            int64_t il = s.icell(ix + 1, iy);
            if (!two_d) {
                for (int v = 0; v < nvar; ++v)
                    s.U(i, v) = s.U(i, v) + (s.FLX(i, v, 0) * s.SURF(i, 0) - s.FLX(il, v, 0) * s.SURF(il, 0)) / s.vol[i] * dt;
            } else {
                int64_t ily = s.icell(ix, iy + 1);
                for (int v = 0; v < nvar; ++v)
                    s.U(i, v) = s.U(i, v) + (s.FLX(i, v, 0) * s.SURF(i, 0) - s.FLX(il, v, 0) * s.SURF(il, 0)) / s.vol[i] * dt +
                                (s.FLX(i, v, 1) * s.SURF(i, 1) - s.FLX(ily, v, 1) * s.SURF(ily, 1)) / s.vol[i] * dt;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Source_terms (src/solver/source_terms.f90:1-118,221), non-MHD, no gravity.
// ---------------------------------------------------------------------------------------------
void source_terms(oracle_state& s) {
    const double dt = s.dt;
    const bool polar = (s.cfg.geom == 2), br = s.flag(SHARK_FLAG_BACK_REACTION), visc = s.flag(SHARK_FLAG_VISCOSITY);
    if (!polar && !(br && s.cfg.iso_cs < 1 && s.ndust > 0) && !visc) return;   // S_U == 0
    std::vector<double> S((size_t)s.ncells * s.nvar, 0.0);
    auto SU = [&](int64_t i, int v) -> double& { return S[(size_t)v * s.ncells + i]; };
    for (int64_t i = 0; i < s.ncells; ++i) {
        if (!s.active[i]) continue;
        if (polar) {
            double rc = s.radii_c[i];
            SU(i, s.ivx) = SU(i, s.ivx) + dt * (s.Q(i, s.irho) * sq(s.Q(i, s.ivy)) + s.Q(i, s.iP)) / rc;
            SU(i, s.ivy) = SU(i, s.ivy) - dt * (s.Q(i, s.irho) * s.Q(i, s.ivy) * s.Q(i, s.ivx) / rc);
            for (int k = 0; k < s.ndust; ++k) {
                SU(i, s.ivdx[k]) = SU(i, s.ivdx[k]) + dt * (s.Q(i, s.irhod[k]) * sq(s.Q(i, s.ivdy[k])) / rc);
                SU(i, s.ivdy[k]) = SU(i, s.ivdy[k]) - dt * (s.Q(i, s.irhod[k]) * s.Q(i, s.ivdy[k]) * s.Q(i, s.ivdx[k]) / rc);
            }
        }
        if (s.ndust > 0 && br && s.cfg.iso_cs < 1) {
            for (int k = 0; k < s.ndust; ++k) {
                double ts = s.TSTOP(i, k);
                SU(i, s.iP) = SU(i, s.iP) + dt * (s.Q(i, s.ivx) * (s.Q(i, s.ivx) - s.Q(i, s.ivdx[k]))) / ts +
                              dt * (s.Q(i, s.ivy) * (s.Q(i, s.ivy) - s.Q(i, s.ivdy[k]))) / ts +
                              dt * (s.Q(i, s.ivz) * (s.Q(i, s.ivz) - s.Q(i, s.ivdz[k]))) / ts;
            }
        }
        if (visc && s.ndim == 2) {   // viscosity (source_terms.f90:99-118)
            const int ix = (int)(i % s.nx_max), iy = (int)(i / s.nx_max);
            const int64_t il = s.icell(ix - 1, iy), ir = s.icell(ix + 1, iy);
            const double eta = s.eta_visc[i], rho = s.Q(i, s.irho), dx = s.DX(i, 0);
            if (!polar) {
                const int64_t jd = s.icell(ix, iy - 1), ju = s.icell(ix, iy + 1);
                const double dy = s.DX(i, 1);
                const double lap_x_u = (s.Q(ir, s.ivx) + s.Q(il, s.ivx) - 2.0 * s.Q(i, s.ivx)) / (dx * dx);
                SU(i, s.ivx) = SU(i, s.ivx) + rho * dt * eta * lap_x_u;
                const double lap_y_u = (s.Q(ju, s.ivx) + s.Q(jd, s.ivx) - 2.0 * s.Q(i, s.ivx)) / (dy * dy);
                SU(i, s.ivx) = SU(i, s.ivx) + rho * dt * eta * lap_y_u;
                const double lap_x_v = (s.Q(ir, s.ivy) + s.Q(il, s.ivy) - 2.0 * s.Q(i, s.ivy)) / (dx * dx);
                const double lap_y_v = (s.Q(ju, s.ivy) + s.Q(jd, s.ivy) - 2.0 * s.Q(i, s.ivy)) / (dy * dy);
                SU(i, s.ivy) = SU(i, s.ivy) + rho * dt * eta * (lap_x_v + lap_y_v);
            } else {
                const double rc = s.radii_c[i];
                const double lap_x_u = (s.Q(ir, s.ivx) + s.Q(il, s.ivx) - 2.0 * s.Q(i, s.ivx)) / (dx * dx) +
                                       (s.Q(ir, s.ivx) + s.Q(il, s.ivx)) / rc / dx / 2.0 - s.Q(i, s.ivx) / rc / rc;
                SU(i, s.ivx) = SU(i, s.ivx) + rho * dt * eta * lap_x_u;
                const double lap_x_v = (s.Q(ir, s.ivy) + s.Q(il, s.ivy) - 2.0 * s.Q(i, s.ivy)) / (dx * dx) -
                                       s.Q(i, s.ivy) / (rc * rc) + (s.Q(ir, s.ivy) + s.Q(il, s.ivy)) / rc / dx / 2.0;
                SU(i, s.ivy) = SU(i, s.ivy) + rho * dt * eta * lap_x_v;
            }
        }
    }
    for (size_t j = 0; j < S.size(); ++j) s.u[j] = s.u[j] + S[j];
}

// ---------------------------------------------------------------------------------------------
// fargo_scheme (src/solver/fargo_scheme.f90:2-81), with the reference's defects fixed:
//   * `one` (undeclared, uninitialised) is 1 and `eps` is FP64 (it is an implicit REAL*4 there);
//   * limited slopes of the conserved variables along phi are computed for every active cell
//     (the reference loops ix=1..nx, iy=1..ny, missing the last active columns and rows), with
//     the periodic wrap of the ring (what its apply_boundaries provides);
//   * the source rows wrap modulo ny (the reference wraps once, i.e. assumes nshft < ny).
// Per ring (fixed radius) the shift vk*dt splits into whole cells nshft and a residual eps; the
// new value is the linear remap of the two donor cells plus their slope correction.
// ---------------------------------------------------------------------------------------------
void fargo_scheme(oracle_state& s) {
    const int ny = s.ny, fy = s.first_active_y, st = s.cfg.slope_type;
    const double forth = 0.25, one = 1.0;
    const std::vector<double> uold = s.u;
    auto UO = [&](int ix, int ay, int v) { return uold[(size_t)v * s.ncells + s.icell(ix, fy + ay)]; };
#pragma omp parallel for schedule(static)
    for (int ix = s.first_active; ix <= s.last_active; ++ix) {
        const int64_t c0 = s.icell(ix, fy);
        const double vk = s.fargo_v[c0];
        const double dy_loc = s.DX(c0, 1) * s.radii_c[c0];
        const double shift = std::fabs(vk * s.dt);
        const int nshft = (int)(shift / dy_loc);
        const double eps = std::fmod(shift, dy_loc) / dy_loc;
        std::vector<double> du(ny);
        for (int v = 0; v < s.nvar; ++v) {
            for (int a = 0; a < ny; ++a) {
                const double um = UO(ix, (a - 1 + ny) % ny, v), u0 = UO(ix, a, v), up = UO(ix, (a + 1) % ny, v);
                du[a] = st > 0 ? slope_limit(st, u0 - um, up - u0) : 0.0;
            }
            for (int a = 0; a < ny; ++a) {
                int j, jp;
                double w0, w1;
                if (vk > 0.0) {
                    j = ((a - nshft - 1) % ny + ny) % ny;
                    w0 = eps; w1 = one - eps;
                } else {
                    j = (a + nshft) % ny;
                    w0 = one - eps; w1 = eps;
                }
                jp = (j + 1) % ny;
                double un = UO(ix, j, v) * w0 + UO(ix, jp, v) * w1;
                un = un + half * du[j] * (forth - sq(half - eps)) + half * du[jp] * (sq(half - eps) - forth);
                s.U(s.icell(ix, fy + a), v) = un;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// dust_drag (src/dust/dust_drag.f90:2-75): Krapp et al. implicit multi-species drag + floor.
// ---------------------------------------------------------------------------------------------
void dust_drag(oracle_state& s, double coeffdt) {
    const int N = s.ndust;
    const double dt = s.dt, dmin = s.cfg.dust_ratio_min;
    const bool br = s.flag(SHARK_FLAG_BACK_REACTION);
#pragma omp parallel
    {
        std::vector<double> alphak(N);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < s.ncells; ++i) {
            if (!s.active[i]) continue;
            double rhon = s.U(i, s.irho), pnx = s.U(i, s.ivx), pny = s.U(i, s.ivy), pnz = s.U(i, s.ivz);
            for (int k = 0; k < N; ++k) {
                alphak[k] = coeffdt * dt / s.TSTOP(i, k);
                pnx = pnx + alphak[k] / (1.0 + alphak[k]) * s.U(i, s.ivdx[k]);
                pny = pny + alphak[k] / (1.0 + alphak[k]) * s.U(i, s.ivdy[k]);
                pnz = pnz + alphak[k] / (1.0 + alphak[k]) * s.U(i, s.ivdz[k]);
                rhon = rhon + alphak[k] / (1.0 + alphak[k]) * s.U(i, s.irhod[k]);
            }
            for (int k = 0; k < N; ++k) {
                double a = alphak[k];
                s.U(i, s.ivdx[k]) = s.U(i, s.ivdx[k]) / (1.0 + a) + (a / (1.0 + a)) * pnx / rhon * s.U(i, s.irhod[k]);
                s.U(i, s.ivdy[k]) = s.U(i, s.ivdy[k]) / (1.0 + a) + (a / (1.0 + a)) * pny / rhon * s.U(i, s.irhod[k]);
                s.U(i, s.ivdz[k]) = s.U(i, s.ivdz[k]) / (1.0 + a) + (a / (1.0 + a)) * pnz / rhon * s.U(i, s.irhod[k]);
            }
            if (br) {
                s.U(i, s.ivx) = pnx / rhon * s.U(i, s.irho);
                s.U(i, s.ivy) = pny / rhon * s.U(i, s.irho);
                s.U(i, s.ivz) = pnz / rhon * s.U(i, s.irho);
            }
        }
#pragma omp for schedule(static)
        for (int64_t i = 0; i < s.ncells; ++i) {
            if (!s.active[i]) continue;
            for (int k = 0; k < N; ++k)
                s.U(i, s.irhod[k]) = fmax2(s.U(i, s.irho) * dmin, s.U(i, s.irhod[k]));
        }
    }
}

// ---------------------------------------------------------------------------------------------
// solve (src/solver/solve.f90:10-181) for the in-scope configurations.
// ---------------------------------------------------------------------------------------------
void solve(oracle_state& s) {
    const bool fk = s.flag(SHARK_FLAG_FORCE_KICK);
    apply_boundaries(s);
    ctoprim(s);
    if (fk) update_force_setup(s);
    if (s.ndust > 0) {
        // distribution_dust(.false.): epsilondust = rho_d/rho over all cells (dust_init.f90:76-82)
        for (int k = 0; k < s.ndust; ++k)
            for (int64_t i = 0; i < s.ncells; ++i) s.EPSD(i, k) = s.Q(i, s.irhod[k]) / s.Q(i, s.irho);
        compute_tstop(s);
        if (s.flag(SHARK_FLAG_CHARGING)) charge(s);
    }
    courant(s);
    if (fk) kick(s, 1.0);
    predictor(s);
    add_delta_u(s);
    source_terms(s);
    if (s.flag(SHARK_FLAG_FARGO)) fargo_scheme(s);
    if (s.ndust > 0 && s.flag(SHARK_FLAG_DRAG)) dust_drag(s, 1.0);
    if (s.ndust > 0 && s.flag(SHARK_FLAG_GROWTH)) dust_growth(s);
    if (s.cfg.setup == SHARK_SETUP_DUSTYTURB && s.cfg.turb_mach > 0.0) turb_kick(s);
    setup_inloop(s);
}

// Counter-based uniform deviate in [0,1): splitmix64 of (seed, counter).
inline double hash_uniform(uint64_t seed, uint64_t counter) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + counter + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------------------------------------
// Initial conditions
// ---------------------------------------------------------------------------------------------
// SOD setup (src/setups/SOD/setup.f90:1-46)
void setup_sod(oracle_state& s) {
    std::fill(s.q.begin(), s.q.end(), 0.0);
    for (int iy = 0; iy < s.ny_max; ++iy)
        for (int ix = 0; ix < s.nx_max; ++ix) {
            int64_t c = s.icell(ix, iy);
            s.Q(c, s.irho) = s.cfg.sod_rho_l;
            s.Q(c, s.ivx) = 0.0;
            s.Q(c, s.iP) = s.cfg.sod_P_l;
            double pos = (s.cfg.sod_direction == 0) ? s.POS(c, 0) : s.POS(c, (s.ndim == 2) ? 1 : 0);
            if (pos > half) {
                s.Q(c, s.irho) = s.cfg.sod_rho_r;
                s.Q(c, s.ivx) = 0.0;
                s.Q(c, s.iP) = s.cfg.sod_P_r;
            }
        }
    apply_boundaries(s);
    primtoc(s);
    if (s.cfg.iso_cs < 1) {  // cs is set by ctoprim for adiabatic runs
        ctoprim(s);
    }
}

// DUSTYWAVE setup (src/setups/DUSTYWAVE/setup.f90:12-79); dust2gas_ratio(idust) = dust_eps[k].
void setup_dustywave(oracle_state& s) {
    const double delta_rho = s.cfg.dw_delta_rho, vx_0 = s.cfg.dw_vx_0, kx = s.cfg.dw_kx_wave;
    const double rho_0 = s.cfg.dw_rho_0, L = s.box_l;
    std::fill(s.q.begin(), s.q.end(), 0.0);
    for (int64_t i = 0; i < s.ncells; ++i) {
        double ph = std::sin(2.0 * pi * s.POS(i, 0) / L * kx);
        s.Q(i, s.irho) = rho_0 * (1 + delta_rho * ph);
        s.Q(i, s.ivx) = vx_0 * ph;
        s.cs[i] = s.cfg.cs0;
        s.Q(i, s.iP) = sq(s.cs[i]) * s.Q(i, s.irho);
        for (int k = 0; k < s.ndust; ++k) {
            s.EPSD(i, k) = s.cfg.dust_eps[k];
            s.Q(i, s.irhod[k]) = s.EPSD(i, k) * s.Q(i, s.irho);
            s.Q(i, s.ivdx[k]) = vx_0 * ph;
        }
    }
    apply_boundaries(s);
    primtoc(s);
}

// KH setup (src/setups/KH/setup.f90:1-51, KH/eos.f90 cs_eos, KH/units.f90): a band |y - L_y/2| <
// L_y/4 of density rho_diffuse moving at -Mach cs/2 inside gas of density rho_dense moving at
// +Mach cs/2, vy seeded with vy0 Mach cs cos(2 kx pi x'/L) over the whole box, one pressure
// rho_dense cs^2, cs = cs_eos(T_dense); cgs inputs divided by unit_d, unit_v, unit_P = unit_d
// unit_v^2.  Dust: epsilondust = dust_eps[k] (distribution_dust, or 0.01 for one species), at rest.
void setup_kh(oracle_state& s) {
    const shark_gpu_config& c = s.cfg;
    const double ul = unit_or_1(c.unit_l), ud = unit_or_1(c.unit_d), ut = unit_or_1(c.unit_t);
    const double uv = ul / ut, uP = ud * (uv * uv);
    constexpr double mH = 1.67e-24, kB = 1.38e-16;                      // phys_const.f90:8-9
    const double cs = std::sqrt(c.gamma * kB * c.kh_T_dense / (c.mu_gas * mH));   // KH/eos.f90
    std::fill(s.q.begin(), s.q.end(), 0.0);
    for (int iy = 0; iy < s.ny_max; ++iy)
        for (int ix = 0; ix < s.nx_max; ++ix) {
            const int64_t i = s.icell(ix, iy);
            const double xx = s.POS(i, 0) - half * s.box_l;
            const double yy = s.POS(i, 1) - half * s.box_l_y;
            s.Q(i, s.irho) = c.kh_rho_dense / ud;
            s.Q(i, s.ivx) = cs * c.kh_mach / uv * half;
            s.Q(i, s.ivy) = (c.kh_vy0 * cs * c.kh_mach * std::cos(xx * 2.0 * c.kh_kx * pi / s.box_l)) / uv;
            s.Q(i, s.iP) = c.kh_rho_dense * (cs * cs) / uP;
            if (std::fabs(yy / s.box_l_y) < 0.25) {
                s.Q(i, s.irho) = c.kh_rho_diffuse / ud;
                s.Q(i, s.ivx) = -(cs * c.kh_mach / uv / 2.0);
                s.Q(i, s.iP) = c.kh_rho_dense * (cs * cs) / uP;
            }
        }
    for (int64_t i = 0; i < s.ncells; ++i)
        for (int k = 0; k < s.ndust; ++k) {
            s.EPSD(i, k) = c.dust_eps[k];
            s.Q(i, s.irhod[k]) = s.EPSD(i, k) * s.Q(i, s.irho);
        }
    apply_boundaries(s);
    primtoc(s);
    ctoprim(s);
}

// sedov setup (src/setups/sedov/setup.f90:1-34): gas at rest, density rho_ext, pressure P_ext,
// plus P_cen inside the disc |x - L/2|^2 + |y - L/2|^2 < r_expl^2 of the active cells; the ghost
// cells stay zero until the boundaries fill them.
void setup_sedov(oracle_state& s) {
    const shark_gpu_config& c = s.cfg;
    std::fill(s.q.begin(), s.q.end(), 0.0);
    for (int iy = 0; iy < s.ny_max; ++iy)
        for (int ix = 0; ix < s.nx_max; ++ix) {
            const int64_t i = s.icell(ix, iy);
            if (!s.active[i]) continue;
            s.Q(i, s.irho) = c.sedov_rho_ext;
            s.Q(i, s.iP) = c.sedov_P_ext;
            const double xn = std::fabs(s.POS(i, 0) - half * s.box_l);
            const double yn = std::fabs(s.POS(i, 1) - half * s.box_l_y);
            if (xn * xn + yn * yn < c.sedov_r_expl * c.sedov_r_expl) s.Q(i, s.iP) = c.sedov_P_ext + c.sedov_P_cen;
        }
    apply_boundaries(s);
    primtoc(s);
}

// SI setup (src/setups/SI/setup.f90:1-117): dust2gas_species = dust_eps[k], Stokes_species =
// dust_stokes[k] (the host computes both, e.g. from the MRN bins of distribution_dust).  Noise:
// uniform in [-noise_amp, noise_amp] on the three dust velocity components from a counter-based
// hash of (seed, component, cell) instead of the reference's ranf stream on all velocities.
void setup_si(oracle_state& s, double noise_amp, uint64_t seed) {
    const int N = s.ndust;
    const double qs = s.cfg.si_q_shear, om = s.cfg.si_omega, eta = s.cfg.si_eta_stream, r0 = s.cfg.si_rad0;
    const double rho_init = s.cfg.si_rho_init;
    const double vkep = r0 * om, cs0 = s.cfg.cs0;
    double A_nak = 0.0, B_nak = 1.0;
    for (int k = 0; k < N; ++k) {
        double e = s.cfg.dust_eps[k], St = s.cfg.dust_stokes[k];
        A_nak = A_nak + e * St / (1.0 + sq(St));
        B_nak = B_nak + e / (1.0 + sq(St));
    }
    double vx_nak = 2.0 * eta * vkep * A_nak / (A_nak + B_nak);
    double vy_nak = -eta * vkep * B_nak / (A_nak + B_nak);
    std::vector<double> ux(N), uy(N);
    for (int k = 0; k < N; ++k) {
        double St = s.cfg.dust_stokes[k];
        ux[k] = (vx_nak + 2.0 * St * vy_nak) / (1.0 + sq(St));
        uy[k] = (vy_nak - half * St * vx_nak) / (1.0 + sq(St));
    }
    std::fill(s.q.begin(), s.q.end(), 0.0);
    for (int64_t i = 0; i < s.ncells; ++i) {
        double xx = s.POS(i, 0) - half * s.box_l;
        s.Q(i, s.irho) = rho_init;
        s.Q(i, s.ivx) = vx_nak;
        s.Q(i, s.ivy) = 0.0;
        s.Q(i, s.ivz) = qs * om * xx + vy_nak;
        s.Q(i, s.iP) = s.Q(i, s.irho) * sq(cs0);
        for (int k = 0; k < N; ++k) {
            s.Q(i, s.irhod[k]) = s.cfg.dust_eps[k] * rho_init;
            s.EPSD(i, k) = s.cfg.dust_eps[k];
            double nx_ = 0, ny_ = 0, nz_ = 0;
            if (noise_amp > 0) {
                uint64_t base = ((uint64_t)k * 3) * (uint64_t)s.ncells + (uint64_t)i;
                nx_ = (2.0 * hash_uniform(seed, base) - 1.0) * noise_amp;
                ny_ = (2.0 * hash_uniform(seed, base + (uint64_t)s.ncells) - 1.0) * noise_amp;
                nz_ = (2.0 * hash_uniform(seed, base + 2 * (uint64_t)s.ncells) - 1.0) * noise_amp;
            }
            s.Q(i, s.ivdx[k]) = nx_ + ux[k];
            s.Q(i, s.ivdy[k]) = ny_;
            s.Q(i, s.ivdz[k]) = nz_ + qs * om * xx + uy[k];
        }
        s.cs[i] = cs0;
    }
    primtoc(s);
    apply_boundaries(s);
}

// Polar disk initial state (disk_polar/setup.f90:12-84), re-specified for the GB300 workload:
// T ~ r^disk_temp_slope through h(r), the matching pressure-supported rotation
// v_phi = Omega r sqrt(1 - h^2 (1 - slope + r/R_out)) (the reference's sqrt(1 - h^2 (2 + r/R_out))
// for slope -1), one grain size per bin (dust_size; the reference gives every bin scut), dust
// starting at the full Keplerian azimuthal velocity with the reference's radial drift, and an
// optional uniform density perturbation of relative amplitude noise_amp (counter-based hash).
void setup_disk(oracle_state& s, double noise_amp, uint64_t seed) {
    const shark_gpu_config& c = s.cfg;
    const bool fargo = s.flag(SHARK_FLAG_FARGO);
    std::fill(s.q.begin(), s.q.end(), 0.0);
    for (int iy = 0; iy < s.ny_max; ++iy)
        for (int ix = 0; ix < s.nx_max; ++ix) {
            const int64_t i = s.icell(ix, iy);
            const double rr = s.radii_c[i];
            const double h = disk_h(c, rr), H = h * rr;
            const double Omega = std::sqrt(c.disk_mstar / powi(rr, 3));
            const double cs0 = Omega * H;
            s.fargo_v[i] = fargo ? -Omega * rr : 0.0;
            double sig = c.disk_sigma0 * (c.disk_r0 / rr) * std::exp(-rr / c.disk_rout);
            if (noise_amp > 0) sig = sig * (1.0 + noise_amp * (2.0 * hash_uniform(seed, (uint64_t)i) - 1.0));
            const double rot = std::sqrt(1.0 - sq(h) * (1.0 - c.disk_temp_slope + rr / c.disk_rout));
            s.Q(i, s.irho) = sig;
            s.Q(i, s.ivx) = 0.0;
            s.Q(i, s.ivy) = Omega * rr * rot;
            s.Q(i, s.iP) = sig * sq(cs0);
            s.cs[i] = cs0;
            for (int k = 0; k < s.ndust; ++k) {
                s.Q(i, s.irhod[k]) = c.dust_eps[k] * sig;
                const double ts = std::sqrt(pi * c.gamma / 8.0) * (c.rhograin) * c.dust_size[k] /
                                  (sig / (std::sqrt(2.0 * pi) * H) * cs0);
                const double St = ts * Omega;
                s.Q(i, s.ivdx[k]) = (rot - 1.0) * Omega * rr / (St + 1.0 / St);
                s.Q(i, s.ivdy[k]) = Omega * rr;
            }
        }
    primtoc(s);
    s.u_init = s.u;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------------------------
extern "C" {

oracle_state* oracle_create(const shark_gpu_config* cfg) {
    if (!cfg || cfg->abi_version != SHARK_GPU_ABI_VERSION) return nullptr;
    if (cfg->nghost != 2 || cfg->nx < 4 || cfg->ny < 1 || cfg->ndust < 0 || cfg->ndust > SHARK_MAX_DUST) return nullptr;
    if (cfg->slope_type < 0 || cfg->slope_type > 3) return nullptr;
    if (cfg->geom != 0 && cfg->geom != 2) return nullptr;
    if (cfg->geom == 2 && cfg->ny == 1) return nullptr;
    oracle_state* s = new oracle_state();
    s->cfg = *cfg;
    s->nx = cfg->nx; s->ny = cfg->ny; s->nghost = cfg->nghost; s->ndust = cfg->ndust;
    s->nvar = 5 + 4 * s->ndust;
    s->ndim = (s->ny == 1) ? 1 : 2;
    s->nx_max = s->nx + 2 * s->nghost;
    s->ny_max = (s->ny == 1) ? 1 : s->ny + 2 * s->nghost;
    s->ncells = (int64_t)s->nx_max * s->ny_max;
    s->first_active = s->nghost;
    s->last_active = s->nx + s->nghost - 1;
    s->first_active_y = (s->ny == 1) ? 0 : s->nghost;
    s->last_active_y = (s->ny == 1) ? 0 : s->ny + s->nghost - 1;
    const int N = s->ndust;
    s->irhod.resize(N); s->ivdx.resize(N); s->ivdy.resize(N); s->ivdz.resize(N);
    s->index_vdn.resize(2 * N); s->index_vdt.resize(2 * N);
    for (int k = 0; k < N; ++k) {
        s->irhod[k] = 5 + k; s->ivdx[k] = 5 + N + k; s->ivdy[k] = 5 + 2 * N + k; s->ivdz[k] = 5 + 3 * N + k;
        s->index_vdn[k * 2 + 0] = s->ivdx[k]; s->index_vdt[k * 2 + 0] = s->ivdy[k];
        s->index_vdn[k * 2 + 1] = s->ivdy[k]; s->index_vdt[k * 2 + 1] = s->ivdx[k];
    }
    s->index_vn[0] = s->ivx; s->index_vt[0] = s->ivy;
    s->index_vn[1] = s->ivy; s->index_vt[1] = s->ivx;
    const size_t nc = (size_t)s->ncells;
    s->u.assign(nc * s->nvar, 0.0);
    s->q.assign(nc * s->nvar, 0.0);
    s->qm.assign(nc * s->nvar * s->ndim, 0.0);
    s->qp.assign(nc * s->nvar * s->ndim, 0.0);
    s->flux.assign(nc * s->nvar * s->ndim, 0.0);
    s->cs.assign(nc, 0.0);
    s->dx.assign(nc * s->ndim, 0.0);
    s->surf.assign(nc * s->ndim, 0.0);
    s->vol.assign(nc, 0.0);
    s->position.assign(nc * s->ndim, 0.0);
    s->radii_c.assign(nc, 1.0);
    s->force.assign(nc * 3, 0.0);
    s->force_dust.assign(nc * 3 * (size_t)N, 0.0);
    s->tstop.assign(nc * (size_t)N, 0.0);
    s->sdust.assign(nc * (size_t)N, 0.0);
    s->epsilondust.assign(nc * (size_t)N, 0.0);
    for (int k = 0; k < N; ++k)
        for (size_t i = 0; i < nc; ++i) s->sdust[(size_t)k * nc + i] = cfg->dust_size[k];
    s->box_l = cfg->box_l;
    s->box_l_y = cfg->box_l_y;
    get_active_cells(*s);
    gridinit(*s);
    // isothermal sound speed: uniform cs0 (the disk: its radial profile) unless the caller
    // overrides it with oracle_set_cs
    s->fargo_v.assign(nc, 0.0);
    if (cfg->iso_cs == 1)
        for (size_t i = 0; i < nc; ++i) s->cs[i] = cfg->cs0;
    if (cfg->setup == SHARK_SETUP_DUSTYTURB && cfg->turb_mach > 0.0) turb_init(*s);
    s->eta_visc.assign(nc, 0.0);
    if (cfg->setup == SHARK_SETUP_DISK_CART) {   // disk/setup.f90: cs0 = HoverR sqrt(Mstar/rr), eta = alpha H cs
        for (size_t i = 0; i < nc; ++i) {
            const double rr = cdisk_cell(*s, (int64_t)i).rr;
            s->cs[i] = cfg->disk_hoverr * std::sqrt(cfg->disk_mstar / rr);
            s->eta_visc[i] = cfg->disk_alpha_visc * (cfg->disk_hoverr * rr) * s->cs[i];
        }
    }
    if (cfg->setup == SHARK_SETUP_DISK_POLAR) {
        for (size_t i = 0; i < nc; ++i) {
            const double rr = s->radii_c[i];
            s->cs[i] = disk_cs(*cfg, rr);
            s->eta_visc[i] = cfg->disk_alpha_visc * (disk_h(*cfg, rr) * rr) * s->cs[i];   // setup.f90:67
            if (cfg->flags & SHARK_FLAG_FARGO) s->fargo_v[i] = -std::sqrt(cfg->disk_mstar / powi(rr, 3)) * rr;
        }
    }
    return s;
}

void oracle_destroy(oracle_state* s) { delete s; }
int64_t oracle_ncells(const oracle_state* s) { return s ? s->ncells : -1; }
int32_t oracle_nvar(const oracle_state* s) { return s ? s->nvar : -1; }

int32_t oracle_setup_ic(oracle_state* s, double noise_amp, uint64_t seed) {
    if (!s) return SHARK_ERR_INVALID_ARG;
    switch (s->cfg.setup) {
        case SHARK_SETUP_SOD: setup_sod(*s); break;
        case SHARK_SETUP_DUSTYWAVE: setup_dustywave(*s); break;
        case SHARK_SETUP_SI: setup_si(*s, noise_amp, seed); break;
        case SHARK_SETUP_DISK_POLAR: setup_disk(*s, noise_amp, seed); break;
        case SHARK_SETUP_KH: setup_kh(*s); break;
        case SHARK_SETUP_SEDOV: setup_sedov(*s); break;
        default: return SHARK_ERR_UNSUPPORTED;
    }
    s->time = 0.0;
    return SHARK_OK;
}

int32_t oracle_get_u(const oracle_state* s, double* u) {
    if (!s || !u) return SHARK_ERR_INVALID_ARG;
    std::memcpy(u, s->u.data(), s->u.size() * sizeof(double));
    return SHARK_OK;
}
int32_t oracle_set_u(oracle_state* s, const double* u) {
    if (!s || !u) return SHARK_ERR_INVALID_ARG;
    std::memcpy(s->u.data(), u, s->u.size() * sizeof(double));
    if (s->u_init.empty()) s->u_init = s->u;   // first state given = relaxation reference (disk)
    return SHARK_OK;
}
int32_t oracle_get_q(oracle_state* s, double* q, double* cs) {
    if (!s) return SHARK_ERR_INVALID_ARG;
    ctoprim(*s);
    if (q) std::memcpy(q, s->q.data(), s->q.size() * sizeof(double));
    if (cs) std::memcpy(cs, s->cs.data(), s->cs.size() * sizeof(double));
    return SHARK_OK;
}
int32_t oracle_get_cs(const oracle_state* s, double* cs) {
    if (!s || !cs) return SHARK_ERR_INVALID_ARG;
    std::memcpy(cs, s->cs.data(), s->cs.size() * sizeof(double));
    return SHARK_OK;
}
int32_t oracle_set_cs(oracle_state* s, const double* cs) {
    if (!s || !cs) return SHARK_ERR_INVALID_ARG;
    std::memcpy(s->cs.data(), cs, s->cs.size() * sizeof(double));
    return SHARK_OK;
}
int32_t oracle_get_grid(const oracle_state* s, double* dx, double* surf, double* vol, double* position,
                        double* radii_c) {
    if (!s) return SHARK_ERR_INVALID_ARG;
    if (dx) std::memcpy(dx, s->dx.data(), s->dx.size() * sizeof(double));
    if (surf) std::memcpy(surf, s->surf.data(), s->surf.size() * sizeof(double));
    if (vol) std::memcpy(vol, s->vol.data(), s->vol.size() * sizeof(double));
    if (position) std::memcpy(position, s->position.data(), s->position.size() * sizeof(double));
    if (radii_c) std::memcpy(radii_c, s->radii_c.data(), s->radii_c.size() * sizeof(double));
    return SHARK_OK;
}

int32_t oracle_solve(oracle_state* s, double* dt_out) {
    if (!s) return SHARK_ERR_INVALID_ARG;
    if (!(s->cfg.flags & SHARK_FLAG_STATIC)) solve(*s);
    if (dt_out) *dt_out = s->dt;
    return SHARK_OK;
}

int32_t oracle_run(oracle_state* s, int64_t nsteps, double tend, double* time_io, int64_t* steps_done) {
    if (!s || !time_io) return SHARK_ERR_INVALID_ARG;
    double time = *time_io;
    int64_t n = 0;
    while (n < nsteps && !(time >= tend)) {
        solve(*s);
        time = time + s->dt;
        ++n;
    }
    *time_io = time;
    s->time = time;
    if (steps_done) *steps_done = n;
    return SHARK_OK;
}

int32_t oracle_totals(const oracle_state* s, double* out) {
    if (!s || !out) return SHARK_ERR_INVALID_ARG;
    oracle_state& S = const_cast<oracle_state&>(*s);
    for (int sp = 0; sp <= s->ndust; ++sp) {
        int vr = sp == 0 ? S.irho : S.irhod[sp - 1];
        int vx = sp == 0 ? S.ivx : S.ivdx[sp - 1];
        int vy = sp == 0 ? S.ivy : S.ivdy[sp - 1];
        int vz = sp == 0 ? S.ivz : S.ivdz[sp - 1];
        int vars[4] = {vr, vx, vy, vz};
        for (int c = 0; c < 4; ++c) {
            double sum = 0.0, comp = 0.0;
            for (int64_t i = 0; i < s->ncells; ++i) {
                if (!s->active[i]) continue;
                double y = S.U(i, vars[c]) - comp;
                double t = sum + y;
                comp = (t - sum) - y;
                sum = t;
            }
            out[4 * sp + c] = sum;
        }
    }
    return SHARK_OK;
}

int32_t oracle_apply_boundaries(oracle_state* s) { if (!s) return SHARK_ERR_INVALID_ARG; apply_boundaries(*s); return SHARK_OK; }
int32_t oracle_charge(oracle_state* s, const double* seed, int32_t* iters) {
    if (!s || s->ndust == 0) return SHARK_ERR_INVALID_ARG;
    if (seed) s->chg_seed.assign(seed, seed + s->ncells);
    ctoprim(*s);
    charge(*s);
    s->chg_seed.clear();
    if (iters) std::memcpy(iters, s->chg_iters.data(), s->chg_iters.size() * sizeof(int32_t));
    return SHARK_OK;
}
int32_t oracle_get_charge(const oracle_state* s, double* zd, double* ni, double* ne, double* psi,
                          double* eta /* 3 x ncells: o, h, a */, double* gamma_d) {
    if (!s || s->psi_old.empty()) return SHARK_ERR_STATE;
    const size_t nc = (size_t)s->ncells, nd = nc * s->ndust;
    if (zd) std::memcpy(zd, s->zd.data(), nd * sizeof(double));
    if (ni) std::memcpy(ni, s->ni.data(), nc * sizeof(double));
    if (ne) std::memcpy(ne, s->ne.data(), nc * sizeof(double));
    if (psi) std::memcpy(psi, s->psi_old.data(), nc * sizeof(double));
    if (eta) {
        std::memcpy(eta, s->eta_o.data(), nc * sizeof(double));
        std::memcpy(eta + nc, s->eta_h.data(), nc * sizeof(double));
        std::memcpy(eta + 2 * nc, s->eta_a.data(), nc * sizeof(double));
    }
    if (gamma_d) std::memcpy(gamma_d, s->gamma_d.data(), nd * sizeof(double));
    return SHARK_OK;
}
int32_t oracle_reset_charge(oracle_state* s) {
    if (!s) return SHARK_ERR_INVALID_ARG;
    std::fill(s->psi_old.begin(), s->psi_old.end(), 0.0);
    return SHARK_OK;
}
int32_t oracle_charge_psi0(const oracle_state* s, double* psi0) {
    if (!s || !psi0) return SHARK_ERR_INVALID_ARG;
    *psi0 = charge_psi0(s->cfg.chg_stick_el * std::sqrt(s->cfg.chg_mu_ions * phys::mH / phys::m_el));
    return SHARK_OK;
}
int32_t oracle_growth(oracle_state* s, int32_t* substeps) {
    if (!s || s->ndust == 0) return SHARK_ERR_INVALID_ARG;
    ctoprim(*s);
    compute_tstop(*s);
    dust_growth(*s);
    if (substeps) std::memcpy(substeps, g_growth_iters.data(), g_growth_iters.size() * sizeof(int32_t));
    return SHARK_OK;
}
int32_t oracle_growth_grid(const oracle_state* s, double* zeta_eta_massmin, double* mk, double* redis) {
    if (!s) return SHARK_ERR_INVALID_ARG;
    const GrowthGrid G = growth_grid(s->cfg);
    if (zeta_eta_massmin) { zeta_eta_massmin[0] = G.zeta; zeta_eta_massmin[1] = G.eta; zeta_eta_massmin[2] = G.massmin; }
    if (mk) std::memcpy(mk, G.mk.data(), G.mk.size() * sizeof(double));
    if (redis) std::memcpy(redis, G.redis.data(), G.redis.size() * sizeof(double));
    return SHARK_OK;
}
int32_t oracle_turb_kick(oracle_state* s) {
    if (!s || s->ou_modes.empty()) return SHARK_ERR_INVALID_ARG;
    turb_kick(*s);
    return SHARK_OK;
}
int32_t oracle_turb_coef(const oracle_state* s, double* modes, double* coef, int32_t* nm) {
    if (!s) return SHARK_ERR_INVALID_ARG;
    if (nm) *nm = (int32_t)(s->ou_modes.size() / 3);
    if (modes) std::memcpy(modes, s->ou_modes.data(), s->ou_modes.size() * sizeof(double));
    if (coef) std::memcpy(coef, s->ou_coef.data(), s->ou_coef.size() * sizeof(double));
    return SHARK_OK;
}
int32_t oracle_fargo(oracle_state* s) {
    if (!s || !s->flag(SHARK_FLAG_FARGO)) return SHARK_ERR_INVALID_ARG;
    fargo_scheme(*s);
    return SHARK_OK;
}
int32_t oracle_ctoprim(oracle_state* s) { if (!s) return SHARK_ERR_INVALID_ARG; ctoprim(*s); return SHARK_OK; }
int32_t oracle_courant(oracle_state* s, double* dt_out) {
    if (!s) return SHARK_ERR_INVALID_ARG;
    ctoprim(*s);
    if (s->flag(SHARK_FLAG_FORCE_KICK)) update_force_setup(*s);
    courant(*s);
    if (dt_out) *dt_out = s->dt;
    return SHARK_OK;
}
int32_t oracle_set_dt(oracle_state* s, double dt) { if (!s) return SHARK_ERR_INVALID_ARG; s->dt = dt; return SHARK_OK; }
int32_t oracle_dust_drag(oracle_state* s, double coeffdt) { if (!s) return SHARK_ERR_INVALID_ARG; dust_drag(*s, coeffdt); return SHARK_OK; }
int32_t oracle_compute_tstop(oracle_state* s) { if (!s) return SHARK_ERR_INVALID_ARG; ctoprim(*s); compute_tstop(*s); return SHARK_OK; }
int32_t oracle_get_tstop(const oracle_state* s, double* tstop) {
    if (!s || !tstop) return SHARK_ERR_INVALID_ARG;
    std::memcpy(tstop, s->tstop.data(), s->tstop.size() * sizeof(double));
    return SHARK_OK;
}
int32_t oracle_set_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
    return SHARK_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// output (src/commons/write_output.f90:2-300): the run's raw stream files, restated for the
// checks of the library's writer.  `prefix` + "output_" + five digits (title, iout) holds
// info.dat (formatted, the reference's labels and edit descriptors I11 / E23.15) and one
// unformatted stream file per field, active cells in cell order, unit-scaled: x (position(:,1)
// or radii_c for GEOM 2), rho (unit_d, or unit_dcol = unit_d unit_l for GEOM 2), v, y (2D:
// position(:,2)), vy, vz (unit_v), P (unit_P: unit_v^2, unit_d unit_v^2 in KH; times unit_l for
// GEOM 2), and with dust rhod_tot, rhod, sd (unit_l), vd, vdy, vdz (species-major), with charging
// eta_a, eta_o, eta_h, ni, ne, zd.  MHD, NDUSTPSCAL and the 1D-turbulence rms files are not part
// of any configuration here (MHD = NDUSTPSCAL = TURB = 0).  ctoprim runs first (the final dump of
// time_loop, shark.f90:114-118).
// ---------------------------------------------------------------------------------------------
namespace {
std::string fortran_i11(long long v) {
    char b[64];
    std::snprintf(b, sizeof b, "%11lld", v);
    return b;
}
// Fortran E23.15: [sign]0.ddddddddddddddd E+ee (the E dropped for three-digit exponents),
// right-justified in 23 characters.
std::string fortran_e23_15(double v) {
    char m[64];
    std::string body;
    if (v == 0.0) {
        body = std::string(std::signbit(v) ? "-" : "") + "0.000000000000000E+00";
    } else {
        std::snprintf(m, sizeof m, "%.14E", v);   // d.dddddddddddddddE+ee, 15 significant digits
        std::string s(m);
        const bool neg = s[0] == '-';
        if (neg) s = s.substr(1);
        const size_t epos = s.find('E');
        const std::string digits = s.substr(0, 1) + s.substr(2, epos - 2);
        const int e = std::atoi(s.c_str() + epos + 1) + 1;
        char ex[16];
        if (std::abs(e) <= 99) std::snprintf(ex, sizeof ex, "E%c%02d", e < 0 ? '-' : '+', std::abs(e));
        else std::snprintf(ex, sizeof ex, "%c%03d", e < 0 ? '-' : '+', std::abs(e));
        body = std::string(neg ? "-" : "") + "0." + digits + ex;
    }
    return std::string(body.size() < 23 ? 23 - body.size() : 0, ' ') + body;
}
bool write_stream(const std::string& path, const std::vector<double>& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(v.data(), sizeof(double), v.size(), f) == v.size();
    return std::fclose(f) == 0 && ok;
}
}  // namespace

int32_t oracle_output(oracle_state* s, int32_t iout, double time, const char* prefix) {
    if (!s || !prefix || iout < 0 || iout > 99999) return SHARK_ERR_INVALID_ARG;
    ctoprim(*s);
    const auto& g = s->cfg;
    const double ul = unit_or_1(g.unit_l), ud = unit_or_1(g.unit_d), ut = unit_or_1(g.unit_t);
    // unit_P: unit_v**2 (disk_polar/units.f90, 1 in the unit-free setups), unit_d unit_v**2 in KH/units.f90
    const double uv = ul / ut, uP = g.setup == SHARK_SETUP_KH ? ud * (uv * uv) : uv * uv, udcol = ud * ul;
    const bool polar = g.geom == 2;
    char nchar[8];
    std::snprintf(nchar, sizeof nchar, "%05d", iout);
    const std::string dir = std::string(prefix) + "output_" + nchar;
    mkdir(dir.c_str(), 0755);
    const bool charging = (g.flags & SHARK_FLAG_CHARGING) != 0;
    {
        FILE* f = std::fopen((dir + "/info.dat").c_str(), "w");
        if (!f) return SHARK_ERR_INVALID_ARG;
        std::fprintf(f, "nvar        =%s\n", fortran_i11(s->nvar).c_str());
        std::fprintf(f, "ndust        =%s\n", fortran_i11(s->ndust).c_str());
        std::fprintf(f, "ndustpscal   =%s\n", fortran_i11(0).c_str());
        std::fprintf(f, "NX        =%s\n", fortran_i11(s->nx).c_str());
        std::fprintf(f, "NY        =%s\n", fortran_i11(s->ny).c_str());
        std::fprintf(f, "MHD        =%s\n", fortran_i11(0).c_str());
        std::fprintf(f, "GEOM        =%s\n", fortran_i11(g.geom).c_str());
        std::fprintf(f, "TURB        =%s\n", fortran_i11(0).c_str());
        std::fprintf(f, "GRIDSPACE       =%s\n", fortran_i11(g.gridspace).c_str());
        std::fprintf(f, "time        =%s\n", fortran_e23_15(time).c_str());
        std::fprintf(f, "unit_t        =%s\n", fortran_e23_15(ut).c_str());
        std::fprintf(f, "unit_d        =%s\n", fortran_e23_15(ud).c_str());
        std::fprintf(f, "unit_l        =%s\n", fortran_e23_15(ul).c_str());
        std::fprintf(f, "unit_v        =%s\n", fortran_e23_15(uv).c_str());
        std::fprintf(f, "unit_p        =%s\n", fortran_e23_15(uP).c_str());
        std::fprintf(f, "charging       =%s\n", fortran_i11(charging ? 1 : 0).c_str());
        std::fclose(f);
    }
    std::vector<int64_t> act;
    for (int64_t i = 0; i < s->ncells; ++i)
        if (s->active[i]) act.push_back(i);
    std::vector<double> buf;
    auto field = [&](const char* name, auto value) -> bool {
        buf.clear();
        for (int64_t i : act) buf.push_back(value(i));
        return write_stream(dir + "/" + name, buf);
    };
    auto species = [&](const char* name, auto value) -> bool {
        buf.clear();
        for (int k = 0; k < s->ndust; ++k)
            for (int64_t i : act) buf.push_back(value(i, k));
        return write_stream(dir + "/" + name, buf);
    };
    const double urho = polar ? udcol : ud;
    bool ok = field("x", [&](int64_t i) { return polar ? s->radii_c[i] : s->POS(i, 0); });
    ok = ok && field("rho", [&](int64_t i) { return s->Q(i, s->irho) * urho; });
    ok = ok && field("v", [&](int64_t i) { return s->Q(i, s->ivx) * uv; });
    if (s->ndim == 2) ok = ok && field("y", [&](int64_t i) { return s->POS(i, 1); });
    ok = ok && field("vy", [&](int64_t i) { return s->Q(i, s->ivy) * uv; });
    ok = ok && field("vz", [&](int64_t i) { return s->Q(i, s->ivz) * uv; });
    ok = ok && field("P", [&](int64_t i) { return polar ? s->Q(i, s->iP) * uP * ul : s->Q(i, s->iP) * uP; });
    if (s->ndust > 0) {
        ok = ok && field("rhod_tot", [&](int64_t i) {
            double t = 0.0;
            for (int k = 0; k < s->ndust; ++k) t = t + s->Q(i, s->irhod[k]) * urho;
            return t;
        });
        ok = ok && species("rhod", [&](int64_t i, int k) { return s->Q(i, s->irhod[k]) * urho; });
        ok = ok && species("sd", [&](int64_t i, int k) { return s->SDUST(i, k) * ul; });
        ok = ok && species("vd", [&](int64_t i, int k) { return s->Q(i, s->ivdx[k]) * uv; });
        ok = ok && species("vdy", [&](int64_t i, int k) { return s->Q(i, s->ivdy[k]) * uv; });
        ok = ok && species("vdz", [&](int64_t i, int k) { return s->Q(i, s->ivdz[k]) * uv; });
    }
    if (charging) {   // before the first charging call the reference's arrays hold zeros
        const bool have = !s->psi_old.empty();
        ok = ok && field("eta_a", [&](int64_t i) { return have ? s->eta_a[i] : 0.0; });
        ok = ok && field("eta_o", [&](int64_t i) { return have ? s->eta_o[i] : 0.0; });
        ok = ok && field("eta_h", [&](int64_t i) { return have ? s->eta_h[i] : 0.0; });
        ok = ok && field("ni", [&](int64_t i) { return have ? s->ni[i] : 0.0; });
        ok = ok && field("ne", [&](int64_t i) { return have ? s->ne[i] : 0.0; });
        if (s->ndust > 0)
            ok = ok && species("zd", [&](int64_t i, int k) { return have ? s->zd[(size_t)k * s->ncells + i] : 0.0; });
    }
    return ok ? SHARK_OK : SHARK_ERR_INVALID_ARG;
}
