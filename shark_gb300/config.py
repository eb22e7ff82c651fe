"""ctypes mirror of ``shark_gpu_config`` (include/shark_gpu.h) and the constants of the C ABI.

The field order and types must match the C struct exactly; ``tests/test_capi_cpu.py`` checks the
size and the offsets of the default-filled fields against the compiled library.
"""
import ctypes as C
import struct

ABI_VERSION = 2
MAX_DUST = 64

OK = 0
ERR_INVALID_ARG = -1
ERR_UNSUPPORTED = -2
ERR_CUDA = -3
ERR_NO_DEVICE = -4
ERR_STATE = -5
ERR_NUMERICS = -6

STATUS_NAN = 0x1
STATUS_NEG_DENSITY = 0x2
STATUS_DT_UNDERFLOW = 0x4
STATUS_NEWTON = 0x8
STATUS_GROWTH = 0x10
STATUS_COPY_WAIT = 0x20

SETUP_SOD = 1
SETUP_DUSTYWAVE = 2
SETUP_SI = 3
SETUP_DISK_POLAR = 4
SETUP_DUSTYTURB = 5
SETUP_KH = 6
SETUP_SEDOV = 7
SETUP_DISK_CART = 8

FLAG_DRAG = 0x1
FLAG_BACK_REACTION = 0x2
FLAG_FORCE_KICK = 0x4
FLAG_FARGO = 0x8
FLAG_GROWTH = 0x10
FLAG_CHARGING = 0x20
FLAG_VISCOSITY = 0x40
FLAG_STATIC = 0x80

CHARGE_RESISTIVITIES = 0x1
CHARGE_ANALYTICAL = 0x2
CHARGE_MLP_SEED = 0x4

GROWTH_FRAGMENTATION = 0x1
GROWTH_DRIFT = 0x2
GROWTH_TURB = 0x4
GROWTH_BROWNIAN = 0x8
GROWTH_AMBIPOLAR = 0x10

PREC_FP64 = 0
PREC_MIXED = 1

_D = C.c_double
_I = C.c_int32
_P = C.POINTER(C.c_double)


class SharkConfig(C.Structure):
    _fields_ = [
        ("abi_version", _I), ("nx", _I), ("ny", _I), ("nghost", _I), ("ndust", _I),
        ("geom", _I), ("gridspace", _I), ("solver", _I), ("solverdust", _I),
        ("slope_type", _I), ("iso_cs", _I), ("precision", _I), ("setup", _I),
        ("flags", _I), ("device", _I), ("pad0", _I),
        ("gamma", _D), ("cfl", _D), ("smallr", _D), ("smallc", _D), ("smallp", _D),
        ("box_l", _D), ("box_l_y", _D), ("inner_r", _D), ("cs0", _D),
        ("dust_ratio_min", _D), ("rhograin", _D),
        ("dust_size", _D * MAX_DUST), ("dust_K", _D * MAX_DUST), ("dust_tstop", _D * MAX_DUST),
        ("dust_eps", _D * MAX_DUST), ("dust_stokes", _D * MAX_DUST),
        ("sod_rho_l", _D), ("sod_rho_r", _D), ("sod_P_l", _D), ("sod_P_r", _D),
        ("sod_direction", _I), ("pad1", _I),
        ("dw_rho_0", _D), ("dw_delta_rho", _D), ("dw_vx_0", _D), ("dw_kx_wave", _D),
        ("si_q_shear", _D), ("si_omega", _D), ("si_eta_stream", _D), ("si_rad0", _D),
        ("si_rho_init", _D), ("si_hoverr", _D),
        ("disk_mstar", _D), ("disk_hoverr", _D), ("disk_sigma0", _D), ("disk_r0", _D),
        ("disk_rout", _D), ("disk_r_relax", _D), ("disk_n_rel", _D), ("disk_temp_slope", _D),
        ("unit_l", _D), ("unit_d", _D), ("unit_t", _D), ("mu_gas", _D), ("T_cloud", _D),
        ("chg_x", _D), ("chg_sigma_att", _D), ("chg_mu_ions", _D), ("chg_stick_el", _D),
        ("chg_eps", _D), ("chg_B0", _D), ("chg_nitermax", _I), ("chg_mode", _I),
        ("turb_rho0", _D), ("turb_mach", _D), ("turb_tcorr", _D), ("turb_kmin", _I), ("turb_kmax", _I),
        ("turb_seed", _I), ("pad2", _I),
        ("grw_smin", _D), ("grw_smax", _D), ("grw_sticking", _D), ("grw_clustered", _D), ("grw_cfl", _D),
        ("grw_eps_thr", _D), ("grw_eps_thr_frag", _D), ("grw_dtcontrol", _D), ("grw_delta_vambi", _D),
        ("grw_alpha_turb", _D), ("grw_size_mono", _D), ("grw_slope_mono", _D), ("grw_Abr", _D),
        ("grw_gamma_grains", _D), ("grw_estar_grains", _D), ("grw_kernel", _I), ("grw_mode", _I),
        ("disk_alpha_visc", _D),
        ("kh_rho_dense", _D), ("kh_rho_diffuse", _D), ("kh_T_dense", _D), ("kh_mach", _D), ("kh_vy0", _D),
        ("kh_kx", _D),
        ("sedov_rho_ext", _D), ("sedov_P_ext", _D), ("sedov_P_cen", _D), ("sedov_r_expl", _D),
        ("cdisk_smooth_r", _D), ("cdisk_frac_r_disk", _D), ("cdisk_buffer_in", _D), ("cdisk_buffer_out", _D),
        ("dx", _P), ("surf", _P), ("vol", _P), ("radii_c", _P), ("position", _P), ("cs", _P),
    ]

    # convenience ------------------------------------------------------------------------
    @property
    def nvar(self):
        return 5 + 4 * self.ndust

    @property
    def ndim(self):
        return 1 if self.ny == 1 else 2

    @property
    def nx_max(self):
        return self.nx + 2 * self.nghost

    @property
    def ny_max(self):
        return 1 if self.ny == 1 else self.ny + 2 * self.nghost

    @property
    def ncells(self):
        return self.nx_max * self.ny_max

    def copy(self):
        c = SharkConfig()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(SharkConfig))
        return c


def default_config():
    """Reference defaults (hydro_commons.f90:16-24, parameters.f90:55, dust_commons.f90:5-29)."""
    c = SharkConfig()
    c.abi_version = ABI_VERSION
    c.nghost = 2
    c.ny = 1
    c.solver = 2
    c.solverdust = 0
    c.slope_type = 1
    c.iso_cs = -1
    c.precision = PREC_FP64
    c.flags = FLAG_DRAG | FLAG_BACK_REACTION
    c.gamma = 1.66667
    c.cfl = 0.5
    c.smallr = 1e-27
    c.smallc = 1e-27
    c.smallp = c.smallr * c.smallc ** 2      # allocate_init.f90:279
    c.box_l = 1.0
    c.box_l_y = 1.0
    c.dust_ratio_min = 1e-11
    c.rhograin = 2.7
    c.unit_l = c.unit_d = c.unit_t = 1.0
    c.mu_gas = 2.31                           # setups' setup_commons.f90
    c.T_cloud = 10.0                          # dustyTurb/setup_commons.f90:18
    c.chg_x = 5e-17                           # ionisation_commons.f90:73-77
    c.chg_mu_ions = 25.0
    c.chg_stick_el = 0.5
    c.chg_eps = 1e-6
    c.chg_nitermax = 1000
    c.chg_B0 = 3e-5
    c.chg_mode = CHARGE_RESISTIVITIES         # res_Marchand = .true.
    c.grw_sticking = 1.0                      # dust_commons.f90:17-63
    c.grw_clustered = 1.0
    c.grw_cfl = 0.1
    c.grw_eps_thr = 1e-10
    c.grw_eps_thr_frag = 1e-10
    c.grw_dtcontrol = -1.0
    c.grw_delta_vambi = 1.0
    c.grw_alpha_turb = 1.5
    c.grw_size_mono = 1e-5
    c.grw_slope_mono = 3.5
    c.grw_Abr = 2.8e3
    c.grw_gamma_grains = 25.0
    c.grw_estar_grains = 2.8e11
    c.disk_alpha_visc = 1e-2                  # disk_polar/setup_commons.f90:21
    c.kh_rho_dense, c.kh_rho_diffuse = 1.0, 0.8              # KH/setup_commons.f90:8-9
    c.kh_T_dense, c.kh_mach, c.kh_vy0, c.kh_kx = 10.0, 0.5, 0.1, 10.0   # KH/setup_commons.f90:13-19
    c.sedov_rho_ext, c.sedov_P_cen = 1.0, 1.0                # sedov/setup_commons.f90:9-10
    c.sedov_P_ext = 1e-5                                     # sedov/setup_commons.f90:11
    c.sedov_r_expl = struct.unpack("f", struct.pack("f", 0.1))[0]   # `r_expl=0.1`: a default-REAL literal
    return c
