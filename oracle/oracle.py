"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline/reference legs import this
module; the product package never does.  ``build()`` compiles oracle/shark_oracle.cpp with the
committed Makefile (portable flags, works on x86-64 and aarch64).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build(force=False):
    srcs = [os.path.join(HERE, "shark_oracle.cpp"), os.path.join(HERE, "shark_oracle.h"),
            os.path.join(HERE, "..", "include", "shark_gpu.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    subprocess.run(["make", "-s", "-C", HERE, "-B"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        D = C.POINTER(C.c_double)
        L.oracle_create.restype = P
        L.oracle_create.argtypes = [C.c_void_p]
        L.oracle_destroy.argtypes = [P]
        L.oracle_ncells.restype = C.c_int64
        L.oracle_ncells.argtypes = [P]
        L.oracle_nvar.restype = C.c_int32
        L.oracle_nvar.argtypes = [P]
        for name, extra in [("oracle_setup_ic", [C.c_double, C.c_uint64]),
                            ("oracle_get_u", [D]), ("oracle_set_u", [D]),
                            ("oracle_get_q", [D, D]), ("oracle_get_cs", [D]), ("oracle_set_cs", [D]),
                            ("oracle_get_grid", [D, D, D, D, D]),
                            ("oracle_solve", [D]),
                            ("oracle_run", [C.c_int64, C.c_double, D, C.POINTER(C.c_int64)]),
                            ("oracle_totals", [D]),
                            ("oracle_apply_boundaries", []), ("oracle_ctoprim", []),
                            ("oracle_courant", [D]), ("oracle_set_dt", [C.c_double]),
                            ("oracle_dust_drag", [C.c_double]), ("oracle_compute_tstop", []),
                            ("oracle_get_tstop", [D]), ("oracle_fargo", []),
                            ("oracle_charge", [D, C.POINTER(C.c_int32)]),
                            ("oracle_get_charge", [D, D, D, D, D, D]),
                            ("oracle_reset_charge", []), ("oracle_charge_psi0", [D]),
                            ("oracle_growth", [C.POINTER(C.c_int32)]), ("oracle_growth_grid", [D, D, D]),
                            ("oracle_output", [C.c_int32, C.c_double, C.c_char_p]),
                            ("oracle_turb_kick", []), ("oracle_turb_coef", [D, D, C.POINTER(C.c_int32)])]:
            f = getattr(L, name)
            f.restype = C.c_int32
            f.argtypes = [P] + extra
        L.oracle_set_threads.restype = C.c_int32
        L.oracle_set_threads.argtypes = [C.c_int32]
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """One oracle run: ``Oracle(cfg)`` mirrors allocate_init + gridinit for that config."""

    def __init__(self, cfg, threads=None):
        L = lib()
        if threads:
            L.oracle_set_threads(int(threads))
        self.cfg = cfg.copy()
        self._h = L.oracle_create(C.byref(self.cfg))
        if not self._h:
            raise ValueError("oracle_create rejected the configuration")
        self.ncells = L.oracle_ncells(self._h)
        self.nvar = L.oracle_nvar(self._h)
        self.time = 0.0

    def close(self):
        if self._h:
            lib().oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with {rc}")

    def setup_ic(self, noise_amp=0.0, seed=1):
        self._chk(lib().oracle_setup_ic(self._h, noise_amp, seed), "oracle_setup_ic")

    def get_u(self):
        u = np.empty(self.ncells * self.nvar)
        self._chk(lib().oracle_get_u(self._h, _dptr(u)), "oracle_get_u")
        return u

    def set_u(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.size == self.ncells * self.nvar
        self._chk(lib().oracle_set_u(self._h, _dptr(u)), "oracle_set_u")

    def get_q(self):
        q = np.empty(self.ncells * self.nvar)
        cs = np.empty(self.ncells)
        self._chk(lib().oracle_get_q(self._h, _dptr(q), _dptr(cs)), "oracle_get_q")
        return q, cs

    def set_cs(self, cs):
        cs = np.ascontiguousarray(cs, dtype=np.float64)
        self._chk(lib().oracle_set_cs(self._h, _dptr(cs)), "oracle_set_cs")

    def get_cs(self):
        cs = np.empty(self.ncells)
        self._chk(lib().oracle_get_cs(self._h, _dptr(cs)), "oracle_get_cs")
        return cs

    def grid(self):
        nd = 1 if self.cfg.ny == 1 else 2
        dx = np.empty(self.ncells * nd)
        surf = np.empty(self.ncells * nd)
        vol = np.empty(self.ncells)
        pos = np.empty(self.ncells * nd)
        rc = np.empty(self.ncells)
        self._chk(lib().oracle_get_grid(self._h, _dptr(dx), _dptr(surf), _dptr(vol), _dptr(pos), _dptr(rc)),
                  "oracle_get_grid")
        return dict(dx=dx.reshape(nd, -1), surf=surf.reshape(nd, -1), vol=vol,
                    position=pos.reshape(nd, -1), radii_c=rc)

    def solve(self):
        dt = C.c_double(0)
        self._chk(lib().oracle_solve(self._h, C.byref(dt)), "oracle_solve")
        return dt.value

    def run(self, nsteps, tend=float("inf")):
        t = C.c_double(self.time)
        n = C.c_int64(0)
        self._chk(lib().oracle_run(self._h, int(nsteps), float(tend), C.byref(t), C.byref(n)), "oracle_run")
        self.time = t.value
        return n.value

    def totals(self):
        out = np.empty(4 * (self.cfg.ndust + 1))
        self._chk(lib().oracle_totals(self._h, _dptr(out)), "oracle_totals")
        return out

    def courant(self):
        dt = C.c_double(0)
        self._chk(lib().oracle_courant(self._h, C.byref(dt)), "oracle_courant")
        return dt.value

    def set_dt(self, dt):
        self._chk(lib().oracle_set_dt(self._h, float(dt)), "oracle_set_dt")

    def dust_drag(self, coeffdt=1.0):
        self._chk(lib().oracle_dust_drag(self._h, float(coeffdt)), "oracle_dust_drag")

    def compute_tstop(self):
        self._chk(lib().oracle_compute_tstop(self._h), "oracle_compute_tstop")
        t = np.empty(self.ncells * self.cfg.ndust)
        self._chk(lib().oracle_get_tstop(self._h, _dptr(t)), "oracle_get_tstop")
        return t.reshape(self.cfg.ndust, -1)

    def apply_boundaries(self):
        self._chk(lib().oracle_apply_boundaries(self._h), "oracle_apply_boundaries")

    def charge(self, seed=None):
        """charge (ionisation.f90:4-214) on the current state; returns the Newton iteration
        count per cell.  ``seed`` (ncells) overrides the start point where nonzero."""
        it = np.zeros(self.ncells, dtype=np.int32)
        sd = None if seed is None else _dptr(np.ascontiguousarray(seed, dtype=np.float64))
        self._keep = seed
        self._chk(lib().oracle_charge(self._h, sd, it.ctypes.data_as(C.POINTER(C.c_int32))), "oracle_charge")
        return it

    def get_charge(self):
        """dict of zd (N, ncells), ni, ne, psi, eta (3, ncells: o, H, a), gamma_d (N, ncells)."""
        N, nc = self.cfg.ndust, self.ncells
        zd, gd = np.empty(N * nc), np.empty(N * nc)
        ni, ne, psi, eta = np.empty(nc), np.empty(nc), np.empty(nc), np.empty(3 * nc)
        self._chk(lib().oracle_get_charge(self._h, _dptr(zd), _dptr(ni), _dptr(ne), _dptr(psi), _dptr(eta),
                                          _dptr(gd)), "oracle_get_charge")
        return dict(zd=zd.reshape(N, nc), ni=ni, ne=ne, psi=psi, eta=eta.reshape(3, nc), gamma_d=gd.reshape(N, nc))

    def reset_charge(self):
        self._chk(lib().oracle_reset_charge(self._h), "oracle_reset_charge")

    def charge_psi0(self):
        v = C.c_double(0)
        self._chk(lib().oracle_charge_psi0(self._h, C.byref(v)), "oracle_charge_psi0")
        return v.value

    def growth(self):
        """dust_growth alone with the dt last set; returns the sub-steps per cell."""
        it = np.zeros(self.ncells, dtype=np.int32)
        self._chk(lib().oracle_growth(self._h, it.ctypes.data_as(C.POINTER(C.c_int32))), "oracle_growth")
        return it

    def output(self, iout, time, prefix=""):
        """output (write_output.f90:2-300) of the current state into prefix + "output_%05d"."""
        self._chk(lib().oracle_output(self._h, int(iout), float(time), prefix.encode()), "oracle_output")

    def growth_grid(self):
        """(zeta, eta, massmin), bin masses m_k, fragment shares redis[ifrag][k]."""
        z = np.zeros(3)
        N = self.cfg.ndust
        mk, rd = np.zeros(N), np.zeros(N * N)
        self._chk(lib().oracle_growth_grid(self._h, _dptr(z), _dptr(mk), _dptr(rd)), "oracle_growth_grid")
        return z, mk, rd.reshape(N, N)

    def turb_kick(self):
        self._chk(lib().oracle_turb_kick(self._h), "oracle_turb_kick")

    def turb_coef(self):
        """(modes (nm, 3): kx', ky', |k'|; coefficients (nm, 2))."""
        nm = C.c_int32(0)
        self._chk(lib().oracle_turb_coef(self._h, None, None, C.byref(nm)), "oracle_turb_coef")
        m, c = np.zeros(3 * nm.value), np.zeros(2 * nm.value)
        self._chk(lib().oracle_turb_coef(self._h, _dptr(m), _dptr(c), C.byref(nm)), "oracle_turb_coef")
        return m.reshape(-1, 3), c.reshape(-1, 2)

    def fargo(self):
        """fargo_scheme alone on the current state with the dt last set (FARGO configs)."""
        self._chk(lib().oracle_fargo(self._h), "oracle_fargo")
