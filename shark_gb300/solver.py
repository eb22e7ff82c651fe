"""Host-side mirror of the reference's step interface over the C ABI (include/shark_gpu.h).

The reference exposes one step as ``solve(verbose, outputing)`` (src/solver/solve.f90:10-181),
the primitive recovery as ``ctoprim`` (src/solver/solve.f90:195-253) and the run loop as
``time_loop`` (src/shark.f90:39-119).  :class:`Shark` offers the same calls over a device-resident
state.  There is no CPU fallback: constructing a :class:`Shark` without the compiled library or
without an sm_103 GPU raises.
"""
import ctypes as C
import os

import numpy as np

from .config import SharkConfig, OK

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libshark_gpu.so")
_lib = None

# every symbol include/shark_gpu.h declares
EXPORTS = [
    "shark_gpu_abi_version", "shark_gpu_config_defaults", "shark_gpu_init", "shark_gpu_upload",
    "shark_gpu_step", "shark_gpu_run", "shark_gpu_sync", "shark_gpu_download", "shark_gpu_ctoprim",
    "shark_gpu_totals", "shark_gpu_last_step_ms", "shark_gpu_timed_run", "shark_gpu_kernel_times",
    "shark_gpu_totals_noalloc", "shark_gpu_last_error", "shark_gpu_free",
    "shark_gpu_charge", "shark_gpu_charge_reset", "shark_gpu_charge_stats", "shark_gpu_download_charge",
    "shark_gpu_mlp_collect", "shark_gpu_mlp_train", "shark_gpu_mlp_save", "shark_gpu_mlp_load",
    "shark_gpu_mlp_eval", "shark_gpu_mlp_features", "shark_gpu_output", "shark_gpu_read_output",
]
MLP_NFEAT, MLP_NPARAM, MLP_NBLOB = 6, 5313, 5327
CHARGE_HIST = 64   # SHARK_CHARGE_HIST


class SharkError(RuntimeError):
    def __init__(self, code, what, msg):
        super().__init__(f"{what} returned {code}: {msg}")
        self.code = code


def load_library(path=None):
    """Load libshark_gpu.so (built by shark_gb300.build).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run shark_gb300.build.build() (nvcc, sm_103a)")
    L = C.CDLL(path)
    P = C.c_void_p
    D = C.POINTER(C.c_double)
    I32 = C.c_int32
    L.shark_gpu_abi_version.restype = I32
    L.shark_gpu_abi_version.argtypes = []
    L.shark_gpu_config_defaults.restype = I32
    L.shark_gpu_config_defaults.argtypes = [C.POINTER(SharkConfig)]
    L.shark_gpu_init.restype = I32
    L.shark_gpu_init.argtypes = [C.POINTER(SharkConfig), C.POINTER(P)]
    L.shark_gpu_upload.restype = I32
    L.shark_gpu_upload.argtypes = [P, D, C.c_int64, I32]
    L.shark_gpu_step.restype = I32
    L.shark_gpu_step.argtypes = [P, D, C.POINTER(I32)]
    L.shark_gpu_run.restype = I32
    L.shark_gpu_run.argtypes = [P, C.c_int64, C.c_double, D, C.POINTER(C.c_int64), C.POINTER(I32)]
    L.shark_gpu_sync.restype = I32
    L.shark_gpu_sync.argtypes = [P, C.POINTER(I32)]
    L.shark_gpu_download.restype = I32
    L.shark_gpu_download.argtypes = [P, D, D]
    L.shark_gpu_ctoprim.restype = I32
    L.shark_gpu_ctoprim.argtypes = [P, D, D]
    L.shark_gpu_totals.restype = I32
    L.shark_gpu_totals.argtypes = [P, D]
    L.shark_gpu_last_step_ms.restype = I32
    L.shark_gpu_last_step_ms.argtypes = [P, C.POINTER(C.c_float)]
    L.shark_gpu_timed_run.restype = I32
    L.shark_gpu_timed_run.argtypes = [P, C.c_int64, D, C.POINTER(C.c_float)]
    L.shark_gpu_kernel_times.restype = I32
    L.shark_gpu_kernel_times.argtypes = [P, C.c_int64, C.POINTER(C.c_float)]
    L.shark_gpu_totals_noalloc.restype = I32
    L.shark_gpu_totals_noalloc.argtypes = [C.c_void_p, I32, I32, I32, I32, C.c_void_p, C.c_void_p]
    L.shark_gpu_last_error.restype = C.c_char_p
    L.shark_gpu_last_error.argtypes = []
    L.shark_gpu_free.restype = I32
    L.shark_gpu_free.argtypes = [P]
    I64P = C.POINTER(C.c_int64)
    FP = C.POINTER(C.c_float)
    for name, args in [("shark_gpu_charge", [P]), ("shark_gpu_charge_reset", [P]),
                       ("shark_gpu_charge_stats", [P, I64P, I64P, I64P]),
                       ("shark_gpu_download_charge", [P, D, D, D, D, D, D, C.POINTER(C.c_int32)]),
                       ("shark_gpu_mlp_collect", [P, C.c_int64, I64P]),
                       ("shark_gpu_mlp_train", [P, I32, I32, C.c_float, C.c_uint64, FP]),
                       ("shark_gpu_mlp_save", [P, FP, C.c_int64]), ("shark_gpu_mlp_load", [P, FP, C.c_int64]),
                       ("shark_gpu_mlp_eval", [P, FP, FP, C.c_int64, FP, FP, FP]),
                       ("shark_gpu_mlp_features", [P, FP]),
                       ("shark_gpu_output", [P, I32, C.c_double, C.c_char_p]),
                       ("shark_gpu_read_output", [P, C.c_char_p, D])]:
        f = getattr(L, name)
        f.restype = I32
        f.argtypes = args
    _lib = L
    return L


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _check(rc, what):
    if rc != OK:
        msg = load_library().shark_gpu_last_error().decode(errors="replace")
        raise SharkError(rc, what, msg)


def totals_noalloc(u_dev_ptr, nx, ny, nghost, ndust, out_dev_ptr, stream_ptr=None):
    """shark_gpu_totals_noalloc on caller-owned device buffers (raw device pointers); queued on
    `stream_ptr` (None = default stream), returns without synchronising."""
    _check(load_library().shark_gpu_totals_noalloc(C.c_void_p(u_dev_ptr), nx, ny, nghost, ndust,
                                                   C.c_void_p(out_dev_ptr), C.c_void_p(stream_ptr or 0)),
           "shark_gpu_totals_noalloc")


class Shark:
    """One device-resident run.  ``Shark(cfg)`` = allocate_init + gridinit on the GPU."""

    def __init__(self, cfg: SharkConfig):
        L = load_library()
        self.cfg = cfg.copy()
        self._h = C.c_void_p()
        _check(L.shark_gpu_init(C.byref(self.cfg), C.byref(self._h)), "shark_gpu_init")
        self.ncells = self.cfg.ncells
        self.nvar = self.cfg.nvar
        self.time = 0.0
        self.dt = 0.0
        self.status = 0

    # -- lifetime ------------------------------------------------------------------------------
    def close(self):
        if self._h:
            load_library().shark_gpu_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state ---------------------------------------------------------------------------------
    def upload(self, u_prim, time=0.0):
        """Hand the conserved state (Fortran order, ncells*nvar) to the device."""
        u = np.ascontiguousarray(u_prim, dtype=np.float64).reshape(-1)
        if u.size != self.ncells * self.nvar:
            raise ValueError(f"state has {u.size} values, expected {self.ncells * self.nvar}")
        _check(load_library().shark_gpu_upload(self._h, _dptr(u), self.ncells, self.nvar), "shark_gpu_upload")
        self.time = float(time)

    def upload_ptr(self, ptr):
        """Upload from a raw host pointer (e.g. pinned memory) without a copy in Python."""
        _check(load_library().shark_gpu_upload(self._h, C.cast(ptr, C.POINTER(C.c_double)), self.ncells, self.nvar),
               "shark_gpu_upload")

    def download(self, out=None):
        """u_prim as the host sees it (ghost cells included)."""
        u = np.empty(self.ncells * self.nvar) if out is None else out
        _check(load_library().shark_gpu_download(self._h, _dptr(u), None), "shark_gpu_download")
        return u

    def download_ptr(self, ptr):
        _check(load_library().shark_gpu_download(self._h, C.cast(ptr, C.POINTER(C.c_double)), None),
               "shark_gpu_download")

    u_prim = property(download)

    # -- output / restart (src/commons/write_output.f90:2-300) ----------------------------------
    def output(self, iout, time=None, prefix=""):
        """Write prefix + "output_%05d" (info.dat and the raw field streams) of the current state."""
        t = self.time if time is None else float(time)
        _check(load_library().shark_gpu_output(self._h, int(iout), t, prefix.encode()), "shark_gpu_output")
        return os.path.join(prefix, "output_%05d" % int(iout)) if prefix else "output_%05d" % int(iout)

    def read_output(self, directory):
        """Restart from an output directory: upload its state; returns (and keeps) its time."""
        t = C.c_double(0.0)
        _check(load_library().shark_gpu_read_output(self._h, str(directory).encode(), C.byref(t)),
               "shark_gpu_read_output")
        self.time = t.value
        return t.value

    def ctoprim(self):
        """(q, cs) of the current device state (src/solver/solve.f90:195-253)."""
        q = np.empty(self.ncells * self.nvar)
        cs = np.empty(self.ncells)
        _check(load_library().shark_gpu_ctoprim(self._h, _dptr(q), _dptr(cs)), "shark_gpu_ctoprim")
        return q, cs

    def totals(self):
        """Kahan-compensated FP64 [mass, px, py, pz] per species (gas first) over active cells."""
        out = np.empty(4 * (self.cfg.ndust + 1))
        _check(load_library().shark_gpu_totals(self._h, _dptr(out)), "shark_gpu_totals")
        return out.reshape(self.cfg.ndust + 1, 4)

    # -- stepping ------------------------------------------------------------------------------
    def solve(self, verbose=False, outputing=False):
        """One step; returns the dt that courant set for it (src/solver/solve.f90:10-181)."""
        dt = C.c_double(0.0)
        st = C.c_int32(0)
        _check(load_library().shark_gpu_step(self._h, C.byref(dt), C.byref(st)), "shark_gpu_step")
        self.dt = dt.value
        self.status = st.value
        return self.dt

    def time_loop(self, tend, max_steps=1 << 62):
        """Steps until time >= tend (dt is not clipped, as in src/shark.f90:71-110)."""
        t = C.c_double(self.time)
        n = C.c_int64(0)
        st = C.c_int32(0)
        _check(load_library().shark_gpu_run(self._h, int(max_steps), float(tend), C.byref(t), C.byref(n),
                                            C.byref(st)), "shark_gpu_run")
        self.time = t.value
        self.status = st.value
        return n.value

    def run_steps(self, nsteps):
        """Exactly nsteps steps (no end time)."""
        return self.time_loop(float("inf"), max_steps=nsteps)

    def sync(self):
        st = C.c_int32(0)
        _check(load_library().shark_gpu_sync(self._h, C.byref(st)), "shark_gpu_sync")
        self.status = st.value
        return st.value

    def timed_run(self, nsteps):
        """nsteps steps between two CUDA events on the library's stream; returns device ms."""
        t = C.c_double(self.time)
        ms = C.c_float(0.0)
        _check(load_library().shark_gpu_timed_run(self._h, int(nsteps), C.byref(t), C.byref(ms)),
               "shark_gpu_timed_run")
        self.time = t.value
        return ms.value

    def kernel_times(self, nsteps):
        """Mean device ms per launch: [boundaries, flux/update, drag+dt, whole step]."""
        ms = (C.c_float * 4)()
        _check(load_library().shark_gpu_kernel_times(self._h, int(nsteps), ms), "shark_gpu_kernel_times")
        return list(ms)

    def last_step_ms(self):
        ms = (C.c_float * 3)()
        _check(load_library().shark_gpu_last_step_ms(self._h, ms), "shark_gpu_last_step_ms")
        return list(ms)

    # ---- charging (SHARK_FLAG_CHARGING) ---------------------------------------------------------
    def charge(self):
        """Charge the current state now (src/chemistry/ionisation.f90:4-214)."""
        _check(load_library().shark_gpu_charge(self._h), "shark_gpu_charge")

    def charge_reset(self):
        """psi_old = 0: the next charging call starts cold."""
        _check(load_library().shark_gpu_charge_reset(self._h), "shark_gpu_charge_reset")

    def charge_stats(self):
        """(iteration histogram[64], non-converged cells, total iterations) of the last call."""
        h = np.zeros(CHARGE_HIST, dtype=np.int64)
        nc, tot = C.c_int64(0), C.c_int64(0)
        _check(load_library().shark_gpu_charge_stats(self._h, h.ctypes.data_as(C.POINTER(C.c_int64)),
                                                     C.byref(nc), C.byref(tot)), "shark_gpu_charge_stats")
        return h, nc.value, tot.value

    def download_charge(self):
        """dict of zd (N, ncells), ni, ne, psi, eta (3, ncells), gamma_d (N, ncells), iters."""
        N, nc = self.cfg.ndust, self.ncells
        zd, gd = np.empty(N * nc), np.empty(N * nc)
        ni, ne, psi, eta = np.empty(nc), np.empty(nc), np.empty(nc), np.empty(3 * nc)
        it = np.zeros(nc, dtype=np.int32)
        _check(load_library().shark_gpu_download_charge(self._h, _dptr(zd), _dptr(ni), _dptr(ne), _dptr(psi),
                                                        _dptr(eta), _dptr(gd), it.ctypes.data_as(C.POINTER(C.c_int32))),
               "shark_gpu_download_charge")
        return dict(zd=zd.reshape(N, nc), ni=ni, ne=ne, psi=psi, eta=eta.reshape(3, nc), gamma_d=gd.reshape(N, nc),
                    iters=it)

    # ---- charging network (SHARK_CHARGE_MLP_SEED) -----------------------------------------------
    def mlp_collect(self, capacity=1 << 22):
        """Cold-charge the current state and add its converged (features, t) pairs to the
        training set; returns the number of pairs held."""
        n = C.c_int64(0)
        _check(load_library().shark_gpu_mlp_collect(self._h, int(capacity), C.byref(n)), "shark_gpu_mlp_collect")
        return n.value

    def mlp_train(self, steps, batch=4096, lr=1e-3, seed=1):
        """Train on the GPU; returns the mini-batch loss curve."""
        loss = np.zeros(steps, dtype=np.float32)
        _check(load_library().shark_gpu_mlp_train(self._h, int(steps), int(batch), float(lr), int(seed),
                                                  loss.ctypes.data_as(C.POINTER(C.c_float))), "shark_gpu_mlp_train")
        return loss

    def mlp_save(self):
        b = np.zeros(MLP_NBLOB, dtype=np.float32)
        _check(load_library().shark_gpu_mlp_save(self._h, b.ctypes.data_as(C.POINTER(C.c_float)), MLP_NBLOB),
               "shark_gpu_mlp_save")
        return b

    def mlp_load(self, blob):
        b = np.ascontiguousarray(blob, dtype=np.float32)
        _check(load_library().shark_gpu_mlp_load(self._h, b.ctypes.data_as(C.POINTER(C.c_float)), b.size),
               "shark_gpu_mlp_load")

    def mlp_eval(self, feat, target=None):
        """(t per sample, gradient or None, loss or None) of the network on raw features."""
        f = np.ascontiguousarray(feat, dtype=np.float32).reshape(-1, MLP_NFEAT)
        n = f.shape[0]
        out = np.zeros(n, dtype=np.float32)
        FPt = C.POINTER(C.c_float)
        if target is None:
            _check(load_library().shark_gpu_mlp_eval(self._h, f.ctypes.data_as(FPt), None, n,
                                                     out.ctypes.data_as(FPt), None, None), "shark_gpu_mlp_eval")
            return out, None, None
        t = np.ascontiguousarray(target, dtype=np.float32)
        g = np.zeros(MLP_NPARAM, dtype=np.float32)
        loss = C.c_float(0)
        _check(load_library().shark_gpu_mlp_eval(self._h, f.ctypes.data_as(FPt), t.ctypes.data_as(FPt), n,
                                                 out.ctypes.data_as(FPt), g.ctypes.data_as(FPt), C.byref(loss)),
               "shark_gpu_mlp_eval")
        return out, g, loss.value

    def mlp_features(self):
        f = np.zeros(self.ncells * MLP_NFEAT, dtype=np.float32)
        _check(load_library().shark_gpu_mlp_features(self._h, f.ctypes.data_as(C.POINTER(C.c_float))),
               "shark_gpu_mlp_features")
        return f.reshape(self.ncells, MLP_NFEAT)
