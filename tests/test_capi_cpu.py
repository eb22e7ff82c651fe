"""C-ABI checks that need no GPU: the library loads, exports every symbol include/shark_gpu.h
declares, the ctypes mirror of shark_gpu_config has the C layout, and the error paths that run
before any device call return the documented codes."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from shark_gb300 import build as gbuild, config as K, setups
from shark_gb300.config import SharkConfig
from shark_gb300 import solver

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "shark_gpu.h")


@pytest.fixture(scope="module")
def lib():
    gbuild.build()
    return solver.load_library()


def test_every_declared_symbol_is_exported(lib):
    text = open(HEADER).read()
    declared = set(re.findall(r"\b(shark_gpu_\w+)\s*\(", text))
    declared -= {"shark_gpu_config"}
    assert declared == set(solver.EXPORTS), declared ^ set(solver.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", gbuild.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(shark_gpu_\w+)\b", out))
    missing = declared - exported
    assert not missing, missing
    for name in declared:
        getattr(lib, name)


def test_config_struct_layout_matches_c(tmp_path):
    fields = [f for f, _ in SharkConfig._fields_]
    src = tmp_path / "probe.c"
    body = "\n".join(f'  printf("{f} %zu\\n", offsetof(shark_gpu_config, {f}));' for f in fields)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "shark_gpu.h"\nint main(void){{\n'
                   f'  printf("sizeof %zu\\n", sizeof(shark_gpu_config));\n{body}\n  return 0;}}\n')
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    assert int(out["sizeof"]) == C.sizeof(SharkConfig)
    for f in fields:
        assert int(out[f]) == getattr(SharkConfig, f).offset, f


def test_defaults_and_abi_version(lib):
    assert lib.shark_gpu_abi_version() == K.ABI_VERSION
    c = SharkConfig()
    assert lib.shark_gpu_config_defaults(C.byref(c)) == K.OK
    py = K.default_config()
    for f, _ in SharkConfig._fields_:
        a, b = getattr(c, f), getattr(py, f)
        if isinstance(a, (int, float)):
            assert a == b, f


def test_invalid_configs_are_rejected_before_touching_a_device(lib):
    cfg, _ = setups.sod(nx=64)
    bad = cfg.copy()
    bad.abi_version = 99
    h = C.c_void_p()
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_INVALID_ARG
    bad = cfg.copy()
    bad.nghost = 3
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_UNSUPPORTED
    bad = cfg.copy()
    bad.flags |= K.FLAG_VISCOSITY
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_UNSUPPORTED
    assert b"viscosity" in lib.shark_gpu_last_error()
    bad = cfg.copy()
    bad.slope_type = 7
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_INVALID_ARG
    assert lib.shark_gpu_init(None, C.byref(h)) == K.ERR_INVALID_ARG
    assert lib.shark_gpu_step(None, None, None) == K.ERR_INVALID_ARG
    assert lib.shark_gpu_free(None) == K.OK


def test_hllc_dust_needs_an_isothermal_gas(lib):
    h = C.c_void_p()
    cfg, _ = setups.sod(nx=64, ndust=2)
    assert cfg.iso_cs != 1
    cfg.solverdust = 3
    assert lib.shark_gpu_init(C.byref(cfg), C.byref(h)) == K.ERR_UNSUPPORTED
    assert b"isothermal" in lib.shark_gpu_last_error()
    cfg.solverdust = 4
    assert lib.shark_gpu_init(C.byref(cfg), C.byref(h)) == K.ERR_UNSUPPORTED


def test_disk_and_fargo_configs_are_checked_before_touching_a_device(lib):
    h = C.c_void_p()
    si, _ = setups.si(n=32, ndust=2)
    bad = si.copy()
    bad.flags |= K.FLAG_FARGO          # the orbital velocity exists for the disk setups only
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_UNSUPPORTED
    assert b"FARGO" in lib.shark_gpu_last_error()
    disk, _ = setups.disk_polar(nr=32, nphi=32, ndust=2, fargo=True)
    bad = disk.copy()
    bad.geom = 0
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_UNSUPPORTED
    bad = disk.copy()
    bad.ny = 8192                      # a ring that does not fit one CTA's shared memory
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_UNSUPPORTED
    bad = disk.copy()
    bad.disk_mstar = 0.0
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_INVALID_ARG
    bad = disk.copy()
    bad.dust_size[1] = 0.0
    assert lib.shark_gpu_init(C.byref(bad), C.byref(h)) == K.ERR_INVALID_ARG


def test_no_cpu_fallback_without_a_gpu(lib):
    """On a machine without an sm_103 device the library refuses to run (no silent fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    cfg, _ = setups.sod(nx=64)
    with pytest.raises(solver.SharkError) as e:
        solver.Shark(cfg)
    assert e.value.code == K.ERR_NO_DEVICE


# ---- the Fortran side of the boundary (shark_gb300/fortran/), checked without a Fortran compiler --
FORTRAN = os.path.join(ROOT, "shark_gb300", "fortran")
_FKIND = {"integer(c_int32_t)": (4, 4), "real(c_double)": (8, 8), "type(c_ptr)": (8, 8)}


def _fortran_config_layout():
    """Offsets of the bind(C) derived type shark_gpu_config of shark_gpu_mod.f90, laid out with the
    C rules bind(C) promises (natural alignment of c_int32_t, c_double and c_ptr, arrays packed)."""
    text = open(os.path.join(FORTRAN, "shark_gpu_mod.f90")).read()
    body = re.search(r"type, bind\(C\) :: shark_gpu_config\n(.*?)\n\s*end type shark_gpu_config", text, re.S).group(1)
    consts = {"SHARK_MAX_DUST": 64}
    off, layout = 0, {}
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        kind, names = [x.strip() for x in line.split("::")]
        size, align = _FKIND[kind]
        for m in re.finditer(r"(\w+)(?:\((\w+)\))?", names):
            n = 1 if m.group(2) is None else int(consts.get(m.group(2), m.group(2)))
            off = (off + align - 1) // align * align
            layout[m.group(1).lower()] = off
            off += size * n
    return layout, (off + 7) // 8 * 8


def test_fortran_config_type_matches_the_c_struct():
    layout, size = _fortran_config_layout()
    c_fields = {f.lower(): getattr(SharkConfig, f).offset for f, _ in SharkConfig._fields_}
    assert size == C.sizeof(SharkConfig)
    assert set(layout) == set(c_fields), set(layout) ^ set(c_fields)
    for f, off in layout.items():
        assert off == c_fields[f], f


def test_fortran_shim_writes_only_existing_fields_and_maps_every_setup():
    layout, _ = _fortran_config_layout()
    src = open(os.path.join(FORTRAN, "solve_gpu.f90")).read()
    written = {m.lower() for m in re.findall(r"\bcfg%(\w+)", src)}
    assert written <= set(layout), written - set(layout)
    # the per-setup parameters of every setup id the library accepts
    for sid in range(1, 9):
        assert f"#if SHARK_GPU_SETUP=={sid}" in src, sid
    for f in ("disk_mstar", "disk_hoverr", "disk_sigma0", "disk_r_relax", "disk_n_rel", "disk_temp_slope",
              "turb_rho0", "t_cloud", "dust_stokes", "turb_mach", "turb_tcorr", "turb_kmin", "turb_kmax",
              "chg_x", "chg_eps", "chg_nitermax", "chg_mode", "grw_smin", "grw_smax", "grw_cfl", "grw_mode",
              "cdisk_smooth_r", "cdisk_frac_r_disk", "cdisk_buffer_in", "cdisk_buffer_out", "dust_eps"):
        assert f in written, f
    # before an output step the charging outputs come back with the state
    assert "shark_gpu_download_charge" in src
    mod = open(os.path.join(FORTRAN, "shark_gpu_mod.f90")).read()
    assert 'bind(C, name="shark_gpu_download_charge")' in mod
    bound = set(re.findall(r'bind\(C, name="(shark_gpu_\w+)"\)', mod))
    assert bound <= set(solver.EXPORTS), bound - set(solver.EXPORTS)
