"""Benchmark: zone-species updates per second of SHARK's per-step Godunov update on one GB300.

Workload (default): the 2D streaming-instability shearing box, 1024 x 1024 active cells over
0.2H x 0.2H, 8 dust species (Stokes 1e-3..1, MRN), dust-to-gas 0.02, Pi = 0.05, NSH equilibrium
plus seeded 1e-3 cs white noise on the dust velocities, force kick + implicit drag.  One "step" is
one `solve` (src/solver/solve.f90:10-181) of that box; 1 zone-species update = one active cell x
one species (gas counts as one) x one step, so one step is 1024^2 x 9 = 9,437,184 updates.

  value       mixed path (FP32 state + flux/update, FP64 drag/dt), state resident in HBM, timed
              with CUDA events on the library's stream around K steps.
  e2e         the same steps through the C ABI with HOST buffers: every step uploads the state
              from pinned host memory, runs `shark_gpu_step`, and downloads the state again.
  fp64        the FP64 path on the same workload (same K), its L1 distance to the mixed path.
  roofline    the fused flux/update kernel (K1): algorithmic bytes 2 x 4 B x nvar per active cell
              per launch over its mean event-timed duration, against MEASURED_PEAKS.json hbm_gbs.
  cpu_baseline the C++ FP64 OpenMP oracle (a restatement of the Fortran, "port") on the host cores,
              a bounded sample of the same workload.

  workloads   (default SI run) the polar disk with FARGO, growth and charging (512 x 1024, 16
              species) and the driven dusty turbulence with charging and growth (2048^2, 32
              species): mixed and FP64 ms/step, their L1 distance, charging iterations.
  charging_mlp (default SI run) the charging network trained on the GPU on (state, converged psi)
              pairs of dusty boxes, then the cold-start Newton iterations on the 2048^2 box with
              and without its seed, at the same residual tolerance.

`--workload disk|turb` prints the same line for one of those two configurations instead.
`--impl reference` times that CPU implementation alone on the host cores (rank 0 only).
Multi-GPU (torchrun): independent replicas, one per GPU; value = total updates / max time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "zone-species updates/s on 1 GB300, mixed vs FP64 GPU at fixed L1 error"
L1_STEPS = 100     # steps from the initial state at which the mixed path's L1 to FP64 is stated
UNIT = "zone-species updates/s"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def max_over_ranks(x, world, device):
    """The largest of a per-rank time over all ranks (the slowest replica sets the job's time)."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_step, steps, world, seconds):
    """Whole-job rate of `world` independent replicas: the units all ranks processed over the
    slowest rank's time (the path has no exchange step, so ranks only share the clock)."""
    return units_per_step * steps * world / seconds


def workload(args, precision, name=None):
    from shark_gb300 import setups
    name = name or args.workload
    if name == "disk":   # polar disk 1-100 AU, FARGO, growth, charging (MLP-seedable Newton)
        return setups.disk_polar_au(growth=True, precision=precision)
    if name == "turb":   # driven dusty turbulence, charging and growth every step (--n: smaller boxes)
        n = args.n if (name == args.workload and getattr(args, "n_given", False)) else 2048
        return setups.dusty_turb(n=n, ndust=32, forcing=True, charging=True, growth=True, precision=precision)
    return setups.si(n=args.n, ndust=args.ndust, precision=precision, noise=1e-3, seed=1)


def describe(args, cfg):
    if args.workload == "disk":
        return (f"polar disk {cfg.nx}x{cfg.ny} (log r 1-100 AU x phi), {cfg.ndust} dust species 1 um-1 cm, FARGO, "
                f"growth, charging, mixed precision")
    if args.workload == "turb":
        return (f"driven dusty turbulence {cfg.nx}x{cfg.ny}, {cfg.ndust} dust species 0.01 um-1 mm, OU forcing, "
                f"charging and growth every step, mixed precision")
    return f"SI shearing box {cfg.nx}x{cfg.ny} active cells, {cfg.ndust} dust species"


def launches_per_step(cfg):
    """Kernels of one mixed-precision step: k_prepare_step, charging, forcing update, K1 (one launch
    on Cartesian grids with the Huang & Bai dust solver, gas and dust launches otherwise), FARGO, K2."""
    from shark_gb300 import config as K
    n = 2
    n += 1 if cfg.flags & K.FLAG_CHARGING else 0
    n += 1 if getattr(cfg, "turb_mach", 0.0) > 0.0 else 0
    cart_hb = cfg.geom != 2 and cfg.solverdust == 0 and cfg.ndust > 0
    n += 1 if (cart_hb or cfg.ndust == 0) else 2
    n += 1 if cfg.flags & K.FLAG_FARGO else 0
    return n


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 50 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def rel_l1_max(cfg, a, b):
    """Max over conserved fields of the relative L1 distance (densities/energy by their own L1
    norm, momentum components by their species' momentum-magnitude L1 norm)."""
    g = cfg.nghost
    A = a.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)[:, g:-g, g:-g]
    B = b.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)[:, g:-g, g:-g]
    N = cfg.ndust
    sc = np.abs(B).sum(axis=(1, 2))
    for c in [(1, 2, 3)] + [(5 + N + k, 5 + 2 * N + k, 5 + 3 * N + k) for k in range(N)]:
        mag = np.sqrt(B[c[0]] ** 2 + B[c[1]] ** 2 + B[c[2]] ** 2).sum()
        for v in c:
            sc[v] = mag
    num = np.abs(A - B).sum(axis=(1, 2))
    return float((num / np.maximum(sc, 1e-300)).max())


def cpu_oracle_rate(args, max_seconds=25.0, n_small=None):
    """Time the FP64 OpenMP oracle on the host cores on a bounded sample of the workload."""
    from oracle.oracle import Oracle
    from shark_gb300 import config as K
    cores = os.cpu_count() or 1
    if args.workload == "turb":
        from shark_gb300 import setups
        cfg, u0 = setups.dusty_turb(n=128, ndust=32, forcing=True, charging=True, growth=True)
        sample = "driven dusty turbulence 128x128 (sub-box of the 2048^2 case), 32 species, charging and growth"
    elif args.workload == "disk":
        from shark_gb300 import setups
        cfg, u0 = setups.disk_polar_au(nr=128, nphi=256, growth=True)
        sample = "polar disk 128x256 (coarser grid of the 512x1024 case), 16 species, FARGO, growth, charging"
    else:
        cfg, u0 = workload(args, K.PREC_FP64)
        sample = f"SI {args.n}x{args.n}, {args.ndust} species"
    if n_small:
        from shark_gb300 import setups
        cfg, u0 = setups.si(n=n_small, ndust=args.ndust, noise=1e-3, seed=1)
        sample = f"SI {n_small}x{n_small}, {args.ndust} species (sub-grid of the {args.n}^2 box)"
    o = Oracle(cfg, threads=cores)
    o.set_u(u0)
    t0 = time.perf_counter()
    o.solve()                       # warm-up (page-in, thread pool)
    t1 = time.perf_counter()
    per = t1 - t0
    nsteps = max(1, min(20, int(max_seconds / max(per, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(nsteps):
        o.solve()
    el = time.perf_counter() - t0
    zs = cfg.nx * cfg.ny * (cfg.ndust + 1) * nsteps
    return zs / el, cores, f"{sample}, {nsteps} timed steps after 1 warm-up, {el:.1f} s", el / nsteps


def run_reference(args):
    rank, local_rank, world = dist_env()
    if rank != 0:
        return
    from oracle.oracle import build as obuild
    obuild()
    cores = os.cpu_count() or 1
    # size each step so that warmup + steps stay within ~2 minutes
    rate, cores, sample, per_step = cpu_oracle_rate(args, max_seconds=5.0)
    n = args.n
    budget = 120.0
    while per_step * (args.steps + args.warmup) > budget and n > 64:
        n //= 2
        per_step /= 4.0
    from oracle.oracle import Oracle
    from shark_gb300 import setups
    cfg, u0 = setups.si(n=n, ndust=args.ndust, noise=1e-3, seed=1)
    o = Oracle(cfg, threads=cores)
    o.set_u(u0)
    for _ in range(args.warmup):
        o.solve()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.solve()
    el = time.perf_counter() - t0
    zs = cfg.nx * cfg.ny * (cfg.ndust + 1)
    value = zs * args.steps / el
    samp = (f"SI {n}x{n} (the {args.n}^2 box at full size if n equals it), {args.ndust} species, "
            f"{args.steps} timed steps after {args.warmup} warm-up")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"SI shearing box {args.n}x{args.n} active cells, {args.ndust} dust species",
                   "zone_species_per_step": args.n * args.n * (args.ndust + 1),
                   "sample_grid": f"{n}x{n}", "parallelism": "OpenMP host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": samp},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "C++ FP64 OpenMP restatement of the Fortran path (no Fortran compiler on this image)",
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    from shark_gb300 import config as K, build as gbuild
    from shark_gb300.solver import Shark

    rank, local_rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    torch.cuda.set_device(local_rank)
    # rank 0 alone compiles; the others wait at the barrier and only load the library
    if rank == 0:
        gbuild.build()
    if world > 1:
        torch.distributed.barrier()
    from shark_gb300 import solver as gsolver
    gsolver.load_library()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- mixed path, state resident -----------------------------------------------------------
    cfg_m, u0 = workload(args, K.PREC_MIXED)
    cfg_m.device = local_rank
    zs_step = cfg_m.nx * cfg_m.ny * (cfg_m.ndust + 1)
    fp64_steps = args.steps if args.workload == "si" else min(args.steps, 3)
    gm = Shark(cfg_m)
    gm.upload(u0)
    for _ in range(args.warmup):
        gm.solve()
    gm.sync()
    barrier()
    # the K timed steps are run `repeats` times back to back (each run exactly K steps, events on
    # the library's stream); the median run is reported, all runs are listed
    runs = []
    with ClockSampler(local_rank) as clocks:
        for _ in range(args.repeats):
            barrier()
            runs.append(gm.timed_run(args.steps))
    barrier()
    ms = float(np.median(runs))
    ms_max = max_over_ranks(ms, world, "cuda")
    value = replica_rate(zs_step, args.steps, world, ms_max * 1e-3)
    st = gm.sync()

    # per-kernel times (separate pass, events around every launch)
    kt = gm.kernel_times(max(5, min(args.steps, 20)))
    u_mixed = gm.download()
    steps_done_m = args.warmup + args.repeats * args.steps + max(5, min(args.steps, 20))
    # the accuracy point of the metric: mixed against FP64 after L1_STEPS steps from the initial
    # state, whatever --steps and --repeats are (the distance grows with the step count)
    l1_steps = L1_STEPS if args.workload == "si" else 9    # FP64 steps of configs 4, 5 take 0.1-1.2 s
    gm.upload(u0)
    gm.run_steps(l1_steps)
    u_mixed_l1 = gm.download()

    # ---- FP64 path on the same workload ----------------------------------------------------
    cfg_d, _ = workload(args, K.PREC_FP64)
    cfg_d.device = local_rank
    gd = Shark(cfg_d)
    gd.upload(u0)
    for _ in range(args.warmup):
        gd.solve()
    ms_d = gd.timed_run(fp64_steps)
    done_d = args.warmup + fp64_steps
    if done_d <= l1_steps:
        gd.run_steps(l1_steps - done_d)
        done_d = l1_steps
        l1 = rel_l1_max(cfg_m, u_mixed_l1, gd.download())
    else:   # more FP64 steps timed than the accuracy point: a second FP64 run for it
        gd1 = Shark(cfg_d)
        gd1.upload(u0)
        gd1.run_steps(l1_steps)
        l1 = rel_l1_max(cfg_m, u_mixed_l1, gd1.download())
        gd1.close()
    l1_all = None
    if args.workload == "si":   # FP64 to the mixed run's own step count (17 ms a step)
        gd.run_steps(max(0, steps_done_m - done_d))
        l1_all = rel_l1_max(cfg_m, u_mixed, gd.download()) if steps_done_m >= done_d else None
    value_fp64 = zs_step * fp64_steps / (ms_d * 1e-3)
    kt_d = gd.kernel_times(3)
    gd.close()

    # ---- e2e: host state in, host state out, every step ------------------------------------
    nbytes = cfg_m.ncells * cfg_m.nvar * 8
    pinned = torch.empty(cfg_m.ncells * cfg_m.nvar, dtype=torch.float64).pin_memory()
    pinned.numpy()[:] = u_mixed
    ptr = pinned.data_ptr()
    e2e_steps = max(3, min(args.steps, 20))
    for _ in range(2):
        gm.upload_ptr(ptr)
        gm.solve()
        gm.download_ptr(ptr)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        gm.upload_ptr(ptr)
        gm.solve()
        gm.download_ptr(ptr)
    gm.sync()
    el = time.perf_counter() - t0
    barrier()
    e2e_value = replica_rate(zs_step, e2e_steps, world, max_over_ranks(el, world, "cuda"))
    # resident variant: what the Fortran driver does (solve + 8-byte dt readback per step)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        gm.solve()
    gm.sync()
    el_res = time.perf_counter() - t0
    gm.close()

    # ---- roofline of the flux/update kernel ---------------------------------------------------
    hbm, peak_kind = peaks()
    nvar = cfg_m.nvar
    ncell = cfg_m.nx * cfg_m.ny
    alg_bytes_k1 = 2 * 4 * nvar * ncell                      # read + write each conserved value once
    k1_s = kt[1] * 1e-3
    achieved = alg_bytes_k1 / k1_s / 1e9
    # K2 (drag, floor, CFL, ghost images): it reads the density and momentum of every species
    # (4S values) and writes every momentum (3S); the floor rewrites a dust density only where it
    # applies, so it is not counted: 4 B x 7S per active cell (252 B for 8 species)
    alg_bytes_k2 = 4 * 7 * (cfg_m.ndust + 1) * ncell
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "k_flux_traffic.txt")
    if os.path.exists(tfile) and args.workload == "si" and args.n == 1024 and args.ndust == 8:
        with open(tfile) as f:
            for line in f:
                if line.startswith("bytes_per_launch_full_size:"):
                    traffic = int(line.split(":")[1])

    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu:
        from oracle.oracle import build as obuild
        obuild()
        rate, cores, sample, _ = cpu_oracle_rate(args, max_seconds=20.0)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (flux/update) + f64 (drag, dt)",
        "data": "synthetic",
        "config": {"workload": describe(args, cfg_m), "zone_species_per_step": zs_step,
                   "parallelism": "replicas only" if world > 1 else "single GPU",
                   "l2": f"state (2 x {cfg_m.ncells * nvar * 4 / 1e6:.0f} MB ping-pong, FP32) larger than the "
                         f"129 MB L2; no flush"},
        "timed_runs_ms": runs,
        "kernel_ms": {"pre_flux": kt[0], "flux_update": kt[1], "drag_dt_ghosts": kt[2], "step": kt[3]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "kernel": "k_flux (K1 fused flux/update)",
                     "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes_k1,
                     "drag_kernel_bytes_per_cell": alg_bytes_k2 // ncell,
                     "drag_kernel_achieved_gbs": alg_bytes_k2 / (kt[2] * 1e-3) / 1e9,
                     "drag_kernel_frac": alg_bytes_k2 / (kt[2] * 1e-3) / 1e9 / hbm},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps,
                "note": "per step: shark_gpu_upload from pinned host FP64 u_prim, shark_gpu_step, shark_gpu_download",
                "resident_value": zs_step * e2e_steps / el_res,
                "resident_note": "state kept on the device, per step shark_gpu_step with its 12-byte dt/status readback"},
        "cpu_baseline": cpu,
        "gpu_launches": launches_per_step(cfg_m) * args.steps,
        "gpu_launches_note": launches_note(cfg_m),
        "status": st,
        "clocks": clocks.summary(),
    }
    if args.workload == "si" and world == 1 and not args.no_extra:
        line["workloads"] = {name: config_leg(args, name, local_rank) for name in ("disk", "turb")}
        line["charging_mlp"] = mlp_leg(local_rank)
    # last, so that the end of the line carries the precision comparison the metric is quoted at
    line["fp64"] = {"value": value_fp64, "unit": UNIT, "ms_per_step": ms_d / fp64_steps, "steps": fp64_steps,
                    "kernel_ms": {"pre_flux": kt_d[0], "flux_update": kt_d[1], "drag_dt_ghosts": kt_d[2],
                                  "step": kt_d[3]},
                    "mixed_over_fp64": value / world / value_fp64,
                    "l1_note": f"max relative L1 over the {nvar} conserved fields after {l1_steps} steps "
                               f"from the initial state; l1_after_all_steps: after the {steps_done_m} steps "
                               f"of this run (warm-up, timed runs, kernel timing)",
                    "l1_after_all_steps": l1_all,
                    "l1_mixed_vs_fp64": l1}
    print(json.dumps(line), flush=True)


def launches_note(cfg):
    from shark_gb300 import config as K
    parts = ["k_prepare_step"]
    if cfg.flags & K.FLAG_CHARGING:
        parts.append("k_charge")
    if getattr(cfg, "turb_mach", 0.0) > 0.0:
        parts.append("k_ou_update")
    if cfg.geom != 2 and cfg.solverdust == 0 and cfg.ndust > 0:
        parts.append("k_flux_strip_mixed (gas and dust strips)")
    else:
        parts.append("k_flux_strip (gas, side stream) + k_flux_strip (dust)")
    if cfg.flags & K.FLAG_FARGO:
        parts.append("k_fargo")
    parts.append("k_finalize_mixed")
    return "per step: " + ", ".join(parts)


def config_leg(args, name, device, mixed_steps=5, fp64_steps=2, warm=6):
    """Mixed and FP64 timing of one of the two larger configurations, their L1 distance after the
    same number of steps from the same state, and the charging iterations of the last step.  Both
    precisions take `warm` untimed steps first: the first steps from the initial state are a
    transient (the cold charging Newton of step 1, a spike of growth sub-steps around step 4 on the
    polar disk), the timed steps the steady state."""
    from shark_gb300 import config as K
    from shark_gb300.solver import Shark
    out = {}
    ctx = {}
    for prec, ns in ((K.PREC_MIXED, mixed_steps), (K.PREC_FP64, fp64_steps)):
        cfg, u0 = workload(args, prec, name)
        cfg.device = device
        g = Shark(cfg)
        g.upload(u0)
        for _ in range(warm):
            g.solve()
        ms = g.timed_run(ns)
        kt = g.kernel_times(2)
        st = g.sync()
        zs = cfg.nx * cfg.ny * (cfg.ndust + 1)
        _, nonconv, tot = g.charge_stats()
        out["mixed" if prec == K.PREC_MIXED else "fp64"] = {
            "value": zs * ns / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / ns, "steps": ns,
            "kernel_ms": {"charge_forcing": kt[0], "flux_update": kt[1], "drag_growth_dt": kt[2], "step": kt[3]},
            "status": st, "charging_nonconverged_cells": nonconv, "charging_iterations_per_cell": tot / (cfg.nx * cfg.ny),
            "status_note": "bits: 1 NaN, 2 negative density, 4 dt underflow, 8 a charging Newton ended above its "
                           "tolerance (the polar disk's outer cells stall at psi0 in the reference's loop too), "
                           "16 growth sub-step cap"}
        ctx[prec] = (cfg, g)
        del u0
    (cm, gm), (cd, gd) = ctx[K.PREC_MIXED], ctx[K.PREC_FP64]
    nm = warm + mixed_steps + 2
    gd.run_steps(nm - (warm + fp64_steps + 2))
    gd.sync()
    out["l1_mixed_vs_fp64"] = rel_l1_max(cm, gm.download(), gd.download())
    out["l1_note"] = f"max relative L1 over the {cm.nvar} conserved fields after {nm} steps from the same state"
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    if name == "turb" and cm.ndust == 32:
        out["mixed"]["alu_roofline"] = alu_roofline_turb(cm, out["mixed"]["kernel_ms"])
    out["workload"] = describe(argparse.Namespace(workload=name), cm)
    gm.close()
    gd.close()
    return out


def alu_roofline_turb(cfg, kernel_ms):
    """Arithmetic roofline of the driven box's two compute-bound kernels: the per-cell FLOP counts
    of an ncu capture of the same kernels (profiles/alu_roofline_turb.txt, 512^2 cells) times this
    run's cells, over this run's event-timed milliseconds.  The growth sub-step and Newton
    iteration counts depend on the state, so the rates are estimates at the captured counts."""
    path = os.path.join(ROOT, "profiles", "alu_roofline_turb.txt")
    if not os.path.exists(path):
        return None
    vals = {}
    with open(path) as f:
        for line in f:
            if ":" in line and not line.startswith("#"):
                k, v = line.split(":", 1)
                vals[k.strip()] = float(v)
    cells = cfg.nx * cfg.ny
    growth_s = kernel_ms["drag_growth_dt"] * 1e-3
    charge_s = kernel_ms["charge_forcing"] * 1e-3
    fp32_peak, fp64_peak = vals["fp32_peak_tflops_at_2070mhz"], vals["fp64_peak_tflops_at_2070mhz"]
    g32 = vals["k_finalize_mixed_growth_fp32_flop_per_cell"] * cells / growth_s / 1e12
    c64 = vals["k_charge_fp64_flop_per_cell"] * cells / charge_s / 1e12
    return {"growth": {"kernel": "k_finalize_mixed (drag + growth + CFL)", "bound": "fp32 issue latency",
                       "achieved": g32, "peak": fp32_peak, "unit": "TFLOP/s", "frac": g32 / fp32_peak},
            "charging": {"kernel": "k_charge (+ OU forcing update)", "bound": "fp64 pipe",
                         "achieved": c64, "peak": fp64_peak, "unit": "TFLOP/s", "frac": c64 / fp64_peak},
            "source": "per-cell FLOPs from profiles/alu_roofline_turb.txt (ncu, 512^2), nominal peaks at 2070 MHz"}


def noisy_box(cfg, u, seed, amp=0.5):
    """Lognormal density structure on a dusty box (gas and each species independently, momenta
    scaled alike): states spanning the charging network's input range."""
    from shark_gb300 import setups
    rng = np.random.default_rng(seed)
    g = u.reshape(cfg.nvar, -1)
    f = np.exp(amp * rng.standard_normal(cfg.ncells))
    g[:5] *= f
    N = cfg.ndust
    for k in range(N):
        fk = f * np.exp(amp * rng.standard_normal(cfg.ncells))
        for c in range(4):
            g[5 + c * N + k] *= fk
    setups.periodic_boundaries(cfg, u)
    return u


def mlp_leg(device):
    """Train the charging network on the GPU (forward/backward kernels, Adam) on (state, converged
    psi) pairs that the charging solver produces on dusty boxes over a range of densities, then
    charge the 2048^2, 32-species box from a cold start with and without the network's seed."""
    from shark_gb300 import config as K, setups
    from shark_gb300.solver import Shark
    t0 = time.perf_counter()
    cfg, u0 = setups.dusty_turb(n=128, ndust=32, charging=True)
    cfg.device = device
    n = 0
    with Shark(cfg) as g:
        for f in (0.03, 0.1, 0.3, 1.0, 3.0, 10.0, 30.0):
            for seed in (11, 12):
                c, u = setups.dusty_turb(n=128, ndust=32, charging=True)
                g.upload(noisy_box(c, u, seed) * f)
                n = g.mlp_collect(capacity=1 << 20)
        loss1 = g.mlp_train(3000, batch=2048, lr=2e-3, seed=7)
        loss2 = g.mlp_train(3000, batch=2048, lr=3e-4, seed=8)
        blob = g.mlp_save()
    t_train = time.perf_counter() - t0
    res = {}
    for mode in ("cold", "seeded"):
        c, u = setups.dusty_turb(n=2048, ndust=32, forcing=True, charging=True, growth=True, precision=K.PREC_MIXED)
        u = noisy_box(c, u, 99)                      # held out: a seed the training did not see
        c.device = device
        if mode == "seeded":
            c.chg_mode |= K.CHARGE_MLP_SEED
        with Shark(c) as g:
            if mode == "seeded":
                g.mlp_load(blob)
            g.upload(u)
            g.charge_reset()
            g.charge()
            hist, nonconv, tot = g.charge_stats()
            ch = g.download_charge()
        res[mode] = (tot, nonconv, ch["psi"], ch["iters"])
        del u
    cells = 2048 * 2048
    conv = res["cold"][3] < c.chg_nitermax          # cells the cold start converges
    dpsi = float(np.max(np.abs(res["seeded"][2][conv] - res["cold"][2][conv]) / np.abs(res["cold"][2][conv])))
    return {"training_pairs": int(n), "train_seconds": t_train,
            "loss_first_50": float(np.mean(loss1[:50])), "loss_last_200": float(np.mean(loss2[-200:])),
            "newton_iterations_per_cell_cold": res["cold"][0] / cells,
            "newton_iterations_per_cell_seeded": res["seeded"][0] / cells,
            "iteration_ratio": res["cold"][0] / max(res["seeded"][0], 1),
            "nonconverged_cells_cold": int(res["cold"][1]), "nonconverged_cells_seeded": int(res["seeded"][1]),
            "max_rel_psi_difference": dpsi,
            "note": "2048^2 dusty box, 32 species, lognormal density structure (held-out seed), mixed precision, "
                    "cold start from psi0 vs the network's seed, residual tolerance chg_eps in both; training on "
                    "128^2 boxes at 7 density factors x 2 seeds"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--repeats", type=int, default=5, help="timed runs of --steps steps; the median is reported")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--ndust", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true", help="skip the disk/turbulence and network legs")
    ap.add_argument("--workload", default="si", choices=["si", "disk", "turb"])
    args = ap.parse_args()
    if args.workload != "si" and "--steps" not in sys.argv:
        args.steps = 5
    args.n_given = "--n" in sys.argv
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
