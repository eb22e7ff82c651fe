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
UNIT = "zone-species updates/s"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def workload(args, precision):
    from shark_gb300 import setups
    cfg, u0 = setups.si(n=args.n, ndust=args.ndust, precision=precision, noise=1e-3, seed=1)
    return cfg, u0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while the timed region runs."""
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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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
        "config": {"workload": f"SI shearing box {args.n}x{args.n}, {args.ndust} dust species",
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
    if rank == 0 or world == 1:
        gbuild.build()
    if world > 1:
        torch.distributed.barrier()
    gbuild.build()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    zs_step = args.n * args.n * (args.ndust + 1)

    # ---- mixed path, state resident -----------------------------------------------------------
    cfg_m, u0 = workload(args, K.PREC_MIXED)
    cfg_m.device = local_rank
    gm = Shark(cfg_m)
    gm.upload(u0)
    for _ in range(args.warmup):
        gm.solve()
    gm.sync()
    barrier()
    with ClockSampler(local_rank) as clocks:
        ms = gm.timed_run(args.steps)
    barrier()
    ms_all = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(ms_all, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(ms_all.item())
    value = zs_step * args.steps * world / (ms_max * 1e-3)
    st = gm.sync()

    # per-kernel times (separate pass, events around every launch)
    kt = gm.kernel_times(max(5, min(args.steps, 20)))
    u_mixed = gm.download()
    steps_done_m = args.warmup + args.steps + max(5, min(args.steps, 20))

    # ---- FP64 path on the same workload ----------------------------------------------------
    cfg_d, _ = workload(args, K.PREC_FP64)
    cfg_d.device = local_rank
    gd = Shark(cfg_d)
    gd.upload(u0)
    for _ in range(args.warmup):
        gd.solve()
    ms_d = gd.timed_run(args.steps)
    gd.run_steps(steps_done_m - args.warmup - args.steps)
    u_fp64 = gd.download()
    value_fp64 = zs_step * args.steps / (ms_d * 1e-3)
    l1 = rel_l1_max(cfg_m, u_mixed, u_fp64)
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
    el_all = torch.tensor([el], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(el_all, op=torch.distributed.ReduceOp.MAX)
    e2e_value = zs_step * e2e_steps * world / float(el_all.item())
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
    alg_bytes_k1 = 2 * 4 * nvar * args.n * args.n            # read + write each conserved value once
    k1_s = kt[1] * 1e-3
    achieved = alg_bytes_k1 / k1_s / 1e9
    alg_bytes_k2 = 4 * (7 * (args.ndust + 1) + args.ndust) * args.n * args.n
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "k_flux_traffic.txt")
    if os.path.exists(tfile) and args.n == 1024 and args.ndust == 8:
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
        "config": {"workload": f"SI shearing box {args.n}x{args.n} active cells, {args.ndust} dust species, "
                               f"mixed precision", "zone_species_per_step": zs_step,
                   "parallelism": "replicas only" if world > 1 else "single GPU",
                   "l2": "state (2 x 160 MB ping-pong, FP32) larger than the 129 MB L2; no flush"},
        "fp64": {"value": value_fp64, "unit": UNIT, "ms_per_step": ms_d / args.steps,
                 "mixed_over_fp64": value / world / value_fp64,
                 "l1_mixed_vs_fp64": l1, "l1_note": f"max relative L1 over the {nvar} conserved fields after "
                                                    f"{steps_done_m} steps from the same state",
                 "kernel_ms": {"pre_flux": kt_d[0], "flux_update": kt_d[1], "drag_dt_ghosts": kt_d[2], "step": kt_d[3]}},
        "kernel_ms": {"pre_flux": kt[0], "flux_update": kt[1], "drag_dt_ghosts": kt[2], "step": kt[3]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "kernel": "k_flux (K1 fused flux/update)",
                     "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes_k1,
                     "drag_kernel_achieved_gbs": alg_bytes_k2 / (kt[2] * 1e-3) / 1e9},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps,
                "note": "per step: shark_gpu_upload from pinned host FP64 u_prim, shark_gpu_step, shark_gpu_download",
                "resident_value": zs_step * e2e_steps / el_res,
                "resident_note": "state kept on the device, per step shark_gpu_step with its 12-byte dt/status readback"},
        "cpu_baseline": cpu,
        "gpu_launches": 4 * args.steps,
        "gpu_launches_note": "per step: k_reset_dt, k_flux_strip (gas, side stream), k_flux_strip (dust), k_finalize",
        "status": st,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--ndust", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
