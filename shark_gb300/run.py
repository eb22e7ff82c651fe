"""Run a few steps of one of the built setups on the GPU and report the status word and the last dt.

    python -m shark_gb300.run si --n 1024 --ndust 8 --steps 3 --precision mixed
    python -m shark_gb300.run turb --n 512 --ndust 32 --forcing --charging --growth --steps 3
    python -m shark_gb300.run disk --nr 512 --nphi 1024 --ndust 16 --growth --steps 3

The same setups the tests and the benchmark build (shark_gb300.setups); useful for a quick check
of a configuration and as the command a profiler wraps.  Exits non-zero when the step status word
reports a numerical failure (a charging Newton cap, which the polar disk's outer cells reach in the
reference's loop too, is reported but not a failure).
"""
import argparse
import json
import sys

from . import config as K, setups
from .solver import Shark


def build_setup(a):
    prec = K.PREC_MIXED if a.precision == "mixed" else K.PREC_FP64
    if a.setup == "si":
        return setups.si(n=a.n, ndust=a.ndust, precision=prec, noise=1e-3, seed=1)
    if a.setup == "turb":
        return setups.dusty_turb(n=a.n, ndust=a.ndust, forcing=a.forcing, charging=a.charging, growth=a.growth,
                                 precision=prec)
    if a.setup == "disk":
        return setups.disk_polar_au(nr=a.nr, nphi=a.nphi, ndust=a.ndust, growth=a.growth, precision=prec)
    if a.setup == "dustywave":
        return setups.dustywave(nx=a.n, ndust=a.ndust, precision=prec)
    return setups.sod(nx=a.n, precision=prec)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("setup", choices=["si", "turb", "disk", "dustywave", "sod"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--nr", type=int, default=512)
    ap.add_argument("--nphi", type=int, default=1024)
    ap.add_argument("--ndust", type=int, default=8)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--forcing", action="store_true")
    ap.add_argument("--charging", action="store_true")
    ap.add_argument("--growth", action="store_true")
    a = ap.parse_args(argv)
    cfg, u0 = build_setup(a)
    with Shark(cfg) as g:
        g.upload(u0)
        dts = [g.solve() for _ in range(a.steps)]
        st = g.sync()
    print(json.dumps({"setup": a.setup, "steps": a.steps, "dt_last": dts[-1] if dts else None, "status": st}))
    return 0 if st & ~K.STATUS_NEWTON == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
