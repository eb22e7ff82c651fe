"""Copies the reference's own golden data for this path into tests/golden/ (run once with the path
of a reference checkout as its only argument; the outputs are committed).

Sources (reference test suite):
  test/test-suite/Sod-tube/solution.dat           exact Sod solution, t=0.245, gamma=1.4, 1024 cells
                                                  columns: i, x, u, rho, P, e
  test/test-suite/DUSTYWAVE/dustywave-K{50,100,1000}.dat
                                                  single-species dusty-wave profiles (128 points)
                                                  columns: x, vgas, vdust, rhogas, rhodust
Their namelists (sod.nml, wave{50,100,1000}.nml) fix the run parameters used by the tests:
  Sod: CFL 0.8, tend 0.245, gamma 1.4, slope_type 3.
  Dusty wave: CFL 0.8, tend 4.5, gamma 1.6666667, slope_type 2, cs=1, rho=1, eps=1, delta=1e-4.
"""
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python make_golden.py <path of the reference checkout>")
REF = sys.argv[1]
HERE = os.path.dirname(os.path.abspath(__file__))

FILES = {
    "test/test-suite/Sod-tube/solution.dat": "sod_exact_t0.245_n1024.dat",
    "test/test-suite/DUSTYWAVE/dustywave-K50.dat": "dustywave_K50.dat",
    "test/test-suite/DUSTYWAVE/dustywave-K100.dat": "dustywave_K100.dat",
    "test/test-suite/DUSTYWAVE/dustywave-K1000.dat": "dustywave_K1000.dat",
}

for src, dst in FILES.items():
    with open(os.path.join(REF, src)) as f:
        text = f.read()
    with open(os.path.join(HERE, dst), "w") as f:
        f.write(text)
    print(dst, len(text.splitlines()), "lines")
