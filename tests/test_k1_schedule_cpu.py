"""The mixed path's flux-kernel schedule (shark_gb300/csrc/k1_schedule.h) on the host: for the
benchmark boxes, small and ragged grids, one to 64 species, isothermal and adiabatic gas, and
several SM counts, every row of every column block of the gas and of each dust species is marched
by exactly one piece of one warp, and a persistent schedule fits in one wave of warps
(tests/k1_schedule_check.cpp, compiled here with the host compiler against the header the kernel
uses)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("k1") / "k1_schedule_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "k1_schedule_check.cpp")], check=True)
    return exe


def _run(exe, cases):
    args = [str(v) for c in cases for v in c]
    r = subprocess.run([exe, *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.splitlines()


def test_benchmark_boxes(checker):
    out = _run(checker, [(1024, 1024, 8, 2432, 1), (2048, 2048, 32, 2432, 1), (512, 1024, 16, 2432, 1),
                         (1024, 1024, 32, 2432, 1), (1024, 1088, 32, 2432, 1), (1024, 1024, 4, 2432, 0)])
    # the SI box: one persistent wave, 14 dust and 23 gas pieces per column block
    assert "warps 414 + 2016" in out[0] and "gas P 1 m 23, dust P 1 m 14" in out[0], out[0]


def test_small_and_ragged_grids(checker):
    _run(checker, [(64, 64, 4, 2432, 1), (70, 45, 3, 2432, 0), (16, 16, 1, 2432, 1), (7, 5, 64, 2432, 1),
                   (61, 17, 2, 8, 1), (121, 3, 5, 2432, 0), (60, 60, 1, 2, 1)])


def test_random_grids_and_sm_counts(checker):
    rng = np.random.default_rng(7)
    cases = []
    for _ in range(60):
        nx, ny = int(rng.integers(4, 3000)), int(rng.integers(3, 3000))
        nd = int(rng.integers(1, 65))
        warps = int(rng.choice([2, 64, 608, 1216, 1824, 2432, 4864]))
        cases.append((nx, ny, nd, warps, int(rng.integers(0, 2))))
    assert len(_run(checker, cases)) == len(cases)
