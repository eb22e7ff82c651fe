"""Builds libshark_gpu.so in-tree with nvcc for sm_103a only.

Three translation units compiled in parallel:
  kernels_f64.cu  -- FP64 step kernels, --fmad=false (round-for-round equal to the CPU oracle)
  kernels_f32.cu  -- FP32 (mixed-precision) step kernels, FMA contraction and approximate
                     FP32 division on (the mixed path is held to 1e-5 L1 against FP64)
  shark_gpu.cu    -- host side of the C ABI (include/shark_gpu.h)
  noalloc.cu      -- shark_gpu_totals_noalloc (no allocations; fixed device scratch array)
  mlp.cu          -- the charging network (tcgen05 BF16 GEMMs, TMEM accumulators, Adam)
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libshark_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr",
          "-I" + os.path.join(HERE, "..", "include")]
UNITS = [
    ("kernels_f64.cu", ["--fmad=false"]),
    ("kernels_f32.cu", ["--fmad=true", "-prec-div=false"]),
    ("shark_gpu.cu", []),
    ("noalloc.cu", []),
    ("mlp.cu", []),
]


def nvcc():
    for cand in [os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")]:
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "shark_gpu.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def compile_unit(unit):
        src, flags = unit
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nv, *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    extra = [a for a in sys.argv[1:] if a.startswith("-")]
    print(build(force=True, verbose=True, extra=extra))
