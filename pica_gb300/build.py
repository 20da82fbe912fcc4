"""Build the pica_gb300 CUDA library in-tree (pica_gb300/_build/libpica_gb300.so).

One nvcc invocation per translation unit, run in parallel, sm_103a only.
The FP64 translation units are compiled with --fmad=false so that double
arithmetic rounds exactly as pica's C++ does; the FP32 push unit too, so that its
roundings are the ones its source writes out.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpica_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-I", os.path.join(HERE, "..", "include")]
UNITS = [
    ("pica_api.cu", ["-Xcompiler", "-ffp-contract=off"]),
    ("push_fp64.cu", ["--fmad=false"]),
    # No implicit contraction: ptxas would otherwise fuse a multiply and an add
    # differently in different instantiations of the same code (launch bounds,
    # register pressure), and launch variants and the batching form would stop
    # rounding alike.  The FP32 push writes its fused multiply-adds out instead.
    ("push_fp32.cu", ["--fmad=false"]),
    ("grid_kernels.cu", ["--fmad=false"]),
    ("noalloc.cu", ["--fmad=false"]),
    ("plasma_gen.cu", ["--fmad=false"]),
    ("domain_kernels.cu", ["--fmad=false"]),
    ("flat.cu", ["--fmad=false"]),
]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(HERE, "..", "include", "pica_gb300.h")
    return os.path.getmtime(hdr) > t


def build(force=False, verbose=False, ptxas_info=False):
    """Compile every CUDA translation unit for sm_103a and link the shared library."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(unit):
        src, flags = unit
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [NVCC] + ARCH + COMMON + flags + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose or ptxas_info:
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
