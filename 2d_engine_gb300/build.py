"""Build recipe of the in-tree CUDA library (libgb2d.so) for sm_103a.

Compiles the csrc/ translation units in parallel with nvcc and links them into
2d_engine_gb300/_build/libgb2d.so (static CUDA runtime, C ABI of include/gb2d.h),
then the headless .sim driver 2d_engine_gb300/_build/gb2d_sim (driver/, C++).
gb2d_exact.cu and gb2d_flow.cu are built with --fmad=false: their FP64 kernels
must round every multiply and add separately, exactly as the reference's CPU
arithmetic.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgb2d.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "gb2d_exact.cu": ["--fmad=false"],
    "gb2d_flow.cu": ["--fmad=false"],
    "gb2d_jump.cu": ["--fmad=false"],
    "gb2d_solver.cu": [],
    "gb2d_api.cu": [],
    "gb2d_noalloc.cu": [],
    "gb2d_adjoint.cu": [],
    "gb2d_batch.cu": [],
    "gb2d_peaks.cu": [],
}


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(ROOT, "include", "gb2d.h"))
    base = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-O2",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if ptxas_info:
        base += ["-Xptxas", "-v"]

    def compile_unit(item):
        src, extra = item
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        if not ptxas_info and not _stale(obj, [path] + headers):
            return obj, ""
        cmd = base + extra + ["-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(compile_unit, UNITS.items()))
    objs = [o for o, _ in results]
    if verbose or ptxas_info:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    build_driver()
    return LIB


DRIVER_DIR = os.path.join(HERE, "driver")
SIM = os.path.join(OUT, "gb2d_sim")


def build_driver():
    """The headless .sim driver (C++, host compiler only), linked to libgb2d.so."""
    src = os.path.join(DRIVER_DIR, "gb2d_sim.cpp")
    deps = [src, os.path.join(DRIVER_DIR, "script.hpp"), os.path.join(ROOT, "include", "gb2d.h"), LIB]
    if not _stale(SIM, deps):
        return SIM
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for the .sim driver")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", DRIVER_DIR, src, "-o", SIM,
           "-L", OUT, "-lgb2d", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gb2d_sim build failed:\n{r.stderr}")
    return SIM


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
