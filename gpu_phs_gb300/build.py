"""Builds libgpuphs.so in-tree (gpu_phs_gb300/libgpuphs.so) for sm_103a.

Device code is compiled by nvcc for exactly one target
(-gencode arch=compute_103a,code=sm_103a); host code by g++ with -ffp-contract=off so
that the mapping constants equal the reference CPU path's on every host (x86-64 and
aarch64).  Translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgpuphs.so")
# the bounds-checked build (-DPHS_CHECKED, csrc/phs_check.h): a second library for tests
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(HERE, "libgpuphs_checked.so")
ROOT = os.path.dirname(HERE)

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["phs_kernels.cu", "phs_kernels_ff.cu", "phs_adjoint.cu", "phs_inverse.cu",
              "phs_grid.cu"]
# The inverse map mirrors the operation order of the reference's algorithm (as the oracle
# restates it) without contraction: its results then differ from the oracle's only by the
# ulps of the transcendental functions, although x(p) is ill-conditioned near the poles.
CU_FLAGS = {"phs_inverse.cu": ["-fmad=false"]}
CPP_SOURCES = ["phs_compile.cpp", "phs_api.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _jobs(build_dir, lib, defines, force):
    """Compile commands of one library (those whose object is stale) and its objects."""
    os.makedirs(build_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc_dir = os.path.join(ROOT, "include")
    headers += [os.path.join(inc_dir, f) for f in os.listdir(inc_dir) if f.endswith(".h")]
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", os.path.join(CUDA_HOME, "include")]
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(build_dir, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v", *defines, *CU_FLAGS.get(src, []), *inc, "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(build_dir, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-Wall", "-Wno-unused-function", *defines, *inc, "-c", s, "-o", o])
    return jobs, objs


def _link(lib, objs):
    tmp = lib + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread", "-ldl",
          "-Xlinker", "-rpath", "-Xlinker", os.path.join(CUDA_HOME, "lib64")])
    shutil.move(tmp, lib)


def build(verbose: bool = False, force: bool = False, checked: bool = True) -> str:
    """Compile and link libgpuphs.so and (checked=True) libgpuphs_checked.so, every
    translation unit of both in parallel; returns the library path.  Raises RuntimeError
    on failure."""
    libs = [(BUILD, LIB, [])]
    if checked:
        libs.append((BUILD_CHECKED, LIB_CHECKED, ["-DPHS_CHECKED"]))
    plans = [(lib, *_jobs(d, lib, defs, force)) for d, lib, defs in libs]
    all_jobs = [j for _, jobs, _ in plans for j in jobs]
    with ThreadPoolExecutor(max_workers=max(1, len(all_jobs))) as ex:
        logs = list(ex.map(_run, all_jobs))
    if verbose:
        for lg in logs:
            sys.stdout.write(lg)
    for lib, jobs, objs in plans:
        if force or jobs or _stale(lib, objs):
            _link(lib, objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
