"""Build the in-tree native libraries of the GB300 hot path.

  libemmi_gpu.so   CUDA kernels + batched solver + drop-in C ABI (nvcc, sm_103a)
  libemmi_host.so  host front end in C (gcc): parameters, grids, homogenization,
                   l-BFGS / line search / regularization of the inversion

Everything is compiled in-tree next to this file (no pip install), in
parallel, with one -gencode for sm_103a.  nvcc cross-compiles without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

GPU_SOURCES = ["emmi_kernels.cu", "emmi_solver.cu", "emmi_survey.cu", "emmi_dropin.cu",
               "emmi_krylov.cu", "emmi_learned.cu", "emmi_noalloc.cu", "emmi_frontend.cu",
               "emmi_stencil.cu"]
HOST_SOURCES = ["emmi_host.c", "emmi_fwi.c"]
GPU_LIB = os.path.join(HERE, "libemmi_gpu.so")
HOST_LIB = os.path.join(HERE, "libemmi_host.so")
MAIN_SOURCES = ["emmi_main.c", "emmi_params.c", "emmi_host.c", "emmi_fwi.c"]
MAIN_BIN = os.path.join(HERE, "emmi_main")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE,
              "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libemmi_gpu.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> None:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    objs, jobs = [], []
    for src in [f for f in GPU_SOURCES if os.path.exists(os.path.join(CSRC, f))]:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            # the survey kernels reproduce the reference's rounding: no FMA
            extra = ["-fmad=false"] if src == "emmi_survey.cu" else []
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
    if force or jobs or _stale(GPU_LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", GPU_LIB] + objs + ["-lcudart"])
    hsrc = [os.path.join(CSRC, f) for f in HOST_SOURCES if os.path.exists(os.path.join(CSRC, f))]
    if hsrc and (force or _stale(HOST_LIB, hsrc + headers)):
        _run(["gcc", "-O2", "-fPIC", "-std=gnu99", "-ffp-contract=off", "-shared", "-I" + INCLUDE,
              "-o", HOST_LIB]
             + hsrc + ["-lm"])
    # the reference's modelling command line on the GPU path
    msrc = [os.path.join(CSRC, f) for f in MAIN_SOURCES]
    if force or _stale(MAIN_BIN, msrc + headers + [GPU_LIB]):
        _run(["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-I" + INCLUDE, "-o", MAIN_BIN]
             + msrc
             + ["-L" + HERE, "-lemmi_gpu", "-Wl,-rpath,$ORIGIN", "-lm"])


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print("built", GPU_LIB, HOST_LIB)
