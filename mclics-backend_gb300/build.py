"""Builds the GB300 engine in-tree: _build/libmcx.so (the C ABI of
include/mcx.h) and _build/mc_sim_gb300 (the command-line drop-in).

sm_103a only; translation units compile in parallel.  Run as a script or call
build()."""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.environ.get("MCX_BUILD_DIR", os.path.join(HERE, "_build"))
EXTRA = os.environ.get("MCX_NVCC_FLAGS", "").split()
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOSTFLAGS = ["-fPIC", "-ffp-contract=off", "-O3", "-fno-strict-aliasing"]
CUDA_TU = ["mcx_kernels.cu", "mcx_march.cu", "mcx_march_odd.cu", "mcx_amarch.cu", "mcx_qmarch.cu", "mcx_pmarch.cu", "mcx_lmarch.cu", "mcx_learned.cu", "mcx_train.cu", "mcx_engine.cu", "mcx_noalloc.cu", "mcx_tcmlp.cu"]
HOST_TU = ["mcx_host.cpp", "mcx_sim.cpp"]
LIB = os.path.join(OUT, "libmcx.so")
CLI = os.path.join(OUT, "mc_sim_gb300")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "mcx.h"))
    jobs = []
    objs = []
    for tu in CUDA_TU + HOST_TU:
        src = os.path.join(SRC, tu)
        obj = os.path.join(OUT, tu + ".o")
        objs.append(obj)
        if not force and _newer(obj, [src] + headers):
            continue
        if tu.endswith(".cu"):
            cmd = [NVCC, *ARCH, *EXTRA, "-O3", "-lineinfo", "-std=c++17", "-Xptxas", "-v", "-Xcompiler",
                   ",".join(HOSTFLAGS), "-c", src, "-o", obj]
        else:
            cmd = ["g++", "-std=c++17", *HOSTFLAGS, "-I", os.environ.get("CUDA_INC", "/usr/local/cuda/include"),
                   "-c", src, "-o", obj]
        jobs.append(cmd)
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or not _newer(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    main_src = os.path.join(SRC, "mcx_sim_main.cpp")
    if force or not _newer(CLI, [LIB, main_src]):
        _run(["g++", "-std=c++17", "-O2", main_src, "-o", CLI, "-L", OUT, "-lmcx", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
