"""Build of libeddy_gpu.so (sm_103a kernels + C ABI) and the eddy CLI.

Everything is compiled in-tree with nvcc/g++ into eddy-gpu_gb300/lib/ and
eddy-gpu_gb300/bin/ (git-ignored).  One -gencode (sm_103a), translation
units compiled in parallel.
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
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
BINDIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIBDIR, "libeddy_gpu.so")
CLI = os.path.join(BINDIR, "eddy")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                  "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")]
CU = ["eddy_kernels.cu", "eddy_mma.cu", "eddy_api.cu", "eddy_noalloc.cu"]
CPP = ["eddy_host.cpp", "eddy_writers.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "eddy_gpu.h"))
    jobs = []
    objs = []
    for f in CU + CPP:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            if f.endswith(".cu"):
                jobs.append([nvcc] + NVFLAGS + ["-c", src, "-o", obj])
            else:
                jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off",
                             "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    cli_src = os.path.join(CSRC, "eddy_cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB] + headers):
        _run(["g++", "-O2", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "include"), cli_src,
              "-o", CLI, "-L", LIBDIR, "-leddy_gpu", "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
