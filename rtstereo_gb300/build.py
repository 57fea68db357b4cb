"""Build the in-tree native library ``rtstereo_gb300/librtstereo_gb300.so``.

CUDA translation units are compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) with ``-fmad=false`` (the plain
form's float arithmetic is the reference's, with no fused multiply-add; kernels
that want FMA call it explicitly) and IEEE division and square root (nvcc's
defaults; ``--use_fast_math`` is never used).  Host C++ is compiled by g++ with
``-ffp-contract=off`` for the same reason.  The CUDA runtime is linked
statically, so the library needs only the driver at run time.

Objects go to ``rtstereo_gb300/_build``; a unit is recompiled when it or any
header is newer than its object.  Units compile in parallel.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "librtstereo_gb300.so")
DRIVER_SRC = os.path.join(PKG, "driver", "rts_stereo.cpp")
DRIVER = os.path.join(PKG, "rts_stereo")  # headless equivalent of the reference driver
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(src: str, obj: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(h) > t for h in headers)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False, jobs: int | None = None) -> str:
    """Compile and link the library; returns its path."""
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    nvcc_flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", CSRC]
    if ptxas_info:
        nvcc_flags += ["-Xptxas", "-v"]
    gxx_flags = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                 "-I", os.path.join(cuda, "include"), "-I", CSRC]
    jobs_list = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        if ptxas_info or _stale(src, obj, headers):
            jobs_list.append([nvcc] + nvcc_flags + ["-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        if _stale(src, obj, headers):
            jobs_list.append(["g++"] + gxx_flags + ["-c", src, "-o", obj])
    logs = []
    if jobs_list:
        with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs_list):
                logs.append(out)
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in cu + cpp]
    if jobs_list or not os.path.exists(LIB):
        libdir = os.path.join(cuda, "lib64")
        if not os.path.isdir(libdir):
            libdir = os.path.join(cuda, "lib")
        tmp = LIB + ".tmp"
        _run(["g++", "-shared", "-o", tmp] + objs +
             ["-L", libdir, "-lcudart_static", "-ldl", "-lrt", "-lpthread"])
        os.replace(tmp, LIB)
    if _stale(DRIVER_SRC, DRIVER, headers + [LIB]):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, DRIVER_SRC, "-o", DRIVER,
              "-L", PKG, "-lrtstereo_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        sys.stdout.write("".join(logs))
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
