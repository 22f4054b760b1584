"""Build recipe of libraytracer_gb300.so (sm_103a only).

Each .cu translation unit is compiled by nvcc in parallel with
-gencode arch=compute_103a,code=sm_103a, then linked into one shared
library next to this file; the C++ host driver (host/rt_main.cpp) is then
compiled with g++ against it.  The binary64 parity arithmetic uses explicit
round-to-nearest intrinsics, so no global -fmad switch is needed.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libraytracer_gb300.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["rt_api.cu", "rt_kernels.cu", "rt_persist.cu", "rt_persist_w2.cu", "rt_persist_fused.cu", "rt_noalloc.cu",
           "rt_forcing.cu", "rt_split.cu", "rt_fast.cu", "rt_probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-I" + CSRC, "-I" + INC]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libraytracer_gb300.so")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INC, "rt_gb300.h")]
    return max(os.path.getmtime(f) for f in files)


HOST_SRC = os.path.join(HERE, "host", "rt_main.cpp")
HOST_BIN = os.path.join(HERE, "host", "rt_main")


def build_host(force=False):
    """The C++ driver over the C ABI (host/rt_main.cpp, g++), linked
    against the library next to it.  No fused multiply-add: its host grid
    must equal the reference's bit for bit."""
    deps = max(os.path.getmtime(f) for f in (HOST_SRC, LIB, os.path.join(INC, "rt_gb300.h")))
    if not force and os.path.exists(HOST_BIN) and os.path.getmtime(HOST_BIN) >= deps:
        return HOST_BIN
    tmp = HOST_BIN + ".tmp"
    cmd = ["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-Wall", HOST_SRC, "-I" + INC, "-L" + HERE,
           "-lraytracer_gb300", "-Wl,-rpath," + HERE, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for the host driver:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, HOST_BIN)
    return HOST_BIN


def build(force=False, verbose=False):
    lib = build_library(force, verbose)
    build_host(force)
    return lib


def build_library(force=False, verbose=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [exe] + ARCH + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        return obj, r.stdout + r.stderr

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose:
        for _, log in results:
            sys.stdout.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
