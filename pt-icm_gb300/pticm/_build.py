"""Build of the in-tree native library (libpticm_gb300.so) and the pt_icm CLI.

nvcc compiles every translation unit for sm_103a only
(-gencode arch=compute_103a,code=sm_103a) in parallel, then links one shared
library next to this file.  No CMake; a minute or less on a 16-core host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                       # pt-icm_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
HOSTSRC = os.path.join(ROOT, "host")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libpticm_gb300.so")
CLI = os.path.join(ROOT, "bin", "pt_icm")
SHIM = os.path.join(PKG, "libpticm_shim.a")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
           "--expt-relaxed-constexpr"] + ARCH
INCS = ["-I", os.path.join(REPO, "include"), "-I", CSRC]

LIB_SOURCES = ["pt_engine.cu", "runtime.cu", "problem_host.cc", "noalloc.cu", "replica.cu", "smem_rate.cu", "mhist.cu", "mhist_host.cc", "tc_gemm.cu", "mlp.cu", "batch.cu", "surrogate.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= _newest_input(src):
        return obj
    cmd = [nvcc()] + NVFLAGS + INCS + ["-c", src, "-o", obj]
    if src.endswith(".cc"):
        cmd = [nvcc(), "-x", "cu"] + NVFLAGS + INCS + ["-c", src, "-o", obj]
    subprocess.check_call(cmd)
    return obj


def _newest_input(src: str) -> float:
    t = os.path.getmtime(src)
    for d in (CSRC, os.path.join(REPO, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hh")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def build(verbose: bool = False) -> str:
    """Compile and link libpticm_gb300.so (and the pt_icm CLI when present)."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in LIB_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        subprocess.check_call([nvcc(), "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    build_shim()
    cli_src = os.path.join(HOSTSRC, "pt_icm_main.cc")
    if os.path.exists(cli_src):
        os.makedirs(os.path.dirname(CLI), exist_ok=True)
        newest = max(os.path.getmtime(x) for x in [cli_src, SHIM, LIB])
        if not os.path.exists(CLI) or os.path.getmtime(CLI) < newest:
            subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                                   "-I", HOSTSRC, "-o", CLI, cli_src, SHIM,
                                   "-L", PKG, "-lpticm_gb300", "-Wl,-rpath,$ORIGIN/../pticm"])
    return LIB


def build_shim() -> str:
    """The reference's C++ interface (host/*.cc but the CLI's main) as a
    static archive, libpticm_shim.a next to the native library: link it and
    libpticm_gb300.so to build code written against pticm_gb300.hh."""
    srcs = [os.path.join(HOSTSRC, f) for f in sorted(os.listdir(HOSTSRC))
            if f.endswith(".cc") and f != "pt_icm_main.cc"]
    hdrs = [os.path.join(HOSTSRC, f) for f in os.listdir(HOSTSRC) if f.endswith(".hh")]
    hdrs.append(os.path.join(REPO, "include", "pticm.h"))
    newest = max(os.path.getmtime(x) for x in srcs + hdrs)
    if os.path.exists(SHIM) and os.path.getmtime(SHIM) >= newest:
        return SHIM

    def one(src):
        obj = os.path.join(BUILD, "shim_" + os.path.basename(src) + ".o")
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-I", os.path.join(REPO, "include"),
                               "-I", HOSTSRC, "-c", src, "-o", obj])
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(one, srcs))
    tmp = SHIM + ".tmp"
    if os.path.exists(tmp):
        os.remove(tmp)
    subprocess.check_call(["ar", "rcs", tmp] + objs)
    os.replace(tmp, SHIM)
    return SHIM


if __name__ == "__main__":
    print(build())
