"""Builds libuwgpu.so (the CUDA library behind include/uwgpu.h) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
earthbyte_underworld_gb300/_build/libuwgpu.so.  No PyTorch or CMake is involved; the same
recipe runs on x86_64 (cross-compiling) and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libuwgpu.so")
SOURCES = ["capi.cu", "binning.cu", "assembly.cu", "operator.cu", "solver.cu", "gwg_stencil.cu", "unet.cu", "advect.cu", "noalloc.cu", "weights.cu", "tc_check.cu", "population.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libuwgpu")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                   "-I", os.path.join(HERE, "..", "include")] + list(extra)


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    deps = [src, os.path.join(CSRC, "internal.cuh"), os.path.join(CSRC, "tc.cuh"), os.path.join(HERE, "..", "include", "uwgpu.h")]
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        if ptxas_info or _stale(obj, src):
            jobs.append([cc, "-c", src, "-o", obj] + _flags(extra))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_info:
                sys.stdout.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if jobs or not os.path.exists(LIB):
        cmd = [cc, "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + r.stdout + r.stderr)
    build_host()
    return LIB


HOST = os.path.join(BUILD, "uw_stokes_host")


def build_host() -> str:
    """Compiles the C host program (host/uw_stokes_host.c) against libuwgpu.so with gcc."""
    src = os.path.join(HERE, "host", "uw_stokes_host.c")
    if os.path.exists(HOST) and os.path.getmtime(HOST) >= max(os.path.getmtime(src), os.path.getmtime(LIB)):
        return HOST
    cc = shutil.which("gcc") or shutil.which("cc")
    cmd = [cc, "-O2", "-std=c11", "-Wall", src, "-I", os.path.join(HERE, "..", "include"), "-L", BUILD, "-luwgpu",
           "-Wl,-rpath,$ORIGIN", "-lm", "-o", HOST]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host build failed: " + r.stdout + r.stderr)
    return HOST


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
