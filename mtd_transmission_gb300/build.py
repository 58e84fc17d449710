"""Builds libtdm.so (sm_103a kernels + C ABI) and the drop-in executables in-tree.

    python -m mtd_transmission_gb300.build

Each translation unit is compiled in parallel with one -gencode for sm_103a;
host code is compiled with -ffp-contract=off so that the geometry tables and
cap indices are rounded as written on both x86 and Arm hosts.
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
LIB = os.path.join(HERE, "libtdm.so")
BIN = os.path.join(HERE, "bin")
APPS = ("tomo_pretraitement", "tomo_reconstruction", "tomo_pipeline")

CU_SOURCES = ("tdm_api.cu", "k_extract.cu", "k_fields.cu", "k_recon.cu", "k_generic.cu", "k_herraez.cu",
              "tdm_noalloc.cu")
CPP_SOURCES = ("host_io.cpp",)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "tdm.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not force and not _stale(o, [s] + headers):
            continue
        cmd = [nvcc, ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
               "-ffp-contract=off", "-c", s, "-o", o]
        if src.endswith(".cu"):
            cmd.insert(2, "--expt-relaxed-constexpr")
            if ptxas_info:
                cmd.insert(2, "-Xptxas=-v")
        else:
            cmd[1:2] = []  # host C++ through nvcc's host compiler
            cmd.insert(1, "-x")
            cmd.insert(2, "c++")
        jobs.append(cmd)
    outs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for o in outs:
            if o.strip():
                print(o)
    if force or _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart"])
    os.makedirs(BIN, exist_ok=True)
    gxx = shutil.which("g++") or "g++"
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for app in APPS:
        src = os.path.join(CSRC, "apps", app + ".cpp")
        exe = os.path.join(BIN, app)
        common = os.path.join(CSRC, "apps", "app_common.h")
        if os.path.exists(src) and (force or _stale(exe, [src, LIB, common])):
            # tomo_pipeline holds the polarisation states' buffers in device memory (CUDA runtime)
            cu = ["-I", os.path.join(cuda, "include"), "-L", os.path.join(cuda, "lib64"), "-lcudart"] \
                if app == "tomo_pipeline" else []
            _run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", src, "-o", exe, "-I", os.path.join(HERE, "..", "include"),
                  "-L", HERE, "-ltdm"] + cu + ["-Wl,-rpath,$ORIGIN/.."])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
