"""Builds libgxcorr.so (the CUDA engine behind include/gxc.h) in-tree.

Each translation unit is compiled for sm_103a in parallel, then linked into
gcorr_gb300/libgxcorr.so.  No torch, no cmake: nvcc and the C++ host compiler.
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
LIB = os.path.join(HERE, "libgxcorr.so")
SOURCES = ["gxc_api.cu", "fstage.cu", "fstage_probe.cu", "fstage_tc.cu", "xstage_fp32.cu", "xstage_tc.cu", "xcorr_api.cu", "xcorr_noalloc.cu", "batch_api.cu",
           "pipeline_api.cu", "conf_io.cpp", "dada_io.cpp", "vdif.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# command-line drivers with the reference harness's interface, linked against the library
APPS = ["testfxkernel", "bench_fxkernel"]
BIN = os.path.join(HERE, "bin")


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgxcorr")


def flags():
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
            "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC] + ARCH


def _needs(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "gxc.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _needs(o, [s] + headers):
            jobs.append([nvcc(), "-c", s, "-o", o] + flags() + (["-Xptxas", "-v"] if verbose else []))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or r.returncode:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode:
                    raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _needs(LIB, objs):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC", "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    build_apps(force=force)
    return LIB


def build_apps(force: bool = False) -> None:
    os.makedirs(BIN, exist_ok=True)
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the command-line drivers")
    hdrs = [os.path.join(ROOT, "include", h) for h in ("gxc.h", "fxkernel_gxc.h", "gxc_common.h")]
    jobs = []
    for app in APPS:
        src = os.path.join(HERE, "apps", app + ".cpp")
        exe = os.path.join(BIN, app)
        if force or _needs(exe, [src, LIB] + hdrs):
            jobs.append([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", exe, "-L", HERE,
                         "-lgxcorr", "-Wl,-rpath,$ORIGIN/..", "-pthread"])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for r, cmd in zip(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs), jobs):
            if r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("driver build failed: " + " ".join(cmd))


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
