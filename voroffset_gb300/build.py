"""Builds libvoroffset_gpu.so (and the host-only input generator
libvoroffset_synth.so) in-tree for sm_103a.

Every CUDA translation unit is compiled with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` in parallel,
host C++ with g++, and everything is linked into
``voroffset_gb300/libvoroffset_gpu.so``. Floating-point contraction is off on
both sides (``--fmad=false``, ``-ffp-contract=off``): the path reproduces the
reference's separately rounded FP64 arithmetic.

Usage: ``python -m voroffset_gb300.build [--force] [--verbose]``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BIN = os.path.join(PKG, "bin")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libvoroffset_gpu.so")
SYNTH_SRC = os.path.join(PKG, "synth", "vo_synth.cpp")
SYNTH_LIB = os.path.join(PKG, "libvoroffset_synth.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cpp"))
    cpp.append(os.path.join(HOST, "voroffset_host.cpp"))
    return cu, cpp


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs += [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max((os.path.getmtime(h) for h in hdrs), default=0.0)


def _compile(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    hdr_time = _deps()
    jobs, objs = [], []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append([nvcc, ARCH, "-lineinfo", "-O3", "-std=c++17", "--fmad=false", "-Xptxas=-v",
                         "-Xcompiler=-fPIC,-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}", "-c", src,
                         "-o", obj])
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread",
                         f"-I{INCLUDE}", f"-I{CSRC}", f"-I{HOST}", "-I/usr/local/cuda/include", "-c", src,
                         "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for log in ex.map(lambda c: _compile(c, verbose), jobs):
                logs.append(log)
        with open(os.path.join(BUILD, "ptxas.log"), "w") as fh:
            fh.write("\n".join(logs))
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _compile([nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-lpthread"], verbose)
        os.replace(tmp, LIB)
    # host-only input generator, a library of its own (no device code, not part of the GPU library)
    if not os.path.exists(SYNTH_LIB) or os.path.getmtime(SYNTH_LIB) < max(os.path.getmtime(SYNTH_SRC), hdr_time):
        tmp = SYNTH_LIB + ".tmp"
        _compile(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", f"-I{INCLUDE}",
                  SYNTH_SRC, "-o", tmp], verbose)
        os.replace(tmp, SYNTH_LIB)
    cli = os.path.join(BIN, "offset3d_gpu")
    cli_src = os.path.join(HOST, "offset3d_gpu.cpp")
    if not os.path.exists(cli) or os.path.getmtime(cli) < max(os.path.getmtime(LIB), os.path.getmtime(cli_src)):
        os.makedirs(BIN, exist_ok=True)
        _compile(["g++", "-std=c++17", "-O2", f"-I{INCLUDE}", f"-I{HOST}", cli_src, "-o", cli, f"-L{PKG}",
                  "-lvoroffset_gpu", "-Wl,-rpath,$ORIGIN/..", "-pthread"], verbose)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(p)
