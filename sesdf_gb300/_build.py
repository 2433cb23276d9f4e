"""Compilation of the native parts (CUDA for sm_103a, C host helpers).

Everything is built in-tree: the CUDA library into sesdf_gb300/lib/libsesgb.so and
the synthetic-molecule generator into sesdf_gb300/lib/libsesgb_synth.so. Translation
units compile in parallel; a unit is rebuilt only when a source or header is newer
than its object.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "lib", "obj")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
CUDA_UNITS = ["sesgb_sort.cu", "sesgb_stages.cu", "sesgb_area.cu", "sesgb_api.cu", "sesgb_noalloc.cu",
              "sesgb_cavities.cu"]
CXX_UNITS = ["bcs_sesdf.cpp", "bcs_loader.cpp"]

LIB = os.path.join(LIBDIR, "libsesgb.so")
SYNTH_LIB = os.path.join(LIBDIR, "libsesgb_synth.so")


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(INCLUDE, "bcs", "**", "*.hpp"), recursive=True)


def build_cuda(force: bool = False, verbose: bool = False) -> str:
    """Compiles the CUDA library for sm_103a (cross-compiles on a machine without a GPU)."""
    os.makedirs(OBJDIR, exist_ok=True)
    hdr_time = _newest(_headers())
    procs = []
    objs = []
    for unit in CUDA_UNITS + CXX_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OBJDIR, unit + ".o")
        objs.append(obj)
        if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
            continue
        if unit.endswith(".cu"):
            cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
        else:
            cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-I", INCLUDE, "-I", "/usr/local/cuda/include", "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((unit, out.decode(errors="replace")))
    if failed:
        raise RuntimeError("CUDA build failed:\n" + "\n".join(f"--- {u}\n{o}" for u, o in failed))
    if force or procs or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def build_synth(force: bool = False) -> str:
    src = os.path.join(CSRC, "synth.c")
    os.makedirs(LIBDIR, exist_ok=True)
    if force or not os.path.exists(SYNTH_LIB) or os.path.getmtime(SYNTH_LIB) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", SYNTH_LIB + ".tmp", src, "-lm"],
                       check=True)
        os.replace(SYNTH_LIB + ".tmp", SYNTH_LIB)
    return SYNTH_LIB


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_synth(force)
    build_cuda(force, verbose)
