"""Builds libglinalg_gb300.so in-tree from csrc/ with nvcc for sm_103a.

Each translation unit compiles in parallel into _build/, then nvcc links the shared library
next to this file.  Usage: ``python generic-linalg_gb300/build.py [--force]`` or
``build_library()`` from Python.
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
LIB = os.path.join(HERE, "libglinalg_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              f"-I{INCLUDE}", f"-I{CSRC}", "--expt-relaxed-constexpr"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _newest_header():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return max(os.path.getmtime(h) for h in hs) if hs else 0.0


def _compile(src, force, extra):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if not force and os.path.exists(obj):
        t = os.path.getmtime(obj)
        if t > os.path.getmtime(path) and t > _newest_header():
            return obj, None
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        # host-only code: no multiply-add contraction, so that the input generators give the
        # same bits on aarch64 (FMA in the base ISA) as on x86_64
        cmd = [nvcc(), "-x", "c++"] + NVCC_FLAGS + ["-Xcompiler", "-ffp-contract=off"] + extra + ["-c", path, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{p.stdout}\n{p.stderr}"
    return obj, None


def build_library(force=False, verbose=False, extra=None):
    """Compile every csrc/ translation unit and link the shared library; returns its path."""
    extra = list(extra or [])
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, force, extra), srcs))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
