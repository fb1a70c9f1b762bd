"""Builds libp3g_gb300.so (the C-ABI library) with nvcc for sm_103a.

Each translation unit is compiled in parallel into _build/, then linked
in-tree as plonky3-gpu_gb300/lib/libp3g_gb300.so.  Rebuilds only what changed
(source or header newer than its object, or other compiler flags).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libp3g_gb300.so")
SOURCES = ["capi.cu", "lde_bb.cu", "lde_gl.cu", "dft_bb.cu", "dft_gl.cu", "merkle.cu", "merkle_s1.cu", "merkle_s2.cu",
           "merkle_s3.cu", "merkle_s4.cu", "fold.cu", "open.cu", "fri.cu", "lde_noalloc.cu", "plan.cu", "server.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    # P3G_NVCC_FLAGS: extra nvcc flags (e.g. -D settings of the kernels' build-time knobs)
    extra = os.environ.get("P3G_NVCC_FLAGS", "").split()
    return ARCH + extra + [
        "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
        "-I", os.path.join(REPO, "include"), "-I", CSRC,
    ]


def _headers_mtime() -> float:
    m = os.path.getmtime(os.path.join(REPO, "include", "p3g.h"))
    for f in os.listdir(CSRC):
        if f.endswith((".cuh", ".hpp", ".h")):
            m = max(m, os.path.getmtime(os.path.join(CSRC, f)))
    return m


def _compile(src: str, hdr_mtime: float, verbose: bool, flags_changed: bool) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    if not flags_changed and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(srcp), hdr_mtime):
        return obj
    cmd = [nvcc()] + _flags() + ["-c", srcp, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hm = _headers_mtime()
    # objects built with other flags (another P3G_NVCC_FLAGS) are stale too
    stamp = os.path.join(BUILD, "flags.txt")
    flags = " ".join(_flags())
    old = open(stamp).read() if os.path.exists(stamp) else None
    changed = old != flags
    with cf.ThreadPoolExecutor(max_workers=jobs or len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, hm, verbose, changed), SOURCES))
    if changed:
        with open(stamp, "w") as f:
            f.write(flags)
    if changed or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
