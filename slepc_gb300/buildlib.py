"""Build recipe for libslepc_gb300.so: every CUDA/C++ translation unit under csrc/ compiled for sm_103a.

nvcc -gencode arch=compute_103a,code=sm_103a, one object per source compiled in parallel, linked into
slepc_gb300/_build/libslepc_gb300.so (in-tree, git-ignored).  Objects are rebuilt only when a source or header
is newer than the object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libslepc_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-Wall", "-Xcompiler", "-fopenmp", "-I", os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build slepc_gb300")
    return exe


def _newest_header() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


NATIVE_LIB = os.path.join(BUILD, "libmatgen_native.so")


def build_native(force: bool = False) -> str:
    """Host-only helpers of the matrix generators (gcc, no CUDA)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "native", "matgen_native.c")
    if force or not os.path.exists(NATIVE_LIB) or os.path.getmtime(NATIVE_LIB) < os.path.getmtime(src):
        cc = shutil.which("gcc") or shutil.which("cc")
        if not cc:
            raise RuntimeError("no C compiler for the native generator helpers")
        r = subprocess.run([cc, "-O2", "-std=c11", "-fopenmp", "-shared", "-fPIC", "-o", NATIVE_LIB + ".tmp", src, "-lm"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"gcc failed for matgen_native.c:\n{r.stdout}\n{r.stderr}")
        os.replace(NATIVE_LIB + ".tmp", NATIVE_LIB)
    return NATIVE_LIB


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    build_native(force)
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr = _newest_header()
    flags = FLAGS + list(extra_flags or [])
    jobs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr):
            jobs.append((s, o))

    def compile_one(job):
        s, o = job
        cmd = [nvcc()] + ARCH + flags + ["-c", s, "-o", o + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(s)}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        os.replace(o + ".tmp", o)
        return o

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, jobs))
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in srcs]
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
