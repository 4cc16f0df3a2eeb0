"""Builds libsph_cuda (sm_103a) in-tree: sph_gb300/lib/libsph_cuda.so.

nvcc compiles each translation unit in parallel with
`-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`, then links one
shared library with the CUDA runtime linked statically, so the library
depends only on the driver.  Rebuilds only when a source or header is newer
than the library.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(ROOT, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libsph_cuda.so")
CHECKED_LIB = os.path.join(LIB_DIR, "libsph_cuda_checked.so")
HOST = os.path.join(PKG, "host")
COMPUTE_RANK = os.path.join(LIB_DIR, "sph_compute_rank")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def sources() -> list:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    return not os.path.exists(COMPUTE_RANK) or _stale_against(LIB)


def _stale_against(lib: str) -> bool:
    t = os.path.getmtime(lib)
    deps = sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) \
        + glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(HOST, "*.c")) \
        + [os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps)


def build_host(verbose: bool = False) -> str:
    """The C compute-rank program (sph_gb300/host/compute_rank.c) linked
    against libsph_cuda, next to it."""
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-std=c99", "-O2", "-Wall", "-I", INCLUDE, os.path.join(HOST, "compute_rank.c"),
           "-L", LIB_DIR, "-lsph_cuda", "-Wl,-rpath,$ORIGIN", "-lm", "-o", COMPUTE_RANK]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("host program build failed:\n" + r.stdout.decode(errors="replace"))
    return COMPUTE_RANK


def _compile_lib(lib: str, obj_dir: str, extra: list, verbose: bool) -> None:
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    procs = []
    objs = []
    for src in sources():
        obj = os.path.join(obj_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, lib)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles libsph_cuda.so (and the compute-rank program) if needed;
    returns the library's path."""
    if not force and not _stale():
        return LIB
    _compile_lib(LIB, OBJ, [], verbose)
    build_host(verbose)
    return LIB


def build_checked(force: bool = False, verbose: bool = False) -> str:
    """The bounds-checked variant (-DSPH_BOUNDS_CHECK), libsph_cuda_checked.so:
    every data-dependent index of the step's kernels is tested before its
    access and a bad one is recorded (sph_cuda_bounds_errors)."""
    if not force and os.path.exists(CHECKED_LIB) and not _stale_against(CHECKED_LIB):
        return CHECKED_LIB
    _compile_lib(CHECKED_LIB, os.path.join(OBJ, "checked"), ["-DSPH_BOUNDS_CHECK"], verbose)
    return CHECKED_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
