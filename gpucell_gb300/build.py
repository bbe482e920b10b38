"""Build the CUDA library and the CPU oracle in-tree.

``build_library()`` compiles every ``csrc/*.cu`` for sm_103a (one nvcc per
translation unit, in parallel, skipped when the object is newer than its
sources) and links ``gpucell_gb300/lib/libgpucell_gb300.so``.
``build_oracle()`` compiles ``oracle/oracle.c`` with gcc into
``oracle/build/liboracle.so``.  Neither needs a GPU.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpucell_gb300")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ_DIR = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libgpucell_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "build", "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def reference_src() -> str:
    """The reference's src/ directory, read only by the development-time
    recipes that pin the reader, writer and step driver against GPUCell's own
    host code: $GPUCELL_REFERENCE/src, by default the development container's
    read-only checkout.  It does not exist on the GPU machine."""
    return os.path.join(os.environ.get("GPUCELL_REFERENCE", "/root/reference"), "src")
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put the CUDA toolkit on PATH)")


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def build_library(verbose: bool = False, extra_flags=None, force: bool = False) -> str:
    """Compile and link libgpucell_gb300.so; returns its path."""
    nvcc = _nvcc()
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                     + glob.glob(os.path.join(INCLUDE, "**", "*.h"), recursive=True))
    hdr_time = _newest(headers)
    flags = NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append([nvcc] + ARCH + flags + ["-c", src, "-o", obj])
    if jobs:
        workers = min(len(jobs), os.cpu_count() or 4)
        with ThreadPoolExecutor(max_workers=workers) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                if o.strip():
                    print(o)
    if jobs or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < _newest(objs):
        tmp = LIB_PATH + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-Xcompiler", "-pthread", "-o", tmp] + objs)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_oracle(verbose: bool = False) -> str:
    """Compile the FP64 CPU oracle into oracle/build/liboracle.so."""
    src = os.path.join(ORACLE_DIR, "oracle.c")
    hdr = os.path.join(ORACLE_DIR, "oracle.h")
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    if os.path.exists(ORACLE_LIB) and os.path.getmtime(ORACLE_LIB) >= _newest([src, hdr]):
        return ORACLE_LIB
    cc = os.environ.get("CC", "gcc")
    tmp = ORACLE_LIB + ".tmp"
    out = _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                "-Wall", "-I" + INCLUDE, src, "-o", tmp, "-lm"])
    os.replace(tmp, ORACLE_LIB)
    if verbose and out.strip():
        print(out)
    return ORACLE_LIB


def build_reference_io(verbose: bool = False) -> str | None:
    """GPUCell's own input loaders and output writers, linked into
    oracle/_ref/ref_io by oracle/ref_io.mk where the reference's sources are
    present (the tests of the reader and writer compare against it); None
    where they are not, or where `make` is missing."""
    out = os.path.join(ORACLE_DIR, "_ref", "ref_io")
    make = shutil.which("make")
    if not make:
        return None
    res = subprocess.run([make, "-s", "-f", os.path.join("oracle", "ref_io.mk"), "NVCC=" + _nvcc(),
                          "REF=" + reference_src()], cwd=ROOT, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle/ref_io.mk failed\n" + res.stdout + res.stderr)
    if verbose and (res.stdout + res.stderr).strip():
        print(res.stdout + res.stderr)
    return out if os.path.exists(out) else None


if __name__ == "__main__":
    print(build_library(verbose=True, force="--force" in sys.argv))
    print(build_oracle(verbose=True))
    print(build_reference_io(verbose=True))
