"""Builds libmprgp_gb300.so in-tree with nvcc for sm_103a.

The translation units in SOURCES are compiled in parallel and linked into
mprgp_gb300/_build/libmprgp_gb300.so.  The same recipe runs on the x86_64
build host and the aarch64 GPU host: no architecture-specific host flags.

build(checks=True) makes the bounds-checked debug build instead
(-DMPRGP_CHECKS: the kernels check the indices they read from device arrays
and report a bad one as MPRGP_INVALID), in mprgp_gb300/_build_checks/; set
MPRGP_LIBRARY to its path to load it in place of the release build.
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
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmprgp_gb300.so")
CHECKS_DIR = os.path.join(HERE, "_build_checks")
CHECKS_LIB = os.path.join(CHECKS_DIR, "libmprgp_gb300_checks.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cu", "capi.cu", "noalloc.cu", "server.cu", "fem.cu", "planes.cu", "ica.cu",
           "beam.cpp"]
# ica.cu reproduces a CPU restatement operation for operation: no contraction
# of products and sums into fused multiply-adds there.  beam.cpp's host
# arithmetic is rounded as written on every host (GCC contracts to FMA by
# default where the host ISA has one), so the beam QPs are the same bits on
# x86_64 and aarch64.
FILE_FLAGS = {"ica.cu": ["-fmad=false"], "beam.cpp": ["-Xcompiler", "-ffp-contract=off"]}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build")
    return path


def _compile(src: str, ptxas_verbose: bool, checks: bool = False) -> str:
    obj = os.path.join(CHECKS_DIR if checks else OUT_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-std=c++17", "-O3",
           "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
    if src.endswith(".cu"):
        cmd += ARCH + ["-lineinfo"] + FILE_FLAGS.get(src, [])
        cmd += os.environ.get("MPRGP_NVCC_FLAGS", "").split()
        if checks:
            cmd += ["-DMPRGP_CHECKS"]
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd += ["-x", "c++"] + FILE_FLAGS.get(src, [])
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if ptxas_verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def _stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "mprgp_gpu.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, ptxas_verbose: bool = False, checks: bool = False) -> str:
    """Compiles the library (checks: the bounds-checked debug build) if any
    source is newer; returns its path."""
    lib, out_dir = (CHECKS_LIB, CHECKS_DIR) if checks else (LIB, OUT_DIR)
    if not force and not ptxas_verbose and not _stale(lib):
        return lib
    os.makedirs(out_dir, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, ptxas_verbose, checks), SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC", "-lcudart_static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
