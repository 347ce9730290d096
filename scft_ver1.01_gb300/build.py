"""Build the in-tree CUDA library ``libscft_gb300.so`` for sm_103a.

Each translation unit is compiled by nvcc in parallel into ``_build/``, then
linked into the package directory.  Objects are rebuilt when any source or
header is newer than them.  No cmake, one ``-gencode``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libscft_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]

SOURCES = ["capi.cu", "io.cpp", "compat.cpp", "k_line.cu", "k_fields.cu", "k_fast.cu",
           "k_anderson.cu", "group.cu", "noalloc.cu", "adjoint.cu", "spline.cu",
           "k_plane256.cu"]
# Per-file extra flags: the spline's host arithmetic keeps the reference's
# rounding (no FMA contraction by the host compiler, which aarch64 gcc does by
# default).
EXTRA_FLAGS = {"spline.cu": ["-Xcompiler", "-ffp-contract=off"]}
# Drop-in driver of the reference's struct API (init_scft -> fft_test ->
# finalize_cufft), linked against the library: the reference's `scan` binary.
DRIVER_SRC = "scft_main.cpp"
DRIVER = os.path.join(HERE, "scft_gb300_driver")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    out = []
    for d in (CSRC, INCLUDE):
        for root, _, files in os.walk(d):
            out += [os.path.join(root, f) for f in files if f.endswith((".h", ".cuh"))]
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    objs, cmds = [], []
    for src in SOURCES:
        spath = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if _stale(obj, [spath] + hdrs + [__file__]):
            cmds.append([cc] + NVCC_FLAGS + EXTRA_FLAGS.get(src, []) + ["-c", spath, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    if cmds or _stale(LIB, objs):
        run([cc] + ARCH + ["-shared", "-o", LIB] + objs)
    dsrc = os.path.join(CSRC, DRIVER_SRC)
    if _stale(DRIVER, [dsrc, LIB] + hdrs):
        run([cc] + NVCC_FLAGS + ["-I" + os.path.join(INCLUDE, "compat"), dsrc, "-o", DRIVER,
                                 "-L" + HERE, "-lscft_gb300", "-Xlinker", "-rpath=$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
