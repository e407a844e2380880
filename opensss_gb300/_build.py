"""Build ``opensss_gb300/libsss300.so`` from ``opensss_gb300/csrc/*.cu`` for sm_103a.

Each translation unit is compiled in parallel with nvcc (one -gencode,
``compute_103a``/``sm_103a``), then linked into one shared library in-tree.
The benchmark's throughput probes (``csrc/probe/probe.cu``) go into a library
of their own, ``libsss300_probe.so``, which only ``bench.py`` loads.
A rebuild happens only when a source or header is newer than the library.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libsss300.so")
PROBE_LIB = os.path.join(PKG, "libsss300_probe.so")
PROBE_SRC = os.path.join(CSRC, "probe", "probe.cu")
OBJ_DIR = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the sm_103a engine cannot be built")
    return path


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(
        os.path.join(INCLUDE, "*.h"))


def needs_build() -> bool:
    for lib, deps in ((LIB, _deps()), (PROBE_LIB, _deps() + [PROBE_SRC])):
        if not os.path.exists(lib):
            return True
        t = os.path.getmtime(lib)
        if any(os.path.getmtime(f) > t for f in deps):
            return True
    return False


def _compile(src: str, extra) -> str:
    obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    """Compile and link; returns the library path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources() + [PROBE_SRC]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    for lib, lib_objs in ((LIB, objs[:-1]), (PROBE_LIB, objs[-1:])):
        tmp = lib + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", *lib_objs, "-o", tmp, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    if verbose:
        print(f"built {LIB}")
    return LIB


def ptxas_report(src: str) -> str:
    """Registers / spills / shared memory per kernel (-Xptxas -v)."""
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-Xptxas", "-v", "-c", src, "-o", os.devnull]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stdout + r.stderr


if __name__ == "__main__":
    import sys

    build(force="--force" in sys.argv, verbose=True)
