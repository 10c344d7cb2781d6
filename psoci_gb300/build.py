"""In-tree build of libpsoci_gpu.so (sm_103a) from psoci_gb300/csrc.

Each translation unit is compiled in parallel with one ``-gencode`` and linked into
``psoci_gb300/_lib/libpsoci_gpu.so``.  The element kernel file (hbuild.cu) is compiled
with ``--fmad=false`` so its products and sums round as the reference's x86 code does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libpsoci_gpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ["util.cu", "dets.cu", "hbuild.cu", "sigma.cu", "davidson.cu", "capi.cu", "io.cu", "noalloc.cu", "density.cu",
           "natorb.cpp", "symeig.cpp"]
PER_FILE = {"hbuild.cu": ["--fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(LIBDIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
           "-Xcompiler", "-pthread",
           "-I" + CSRC, "-c", os.path.join(CSRC, src), "-o", obj] + PER_FILE.get(src, []) + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "psoci_gpu.h"), __file__,
                                                               os.path.join(HERE, "host", "driver_splittest.cpp"),
                                                               os.path.join(HERE, "..", "include", "psoci", "PsociGpu.hpp")]
    if not os.path.exists(DRIVER):
        return True
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False) -> str:
    """Compile (when stale) and return the path of libpsoci_gpu.so."""
    if not force and not _stale():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), ARCH, "-shared", "-Xcompiler", "-pthread", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver()
    if verbose:
        print("built", LIB, file=sys.stderr)
    return LIB


DRIVER = os.path.join(LIBDIR, "psoci_driver")


def build_driver() -> str:
    """The C++ host driver (psoci_gb300/host/driver_splittest.cpp) linked against the library."""
    src = os.path.join(HERE, "host", "driver_splittest.cpp")
    inc = os.path.join(HERE, "..", "include")
    cmd = ["g++", "-std=c++17", "-O2", "-I" + inc, src, "-o", DRIVER, "-L" + LIBDIR, "-lpsoci_gpu",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
