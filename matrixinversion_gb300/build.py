"""In-tree build of the CUDA library ``lib/libmi_inverse.so`` for sm_103a.

Each translation unit under ``csrc/`` is compiled by its own nvcc process (in
parallel), then linked with ``nvcc -shared``.  The units of the single
persistent descriptor launch (RDC_UNITS: the kernel and its 128 walks, one
unit per pivot mode) are relocatable device code, joined by one device-link
step before the library link.  Objects are rebuilt only when a source or
header is newer than the object.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libmi_inverse.so")
CSRC_CMP = os.path.join(PKG, "csrc_compare")
LIB_CUBLAS = os.path.join(LIBDIR, "libmi_cublas_ref.so")
DRIVER_SRC = os.path.join(PKG, "driver", "mi_driver.cpp")
BINDIR = os.path.join(PKG, "bin")
DRIVER = os.path.join(BINDIR, "mi_driver")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]
RDC_UNITS = {"mi_descr_persist.cu", "mi_pwalk_none.cu", "mi_pwalk_reference.cu", "mi_pwalk_reference_serial.cu",
             "mi_pwalk_partial.cu"}
DLINK = os.path.join(BUILD, "mi_rdc_dlink.o")


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA library cannot be built")
    return p


def _deps() -> float:
    files = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max(os.path.getmtime(f) for f in files) if files else 0.0


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps()):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *(["-rdc=true"] if os.path.basename(src) in RDC_UNITS else []), "-c", src,
           "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{out.stderr[-4000:]}")
    if verbose:
        sys.stderr.write(out.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every CUDA unit and link the shared library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    rdc = [o for s, o in zip(srcs, objs) if os.path.basename(s) in RDC_UNITS]
    if rdc and (not os.path.exists(DLINK) or os.path.getmtime(DLINK) < max(os.path.getmtime(o) for o in rdc)):
        out = subprocess.run([nvcc(), *ARCH, "-Xcompiler", "-fPIC", "-dlink", *rdc, "-o", DLINK], capture_output=True,
                             text=True)
        if out.returncode != 0:
            raise RuntimeError("device link failed:\n" + out.stderr[-4000:])
    objs = objs + ([DLINK] if rdc else [])
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("link failed:\n" + out.stderr[-4000:])
    build_comparator()
    return LIB


def build_comparator() -> str:
    """The cuBLAS getrf+getri comparison library (measurement only)."""
    src = os.path.join(CSRC_CMP, "mi_cublas_ref.cu")
    if os.path.exists(LIB_CUBLAS) and os.path.getmtime(LIB_CUBLAS) >= os.path.getmtime(src):
        return LIB_CUBLAS
    cmd = [nvcc(), *ARCH, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", src, "-o", LIB_CUBLAS, "-lcublas"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("cuBLAS comparator build failed:\n" + out.stderr[-4000:])
    return LIB_CUBLAS



def build_driver() -> str:
    """The command-line driver ``bin/mi_driver`` (the reference's per-run
    stdout contract over the C ABI), linked against ``lib/libmi_inverse.so``
    through an rpath relative to the binary.  Built on demand, not by
    :func:`build`: the library does not depend on it."""
    if not os.path.exists(LIB):
        build()
    os.makedirs(BINDIR, exist_ok=True)
    newest = max(os.path.getmtime(DRIVER_SRC), os.path.getmtime(LIB), _deps())
    if os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= newest:
        return DRIVER
    cmd = [nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-pthread", "-I" + INCLUDE, DRIVER_SRC, "-o", DRIVER,
           "-L" + LIBDIR, "-lmi_inverse", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN/../lib"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("driver build failed:\n" + out.stderr[-4000:])
    return DRIVER


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    if "--driver" in sys.argv:
        print(build_driver())
