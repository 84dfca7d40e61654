"""Build the in-tree CUDA library ``tinysph_old_gb300/libtsph.so`` for sm_103a.

Three translation units compiled in parallel with nvcc and linked into one
shared library that exports the C ABI of ``include/tsph.h``:

* ``csrc/tsph_api.cu``        the extern "C" boundary and the grid tables
* ``csrc/tsph_engine_f32.cu`` FP32 pair math, FP64 positions
* ``csrc/tsph_engine_f64.cu`` FP64 throughout, ``-fmad=false``
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "libtsph.so")
BUILD = os.path.join(ROOT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-Xcudafe", "--diag_suppress=177"]
UNITS = [
    ("tsph_api.cu", []),
    ("tsph_engine_f32.cu", []),
    ("tsph_engine_f64.cu", ["-fmad=false"]),
    ("tsph_noalloc.cu", []),
    ("tsph_ale.cu", []),
    ("tsph_io.cu", []),
    ("tsph_gnn.cu", []),
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtsph.so")
    return exe


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".cu", ".cuh", ".h"))] + [os.path.join(ROOT, "include", "tsph.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src, extra in UNITS:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"--- {s}\n{o}" for s, o in failed))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


TRACE_LIB = os.path.join(PKG, "libtsph_trace.so")


def _cupti_dirs():
    """(include dir, library dir) of CUPTI in the CUDA toolkit, or None."""
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    for inc, lib in ((os.path.join(cuda, "include"), os.path.join(cuda, "lib64")),
                     *[(os.path.join(cuda, "targets", t, "include"),
                        os.path.join(cuda, "targets", t, "lib"))
                       for t in ("x86_64-linux", "sbsa-linux", "aarch64-linux")],
                     (os.path.join(cuda, "extras", "CUPTI", "include"),
                      os.path.join(cuda, "extras", "CUPTI", "lib64"))):
        if os.path.exists(os.path.join(inc, "cupti.h")) and os.path.exists(
                os.path.join(lib, "libcupti.so")):
            return inc, lib
    return None


def build_trace(force: bool = False) -> str | None:
    """The optional kernel-timeline library (csrc/tsph_trace.cpp, CUPTI
    activity records), used by the benchmark's per-kernel split of a graph
    step.  Returns None where CUPTI is not installed."""
    src = os.path.join(CSRC, "tsph_trace.cpp")
    if not force and os.path.exists(TRACE_LIB) and \
            os.path.getmtime(TRACE_LIB) >= os.path.getmtime(src):
        return TRACE_LIB
    dirs = _cupti_dirs()
    cxx = shutil.which("g++")
    if dirs is None or cxx is None:
        return None
    inc, lib = dirs
    tmp = TRACE_LIB + ".tmp"
    cmd = [cxx, "-std=c++17", "-O2", "-shared", "-fPIC", src, "-o", tmp, f"-I{inc}",
           f"-I{os.path.join(os.path.dirname(inc), 'include')}", f"-L{lib}", "-lcupti",
           f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        print("libtsph_trace.so not built:\n" + r.stdout.decode(errors="replace"),
              file=sys.stderr)
        return None
    os.replace(tmp, TRACE_LIB)
    return TRACE_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_trace(force="--force" in sys.argv))
