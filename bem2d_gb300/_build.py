"""In-tree build of the native parts (no cmake, no setuptools).

  libbem2d_gpu.so   CUDA kernels + C ABI (csrc/*.cu) for sm_103a
  lib/bem2d.a       the C++ API of the reference library's lib/ (lib/*.cpp),
                    written over the C ABI
Object files go to _build/ at the repository root; translation units are
compiled in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(ROOT, "_build")
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
GPU_LIB = os.path.join(PKG, "libbem2d_gpu.so")
CPP_LIB = os.path.join(LIBDIR, "bem2d.a")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_gpu(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + [os.path.join(ROOT, "include", "bem2d_gpu.h")])
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or not _newer(o, [s] + hdrs)]
    nv = nvcc()

    def comp(so):
        s, o = so
        return _run([nv] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o])

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        for r in ex.map(comp, todo):
            if verbose and r.stderr:
                print(r.stderr)
    if todo or not os.path.exists(GPU_LIB):
        _run([nv] + ARCH + ["-shared", "-o", GPU_LIB] + objs + ["-lcuda"])
    return GPU_LIB


def build_cpp(force=False):
    """The reference-compatible C++ API (bem2d_gb300/lib) as a static archive."""
    srcs = sorted(glob.glob(os.path.join(LIBDIR, "*.cpp")))
    if not srcs:
        return None
    hdrs = glob.glob(os.path.join(LIBDIR, "*.h")) + [os.path.join(ROOT, "include", "bem2d_gpu.h")]
    objs = [os.path.join(BUILD, "lib_" + os.path.basename(s) + ".o") for s in srcs]
    os.makedirs(BUILD, exist_ok=True)
    todo = [(s, o) for s, o in zip(srcs, objs) if force or not _newer(o, [s] + hdrs)]

    def comp(so):
        s, o = so
        return _run(["g++", "-std=c++14", "-O2", "-fPIC", "-w", "-I" + LIBDIR,
                     "-I" + os.path.join(ROOT, "include"), "-c", s, "-o", o])

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo) or 1, os.cpu_count() or 4))) as ex:
        list(ex.map(comp, todo))
    if todo or not os.path.exists(CPP_LIB):
        if os.path.exists(CPP_LIB):
            os.remove(CPP_LIB)
        _run(["ar", "rcs", CPP_LIB] + objs)
    return CPP_LIB


def build_oracle(with_reference=None):
    """The CPU oracle (test infrastructure): the C restatement always, the
    reference library itself when BEM2D_REFERENCE names its checkout."""
    oracle = os.path.join(ROOT, "oracle")
    _run(["make", "-C", oracle, "port"])
    ref = os.environ.get("BEM2D_REFERENCE", "")
    if with_reference is None:
        with_reference = bool(ref) and os.path.isdir(os.path.join(ref, "lib"))
    if with_reference:
        _run(["make", "-C", oracle, "-j8", "ref", "REF=" + ref])


def build_all(force=False):
    build_gpu(force)
    build_cpp(force)
    build_oracle()
