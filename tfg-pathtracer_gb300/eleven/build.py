"""Build the native parts in-tree.

- libeleven.so: the product (CUDA kernels for sm_103a + C++ host + C-ABI),
  compiled with nvcc, translation units in parallel, then linked.
- oracle/liborc.so: the plain-C restatement used by the tests (make).
- oracle/_ref/libref.so: the reference's own headers behind the probe ABI,
  only where the reference sources are present.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(PKG)                      # tfg-pathtracer_gb300/
ROOT = os.path.dirname(PKG_ROOT)                     # repository root
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB = os.path.join(PKG_ROOT, "libeleven.so")
CLI = os.path.join(PKG_ROOT, "bin", "eleven")  # the command-line renderer
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")
# the reference tree: an unmodified copy in baseline/_ref/ (git-ignored; made
# by `make -C oracle ref-copy` where the original exists, and carried with the
# working tree to the GPU machine)
REF_SRC = os.environ.get("ELEVEN_REF_DIR", os.path.join(ROOT, "baseline", "_ref", "src", "tfg-pathtracer"))

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no multiply-add contraction in device code, so every kernel
# that inlines the same shading code (the wavefront's shade, its gradient
# variant, the replay walk) rounds every operation alike and their paths
# agree bit for bit whatever register budget each kernel is compiled for;
# explicit fmaf() (the slab tests) is unaffected.
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "--fmad=false", "-Xcompiler", "-fPIC",
            "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]
# extra nvcc flags (tuning sweeps); a change needs build_product(force=True)
CU_FLAGS += os.environ.get("ELEVEN_NVCC_FLAGS", "").split()

SOURCES = ["capi.cpp", "scene.cpp", "bvh_build.cpp", "loader.cpp", "tangents.cpp",
           "trace.cu", "render.cu", "env.cu", "batch.cu", "adjoint.cu", "post.cu", "bvh_gpu.cu", "probe.cu"]


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers():
    hs = [os.path.join(INCLUDE, "eleven.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".h", ".cuh", ".hpp")):
            hs.append(os.path.join(CSRC, f))
    return hs


def build_product(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    objs, jobs = [], []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            flags = list(CU_FLAGS)
            if s.endswith(".cu"):
                flags += ARCH + ["-Xptxas", "-v"] if verbose else ARCH
            jobs.append([NVCC] + flags + ["-x", "cu" if s.endswith(".cu") else "c++", "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"])
    cli_src = os.path.join(CSRC, "cli.cpp")
    if force or _stale(CLI, [cli_src, LIB, os.path.join(INCLUDE, "eleven.h")]):
        os.makedirs(os.path.dirname(CLI), exist_ok=True)
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", CLI, "-L" + PKG_ROOT, "-leleven",
              "-Wl,-rpath,$ORIGIN/.."])
    return LIB


def build_oracle(force=False):
    target = os.path.join(ORACLE, "liborc.so")
    args = ["make", "-s", "-C", ORACLE, "liborc.so"]
    if force:
        args.insert(1, "-B")
    _run(args)
    return target


def copy_ref():
    """Makes the baseline/_ref/ copy of the reference tree where the original
    is present (the Makefile names its location); no-op otherwise."""
    if os.path.isdir(REF_SRC) or "ELEVEN_REF_DIR" in os.environ:
        return
    r = subprocess.run(["make", "-s", "-C", ORACLE, "ref-copy"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    if r.returncode != 0 and os.path.isdir(REF_SRC):
        raise RuntimeError("reference copy failed:\n" + r.stdout)


def build_ref(force=False):
    """Reference headers through oracle/ref_shim.cpp; only where they exist."""
    copy_ref()
    if not os.path.isdir(REF_SRC):
        return None
    args = ["make", "-s", "-C", ORACLE, "ref", "REF_DIR=" + REF_SRC]
    if force:
        args.insert(1, "-B")
    _run(args)
    return os.path.join(ORACLE, "_ref", "libref.so")


def build_all(force=False, verbose=False):
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f1 = ex.submit(build_product, force, verbose)
        f2 = ex.submit(build_oracle, force)
        f3 = ex.submit(build_ref, force)
        return f1.result(), f2.result(), f3.result()


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    for p in (LIB,):
        if os.path.exists(p):
            os.remove(p)


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv, verbose="-v" in sys.argv))
