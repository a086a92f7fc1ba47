"""Build of the native parts, in-tree, with nvcc and gcc only (no cmake, no torch extension).

  computeql_gb300/libcqlcuda.so  - the CUDA backend behind include/cqlcuda.h (sm_103a)
  computeql_gb300/libcqlops.so   - the C99 operator layer over that ABI (include/cqlops.h)

Translation units compile in parallel; a unit is rebuilt only when its source or a header is newer
than its object. The same recipe runs on x86_64 (cross-compiling device code) and on the aarch64
GPU host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["runtime.cu", "k_aggregate.cu", "k_scan.cu", "k_hash.cu", "k_join.cu", "k_sort.cu", "k_fixed.cu", "k_window.cu"]
C_SOURCES = ["cql_ops.c", "cql_program.c", "cql_codegen.c", "cql_ops_filter.c", "cql_ops_hash.c", "cql_ops_join.c", "cql_ops_sort.c", "cql_ops_fixed.c", "cql_zonemap.c", "cql_pool.c", "cql_batch.c", "cql_serve.c", "cql_having.c", "cql_resident.c", "cql_gather.c"]

LIB_CUDA = os.path.join(PKG, "libcqlcuda.so")
LIB_OPS = os.path.join(PKG, "libcqlops.so")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _compile_cu(src, ptxas_verbose=False):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()) and not ptxas_verbose:
        return obj, ""
    cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "--std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
           "-c", src, "-o", obj]
    if ptxas_verbose:
        cmd.insert(1, "-Xptxas=-v")
    out = _run(cmd)
    return obj, out


def _compile_c(src):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj
    _run(["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-Wno-unused-function", "-Werror=implicit-function-declaration", "-I", INCLUDE, "-I", HOST, "-c", src, "-o", obj])
    return obj


def build(verbose=False, ptxas_verbose=False):
    """Compile both libraries; returns their paths."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in CU_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile_cu(s, ptxas_verbose), srcs))
    objs = [o for o, _ in results]
    if verbose or ptxas_verbose:
        for _, out in results:
            if out:
                sys.stdout.write(out)
    if _stale(LIB_CUDA, objs):
        cudart_dir = os.path.join(CUDA_HOME, "lib64")
        if not os.path.isdir(cudart_dir):
            cudart_dir = os.path.join(CUDA_HOME, "lib")
        _run([NVCC, *ARCH, "-shared", "-o", LIB_CUDA, *objs, "-L", cudart_dir, "-lcudart", "-lnvrtc",
              "-Xlinker", "-rpath=" + cudart_dir])
    cobjs = [_compile_c(os.path.join(HOST, f)) for f in C_SOURCES]
    if _stale(LIB_OPS, cobjs + [LIB_CUDA]):
        _run(["gcc", "-shared", "-o", LIB_OPS, *cobjs, "-L", PKG, "-lcqlcuda", "-Wl,-rpath,$ORIGIN", "-lm", "-lpthread"])
    return LIB_CUDA, LIB_OPS


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    for p in (LIB_CUDA, LIB_OPS):
        if os.path.exists(p):
            os.remove(p)


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv)
    print(LIB_CUDA)
    print(LIB_OPS)
