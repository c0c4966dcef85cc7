"""In-tree build of the CUDA library (libnsfem_gb300.so) and the C++ command-line driver (bin/nsfem).

Every .cu translation unit is compiled for sm_103a only, in parallel, then linked into one shared library that
exports the C ABI of include/nsfem_gb300.h.  No CMake: nvcc and g++ are called directly.
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
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnsfem_gb300.so")
CLI = os.path.join(PKG, "bin", "nsfem")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]
CU_SOURCES = ["nsf_cg.cu", "nsf_cg_multi.cu", "nsf_bc.cu", "nsf_sparse.cu", "nsf_locate.cu", "nsf_assembly.cu", "nsf_api.cu", "nsf_noalloc.cu",
              "nsf_step.cu", "nsf_precond.cu", "nsf_tc_gemm.cu", "nsf_learn.cu"]
HOST_SOURCES = ["host/json.cpp", "host/expression.cpp", "host/scene.cpp", "host/nsfem_main.cpp"]
LIB_HOST_SOURCES = ["host/expression.cpp"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    """Compile what changed; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "nsfem_gb300.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    # host C++ compiled into the library (boundary-expression evaluator behind nsf_eval_expression)
    for src in LIB_HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.basename(src).replace(".cpp", ".host.o"))
        objs.append(o)
        if force or _stale(o, [s] + headers + [s.replace(".cpp", ".h")]):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-I", os.path.join(ROOT, "include"), "-c", s, "-o", o])
    out = []
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for res in ex.map(_run, jobs):
            out.append(res)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    # command-line driver: host C++ over the C ABI
    host_srcs = [os.path.join(CSRC, h) for h in HOST_SOURCES]
    if all(os.path.exists(h) for h in host_srcs):
        os.makedirs(os.path.dirname(CLI), exist_ok=True)
        host_hdrs = [os.path.join(CSRC, "host", f) for f in os.listdir(os.path.join(CSRC, "host")) if f.endswith(".h")]
        if force or _stale(CLI, host_srcs + host_hdrs + [LIB]):
            _run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-o", CLI, *host_srcs,
                  "-L", PKG, "-lnsfem_gb300", "-Wl,-rpath,$ORIGIN/.."])
    if verbose:
        sys.stdout.write("".join(out))
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv, force="--force" in sys.argv)
    print(LIB)
