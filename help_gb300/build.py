"""Compile the native libraries of help_gb300 in-tree.

* ``help_gb300/_lib/libhelp_gpu.so`` -- the sm_103a CUDA backend behind the
  C ABI of ``include/help_gpu.h`` (nvcc, one ``-gencode``, translation units
  compiled in parallel);
* ``help_gb300/_lib/libhelp_lp.so`` -- host C++: instance generators, MPS
  writer and the HSD interior-point driver (``include/help_lp.h``).

Host code is compiled with ``-ffp-contract=off`` so generated instances and
the driver's arithmetic are identical on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_lib", "obj")

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

GPU_CU = ["api.cu", "pcg.cu", "pcg_resident.cu", "renew.cu", "dense.cu", "vec.cu", "adat.cu", "noalloc.cu", "mlp.cu",
          "learned.cu", "mlp_api.cu"]
GPU_CPP = ["items.cpp", "pair.cpp"]
GPU_HDR = ["common.cuh", "spmv.cuh", "kernels.h", "context.h", "items.h", "mlp.h", "guard.h"]
LP_CPP = ["lp_gen.cpp", "hsd.cpp", "lp_io.cpp", "lindep.cpp"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_gpu(verbose: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    out = os.path.join(LIBDIR, "libhelp_gpu.so")
    hdrs = [os.path.join(CSRC, h) for h in GPU_HDR] + [os.path.join(ROOT, "include", "help_gpu.h")]
    jobs = []
    objs = []
    for src in GPU_CU:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append([NVCC, GENCODE, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "-c", s, "-o", o])
    for src in GPU_CPP:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append([CXX, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if jobs or _newer(out, objs):
        _run([NVCC, GENCODE, "-shared", "-o", out] + objs + ["-lcudart"])
    if verbose:
        print("built", out)
    return out


def build_lp(verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    out = os.path.join(LIBDIR, "libhelp_lp.so")
    srcs = [os.path.join(CSRC, s) for s in LP_CPP]
    deps = srcs + [os.path.join(ROOT, "include", "help_lp.h"), os.path.join(CSRC, "guard.h")]
    if _newer(out, deps):
        _run([CXX, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-o", out] + srcs)
    if verbose:
        print("built", out)
    return out


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_gpu, verbose)
        f2 = ex.submit(build_lp, verbose)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
