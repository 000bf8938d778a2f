"""In-tree build of the native parts of biospring_gb300.

* ``libbiospring_gb300.so`` -- the sm_103a kernels and the C ABI of
  ``include/biospring_gb300.h`` (nvcc, one ``-gencode``, translation units in parallel);
* ``libbs_synth.so`` -- host-only generators of the synthetic systems.

Everything is compiled next to its sources and git-ignored. Host code is built with
``-ffp-contract=off`` so that it gives the same floats on x86-64 and aarch64.
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
LIB = os.path.join(PKG, "libbiospring_gb300.so")
SYNTH = os.path.join(PKG, "libbs_synth.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["bs_kernels.cu", "bs_batch.cu", "bs_adjoint.cu", "bs_rigid.cu", "bs_capi.cu", "bs_noalloc.cu"]
HOST_SOURCES = ["bs_msp.cpp", "bs_field.cpp", "bs_nc.cpp", "bs_xtc.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build biospring_gb300")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + proc.stdout)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "biospring_gb300.h"))
    return hs


def build_library(verbose_ptxas: bool = False) -> str:
    """Compiles libbiospring_gb300.so for sm_103a (cross-compiles without a GPU)."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    objs = []
    jobs = []
    for src in CUDA_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if _stale(obj, [path] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-c", path, "-o", obj]
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in HOST_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if _stale(obj, [path] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


def build_synth() -> str:
    src = os.path.join(CSRC, "synth.cpp")
    if _stale(SYNTH, [src]):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", src, "-o", SYNTH])
    return SYNTH


def build_all(verbose_ptxas: bool = False) -> None:
    build_synth()
    build_library(verbose_ptxas=verbose_ptxas)


if __name__ == "__main__":
    build_all(verbose_ptxas="-v" in sys.argv)
    print(LIB)
