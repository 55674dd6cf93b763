"""Build libngbem_gb300.so in-tree: host C++ with g++, kernels with nvcc for sm_103a.

Host code is compiled with -ffp-contract=off so the cluster tree is bit-identical on
x86_64 and aarch64.  Objects go to ngbem_gb300/_build/, the library next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libngbem_gb300.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["quadrature.cpp", "geometry.cpp", "operator.cpp", "apply.cpp", "gmres.cpp", "energy_host.cpp",
                "tc_host.cpp", "serialize.cpp", "capi.cpp"]
CUDA_SOURCES = ["nearfield.cu", "nearfield_l2p12.cu", "nearfield_l2p3r.cu", "nearfield_l2p3s.cu", "nearfield_h1p2.cu", "nearfield_h1p3r.cu", "nearfield_h1p3s.cu", "nearfield_hdiv.cu", "nearfield_hdivs.cu", "nearfield_hdiv34r.cu", "nearfield_hdiv34s.cu", "aca.cu", "matvec.cu", "mult_noalloc.cu", "energy.cu", "gmres_batch.cu",
                "tc_matvec.cu", "potential.cu"]
HEADERS = ["bem_shared.h", "bem_device.cuh", "kernels.h", "host.hpp", "nearfield_kernels.cuh"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link; returns the path of the shared library."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "ngbem_gb300.h")]
    cxx = shutil.which("g++") or "g++"
    cmds = []
    objs = []
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            cmds.append([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-Wno-unused-variable", "-Wno-unused-but-set-variable",
                         f"-I{CUDA_HOME}/include", "-c", s, "-o", o])
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            cmds.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
                         "-c", s, "-o", o])
    jobs = jobs or min(8, max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for r in ex.map(_run, cmds):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, file=sys.stderr)
    if _newer(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
