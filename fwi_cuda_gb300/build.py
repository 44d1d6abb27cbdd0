"""Build the engine library ``fwi_cuda_gb300/_build/libfwi_psv.so`` and the
program ``fwi_cuda_gb300/_build/seis_fwi`` linked to it.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), host C++ with g++; the units
compile in parallel and link into one shared library with a plain C ABI
(``include/fwi_psv.h``).  Usage: ``python -m fwi_cuda_gb300.build``.
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
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libfwi_psv.so")
EXE = os.path.join(OUT, "seis_fwi")  # the reference program's name, on this library

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
             "-I", os.path.join(ROOT, "include"), "-I", CSRC]

# (source, extra flags); the model-side kernels keep FP64 rounding like the
# reference's host code (no FMA contraction).
UNITS = [
    ("psv_kernels_f32.cu", []),
    ("psv_kernels_f64.cu", []),
    ("psv_tiled.cu", []),
    ("psv_vec.cu", []),
    ("psv_fused.cu", []),
    ("psv_march.cu", []),
    ("psv_exact.cu", []),
    ("psv_joint.cu", []),
    ("psv_fwi_kernels.cu", ["-fmad=false"]),
    ("psv_plan_f32.cu", []),
    ("psv_plan_f64.cu", []),
    ("psv_capi.cu", []),
    ("psv_noalloc.cu", []),
    ("psv_host.cpp", []),
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", path, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I", "/usr/local/cuda/include"] + extra + ["-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(EXE):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(EXE))
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (when sources changed) and return the library path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose), UNITS))
    tmp = LIB + ".tmp"
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    cmd = ["g++"] + CXX_FLAGS + [os.path.join(CSRC, "psv_main.cpp"), "-o", EXE, "-L", OUT,
                                 "-lfwi_psv", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:  # the program is a convenience: the library stands without it
        print(f"warning: linking seis_fwi failed:\n{r.stdout}\n{r.stderr}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
