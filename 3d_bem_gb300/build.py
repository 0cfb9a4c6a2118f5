"""Build libbemgpu.so in-tree (sm_103a only).

Every CUDA translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a`` and the host C++ by g++, in
parallel; the result is ``3d_bem_gb300/_build/libbemgpu.so``.  Run as
``python 3d_bem_gb300/build.py`` or call :func:`build`.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libbemgpu.so")
ROOT = os.path.dirname(HERE)

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(
    os.path.join(CUDA_HOME, "bin", "nvcc")) else shutil.which("nvcc") or "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["nearfield.cu", "aca.cu", "hmatvec.cu", "krylov.cu", "post.cu", "hlu_solve.cu", "recompress.cu",
              "selector.cu", "field.cu", "hlu_exec.cu"]
CPP_SOURCES = ["host_tree.cpp", "hlu.cpp", "hlu_plan.cpp", "capi.cpp", "msh.cpp"]


def _sources():
    return [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "bemgpu.h"))
    return hs


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _sources() + _headers() + [__file__])


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include")]
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", *inc, "-c", src, "-o", obj]
    else:
        # hlu.cpp: std::complex products inline (-fcx-limited-range) instead of
        # the library routine that guards against Inf/NaN operands; the H-LU
        # factors only see finite matrix entries, and its many small QRs and
        # SVDs run ~1.6x faster
        extra = ["-fcx-limited-range"] if os.path.basename(src) == "hlu.cpp" else []
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", *extra,
               "-I", os.path.join(CUDA_HOME, "include"), *inc, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA library if any source changed; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), _sources()))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
