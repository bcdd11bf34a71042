"""Build libqvmgpu.so (the C-ABI CUDA library) in-tree for sm_103a.

Every translation unit is compiled in parallel with nvcc into
``qvm_gb300/_build/`` and linked into ``qvm_gb300/libqvmgpu.so`` with the
CUDA runtime linked statically, so the library depends on nothing but the
driver.  Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libqvmgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["state.cu", "gates.cu", "measure.cu", "tile.cu", "program.cu", "plan.cpp",
           "batch.cu", "sbatch.cu", "endpoints.cu", "noise.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-Wall", "--expt-relaxed-constexpr", "-I", INCLUDE]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or os.path.join(
        os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    hs.append(os.path.join(INCLUDE, "qvmgpu.h"))
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, src + ".o")
    path = os.path.join(CSRC, src)
    if not _stale(obj, [path] + _headers()):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-x", "cu", "-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
