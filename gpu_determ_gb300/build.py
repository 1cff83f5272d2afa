"""In-tree build of libgpu_determ.so for sm_103a (nvcc, no cmake).

Each translation unit compiles to ``_build/<name>.o`` in parallel, then one
``nvcc -shared`` link writes ``gpu_determ_gb300/libgpu_determ.so``.  Units are
rebuilt when their source or any header is newer than the object.

    python -m gpu_determ_gb300.build [--force] [--verbose]
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
LIB = os.path.join(PKG, "libgpu_determ.so")
APP_SRC = os.path.join(CSRC, "app", "determ_main.cpp")
APP = os.path.join(PKG, "gd_determ")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
               "-ffp-contract=off", "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]

# per-unit extra flags: the weight builder rounds every expression as written
UNIT_FLAGS = {
    "gd_weights.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gpu_determ_gb300")


def _sources() -> list[str]:
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _newest(paths: list[str]) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src: str, force: bool, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if (not force and os.path.exists(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(path), _newest(_headers()))):
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj + ".tmp"] + ARCH + NVCC_COMMON + UNIT_FLAGS.get(src, [])
    if src.endswith(".cpp"):
        cmd += ["-x", "c++"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose), srcs))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        cmd = [nvcc(), "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    hdrs = [os.path.join(INCLUDE, "gpu_determ_api.hpp"), os.path.join(INCLUDE, "gpu_determ.h")]
    if force or not os.path.exists(APP) or os.path.getmtime(APP) < _newest([LIB, APP_SRC] + hdrs):
        cmd = [nvcc(), "-x", "c++", APP_SRC, "-o", APP + ".tmp", "-std=c++17", "-O2", "-I" + INCLUDE,
               "-Xcompiler", "-ffp-contract=off", "-L" + PKG, "-lgpu_determ", "-lcudart",
               "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(APP + ".tmp", APP)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
