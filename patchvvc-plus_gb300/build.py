"""Build recipe of libpvvc_gb300.so: the CUDA kernels (sm_103a) and the host
C++ layer, compiled in parallel and linked into one shared library next to
this file.  Used by the repository's build entry point; runnable directly
(`python patchvvc-plus_gb300/build.py`)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "libpvvc_gb300.so")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-fmad=false", "-I", INCLUDE] + ARCH
# -ffp-contract=off: host float code must not fuse a*b+c on any host (aarch64 would)
PER_FILE_FLAGS: dict[str, list[str]] = {}
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
             "-pthread", "-I", INCLUDE]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(os.path.join(HERE, "csrc", f) for f in os.listdir(os.path.join(HERE, "csrc")) if f.endswith(".cu"))
    cc = sorted(os.path.join(HERE, "host", f) for f in os.listdir(os.path.join(HERE, "host")) if f.endswith(".cc"))
    return cu, cc


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(d, f) for d in (os.path.join(HERE, "csrc"), os.path.join(HERE, "host"), INCLUDE)
                    for f in os.listdir(d) if f.endswith((".h", ".cuh"))]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(p) for p in deps):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), "-c", src, "-o", obj] + NVCC_FLAGS + PER_FILE_FLAGS.get(os.path.basename(src), [])
    else:
        cmd = [os.environ.get("CXX", "g++"), "-c", src, "-o", obj] + CXX_FLAGS
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cu, cc = sources()
    with cf.ThreadPoolExecutor(max_workers=max(2, min(16, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), cu + cc))
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(o) for o in objs):
        return OUT
    tmp = OUT + ".tmp"
    cmd = [_nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart_static", "-ldl", "-lpthread", "-lrt"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True))
