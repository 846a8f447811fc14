"""Build the engine library for sm_103a, in tree.

    python acoustic3d-fd_gb300/build.py

Compiles csrc/*.cu and csrc/*.cpp in parallel with nvcc into _build/, links
lib/libacoustic3d.so, and copies it under the reference's four library names
(lib/acoustic2order.so, lib/acoustic1order.so, lib/acoustic1vti.so,
lib/acoustic1tti.so), each exporting all four drop-in symbols.

Floating point: --fmad=false and -ffp-contract=off, so every fused
multiply-add is one written in the source (the CPU oracle performs the same
operations and the engines reproduce it bit for bit).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")
LEGACY_NAMES = ("acoustic2order.so", "acoustic1order.so", "acoustic1vti.so", "acoustic1tti.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "-I", os.path.join(HERE, "..", "include")]


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale(src: str, obj: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "acoustic3d.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(name: str) -> str:
    src = os.path.join(CSRC, name)
    obj = os.path.join(BUILD, name + ".o")
    if _stale(src, obj):
        cmd = [NVCC, *ARCH, *FLAGS, "-x", "cu", "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {name}:\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    out = os.path.join(LIB, "libacoustic3d.so")
    if not os.path.exists(out) or any(os.path.getmtime(o) > os.path.getmtime(out) for o in objs):
        tmp = out + ".tmp"
        cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, out)
    for n in LEGACY_NAMES:
        dst = os.path.join(LIB, n)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(out):
            shutil.copy2(out, dst + ".tmp")
            os.replace(dst + ".tmp", dst)
    if verbose:
        print("built", out)
    return out


if __name__ == "__main__":
    try:
        build(verbose=True)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
