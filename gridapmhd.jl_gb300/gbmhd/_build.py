"""Builds libgbmhd.so in-tree from csrc/ with nvcc for sm_103a (no cmake)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "csrc")
OUT = os.path.join(HERE, "libgbmhd.so")
BUILD = os.path.join(os.path.dirname(HERE), "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-O3"]


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _nvcc():
    n = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(n):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbmhd")
    return n


def build(force: bool = False, verbose: bool = False) -> str:
    srcs = sources()
    newest = max(os.path.getmtime(os.path.join(CSRC, s)) for s in os.listdir(CSRC))
    hdr = os.path.join(os.path.dirname(os.path.dirname(HERE)), "include", "gbmhd.h")
    newest = max(newest, os.path.getmtime(hdr), os.path.getmtime(__file__))
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= newest:
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(s):
        obj = os.path.join(BUILD, s + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, "-c", os.path.join(CSRC, s), "-o", obj]
        if s.endswith(".cpp"):
            cmd = [nvcc, "-x", "c++", *FLAGS, "-c", os.path.join(CSRC, s), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {s}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = OUT + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp", "-lcublas"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True, verbose=True))
