"""Builds libkvtomo.so, the engine's C-ABI library, for sm_103a.

Each CUDA translation unit is compiled by nvcc in parallel and the objects are
linked into kevernals_gb300/libkvtomo.so (in-tree; git-ignored).  kv_rc.cu is
compiled with -fmad=false so that no multiply-add is fused in the
reference-compatible operators.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkvtomo.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "kv_api.cu": [],
    "kv_exact.cu": [],
    "kv_rc.cu": ["-fmad=false"],
    "kv_misc.cu": [],
    "kv_fwd_slab.cu": [],
    "kv_back_stage.cu": [],
    "kv_unet.cu": [],
}


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _sources_newer_than(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "kvtomo.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
           "-I", INCLUDE, "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj, *extra]
    if verbose_ptxas:
        cmd.append("-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose_ptxas=False):
    """Compiles and links libkvtomo.so; returns its path."""
    if not force and not _sources_newer_than(LIB):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = {ex.submit(_compile, s, e, verbose_ptxas): s for s, e in SOURCES.items()}
        objs, logs = [], []
        for f in futs:
            obj, log = f.result()
            objs.append(obj)
            logs.append(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose_ptxas:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose_ptxas="-v" in sys.argv))
