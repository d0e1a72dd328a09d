"""Build the CUDA library (sm_103a) in-tree: landslidehysea_gb300/liblsh.so.

nvcc only, no cmake: each translation unit is compiled in parallel and linked
into one shared library exporting the C ABI of include/lsh.h.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "liblsh.so")
BUILD_DIR = os.path.join(PKG, "_build")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale(srcs, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "lsh.h"))
    deps.append(os.path.join(ROOT, "include", "lsh_compat.h"))
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    srcs = sources()
    if not force and not _stale(srcs, LIB):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = nvcc_path()
    # --fmad=false: no implicit FMA contraction in device code; every fused
    # multiply-add is an explicit fma() that the CPU oracle performs too.
    # -ffp-contract=off: the same for host code (geometry, constants).
    common = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "-I", os.path.join(ROOT, "include"), *extra_flags]
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        cmd = common + ["-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(8, len(srcs)))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
