"""Builds libphoton_cuda.so in-tree for sm_103a with nvcc.

Every translation unit compiles in parallel into photon_gb300/_build/, then
links into photon_gb300/libphoton_cuda.so.  Device code is compiled with
--fmad=false so float expressions round like the reference's (no implicit
multiply-add contraction); the traversal kernels use explicit fmaf where
contraction is wanted.  Host code uses -ffp-contract=off for the same reason
(the aarch64 host compiler contracts by default).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libphoton_cuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    p = shutil.which("nvcc")
    if p:
        return p
    p = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(p):
        return p
    raise RuntimeError("nvcc not found")


def sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, f))
    return out


def _compile(src, extra, verbose):
    nvcc = nvcc_path()
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "photon_cuda.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp", "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc] + ARCH + common + ["-lineinfo", "--fmad=false", "-c", src, "-o", obj] + extra
    else:
        cmd = [nvcc] + common + ["-x", "c++", "-c", src, "-o", obj] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, (r.stdout + r.stderr) if verbose else ""


def build(force: bool = False, verbose: bool = False, extra=()):
    """Compiles all sources (incrementally) and links the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra), verbose), srcs))
    objs = [o for o, _ in results]
    logs = "".join(l for _, l in results)
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc_path()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB, logs


if __name__ == "__main__":
    import sys
    lib, logs = build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                      extra=["-Xptxas", "-v"] if "-v" in sys.argv else [])
    print(logs)
    print(lib)
