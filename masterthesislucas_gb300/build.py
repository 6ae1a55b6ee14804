"""Builds libtreecode.so (the CUDA kernels and the C ABI) in-tree for sm_103a.

Every translation unit is compiled by nvcc in parallel and linked into
``masterthesislucas_gb300/libtreecode.so``.  tree.cu is compiled without FMA
contraction so that the FP64 tree build rounds exactly like the reference.
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
LIB = os.path.join(PKG, "libtreecode.so")
BUILD = os.path.join(PKG, "_build")

# longest compiles first
SOURCES = ["fmm_p.cu", "lists.cu", "fmm.cu", "tree.cu", "tree_p.cu", "bh.cu", "pm.cu", "tsne.cu", "learned.cu",
           "mlp.cu", "direct.cu", "integrate.cu", "affinity.cu", "sort.cu", "scan.cu", "api.cu"]
# FP64 tree build and the affinity matrix: operations in a fixed, stated form (fused only where written)
NO_FMA = {"tree.cu", "affinity.cu"}
# FP32 force kernels: denormals flushed (squared distances never reach them) so
# that rsqrt/reciprocal map to single SFU instructions
FTZ = {"fmm.cu", "fmm_p.cu", "tree_p.cu"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# fmm_p.cu is compiled once per expansion order (each object holds one order's
# kernels) and once for the order switch, so the orders compile in parallel
ORDERS = (12, 10, 8, 6, 4, 3)
OBJECTS = {"fmm_p.cu": [(f"fmm_p_o{p}.o", [f"-DTC_FMM_ORDER={p}"]) for p in ORDERS] + [("fmm_p.o", [])]}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(src: str) -> list:
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                "--expt-relaxed-constexpr"]
    if src in NO_FMA:
        f.append("-fmad=false")
    if src in FTZ:
        f.append("-ftz=true")
    # extra nvcc flags for every translation unit (tuning builds, e.g. -DTC_NEAR_MIN_WARPS=40)
    f += os.environ.get("TREECODE_NVCC_FLAGS", "").split()
    return f


def _stale(out: str, deps: list) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "treecode.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        for name, defs in OBJECTS.get(s, [(s.replace(".cu", ".o"), [])]):
            obj = os.path.join(BUILD, name)
            objs.append(obj)
            if force or _stale(obj, [src] + headers):
                jobs.append([cc, "-c", src, "-o", obj] + _flags(s) + defs)
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose and (res.stdout or res.stderr):
                sys.stderr.write(res.stdout + res.stderr)
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if force or _stale(LIB, objs):
        cmd = [cc, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
