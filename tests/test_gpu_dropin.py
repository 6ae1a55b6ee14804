"""The drop-in adaptor (include/gpu_tree_solver.hpp) run on the GPU: a C++
program holds GpuTreeSolver<TsnePoint2D> through the NBodySolver<T>* interface
the reference's drivers use (compiled against a stand-in of that interface,
tests/dropin/nbody_interface.hpp, since the reference's sources are not on the
GPU machine), calls updateTree + solveNbody + getNodesBufferData, and its
reordered points, forces and pair sum are checked against the oracle's
restatement of NBodySolverFMM_SYM_MORTON on the same points."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from masterthesislucas_gb300 import datasets

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dropin_adaptor_through_the_solver_interface(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    pkg = os.path.join(ROOT, "masterthesislucas_gb300")
    exe = str(tmp_path / "dropin_gpu")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "tests", "dropin"), os.path.join(ROOT, "tests", "dropin", "dropin_gpu.cpp"),
                        "-o", exe, "-L" + pkg, "-ltreecode", "-Wl,-rpath," + pkg], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n = 20000
    pos = np.random.default_rng(216308).normal(0.0, 3.0, (n, 2))
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        f.write(np.int64(n).tobytes())
        f.write(np.ascontiguousarray(pos, np.float64).tobytes())
    r = subprocess.run([exe, fin, fout, "16", "0.5"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(fout, "rb").read()
    ids = np.frombuffer(raw, np.int32, n)
    off = 4 * n
    p_sorted = np.frombuffer(raw, np.float64, 2 * n, off).reshape(n, 2)
    off += 16 * n
    grad = np.frombuffer(raw, np.float64, 2 * n, off).reshape(n, 2)
    off += 16 * n
    total, nverts = np.frombuffer(raw, np.float64, 1, off)[0], np.frombuffer(raw, np.int64, 1, off + 8)[0]
    ref = oracle.sym_fmm(pos, kernel=oracle.KERNEL_TSNE, max_children=16, theta=0.5)
    # the vector comes back in the reference's Morton order, records moved whole
    assert np.array_equal(ids, ref["ids"])
    assert np.array_equal(p_sorted, ref["pos"])
    # FP64 handle: the reference's forces and pair sum
    rel = np.linalg.norm(grad - ref["grad"], axis=1) / np.linalg.norm(ref["grad"], axis=1)
    assert rel.max() < 1e-9
    assert total == pytest.approx(ref["total"], rel=1e-10)
    # getNodesBufferData(-1): four line segments (eight vertices) per non-empty node of every level
    assert nverts == 8 * int((ref["nodes"]["count"] > 0).sum())
