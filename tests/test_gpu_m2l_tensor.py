"""Tensor-core M2L (tcgen05, BF16 hi/lo split, FP32 accumulation in tensor
memory) against the FP32 SIMT M2L on the same box-centred expansions and
lists, and against the FP64 direct sum.

The two engines evaluate the same translations (M2L of the reference's
TSNE_FMM_SYM_MORTON_NN_Kernel, nBodySolverFMM_SYM_MORTON.h:622-723,
generalised to order p about cell centres); the tensor cores round their
operands to about 16 significant bits, so per-particle forces agree to a
relative 2e-5 (median) and the error against the direct sum stays within 20 %
(plus 2e-6) of the SIMT engine's: the rounding adds a few 1e-6 to a
truncation error of 1e-5 to 1e-4."""
import numpy as np
import pytest

from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON, Points, datasets, direct
from masterthesislucas_gb300._lib import TreecodeError

pytestmark = pytest.mark.gpu

MEDIAN_AGREE = 2e-5


def run(pos, kernel, order, theta, depth, m2l, mac="bmax"):
    s = NBodySolverFMM_SYM_MORTON(kernel, max_children=16, tree_depth=depth, theta=theta, softening=1e-3,
                                  order=order, mac=mac, centre="box", m2l=m2l)
    pts = Points.from_positions(pos)
    s.updateTree(pts, pos.min(0), pos.max(0))
    z = s.solveNbody(0.0, pts)
    g = np.zeros_like(pos)
    g[pts.ID] = pts.derivative
    c = s.counters()
    s.close()
    return g, z, c


def rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


@pytest.mark.parametrize("kernel,order,theta,depth", [("gravity", 8, 0.6, 8), ("tsne", 8, 0.5, 7),
                                                      ("gravity", 12, 0.7, 8), ("gravity", 4, 0.5, 7),
                                                      ("gravity", 10, 0.6, 9), ("tsne", 6, 0.45, 8)])
def test_tensor_m2l_matches_simt_and_direct(kernel, order, theta, depth):
    n = 65536
    if kernel == "gravity":
        pos = datasets.two_disks(n, seed=21).astype(np.float64)
    else:
        pos = np.random.default_rng(22).normal(0.0, 10.0, (n, 2))
    g_s, z_s, c_s = run(pos, kernel, order, theta, depth, "simt")
    g_t, z_t, c_t = run(pos, kernel, order, theta, depth, "tensor_all")
    assert c_t["m2l"] == c_s["m2l"] > 0 and c_t["p2p_pairs"] == c_s["p2p_pairs"]
    d = rel(g_t, g_s)
    print(kernel, order, "median", np.median(d), "max", d.max())
    assert np.median(d) < MEDIAN_AGREE and np.percentile(d, 99) < 20 * MEDIAN_AGREE
    assert z_t == pytest.approx(z_s, rel=1e-5)
    rows = np.random.default_rng(1).choice(n, 1024, replace=False)
    fd, _ = direct(pos, kernel=kernel, softening=1e-3, precision="fp64", rows=rows)
    e_s, e_t = np.median(rel(g_s[rows], fd)), np.median(rel(g_t[rows], fd))
    print("error vs direct: simt", e_s, "tensor", e_t)
    assert e_t <= 1.2 * e_s + 2e-6


def test_tensor_m2l_repeat_is_identical():
    """The tile sums run in a fixed order: two solves give the same bits."""
    pos = datasets.two_disks(32768, seed=5).astype(np.float64)
    g1, z1, _ = run(pos, "gravity", 8, 0.6, 8, "tensor_all")
    g2, z2, _ = run(pos, "gravity", 8, 0.6, 8, "tensor_all")
    assert np.array_equal(g1, g2) and z1 == z2


def test_tensor_m2l_on_the_deep_levels_only():
    """The default engine puts the levels with at least 128 parents per SM on
    the tensor cores (here levels 9 and 10) and keeps the coarse ones SIMT."""
    n = 262144
    pos = datasets.two_disks(n, seed=23).astype(np.float64)
    g_s, z_s, _ = run(pos, "gravity", 8, 0.7, 10, "simt")
    g_t, z_t, _ = run(pos, "gravity", 8, 0.7, 10, "tensor")
    d = rel(g_t, g_s)
    assert 0 < np.median(d) < MEDIAN_AGREE
    assert z_t == pytest.approx(z_s, rel=1e-5)


def test_tensor_m2l_rejects_angles_beyond_its_operator_table():
    pos = datasets.two_disks(4096, seed=6).astype(np.float64)
    s = NBodySolverFMM_SYM_MORTON("gravity", max_children=16, theta=0.1, order=8, mac="bmax", centre="box",
                                  m2l="tensor")
    pts = Points.from_positions(pos)
    s.updateTree(pts, pos.min(0), pos.max(0))
    with pytest.raises(TreecodeError):
        s.solveNbody(0.0, pts)
    s.close()
