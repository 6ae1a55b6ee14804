"""Size-independent properties at larger N, checked against the oracle where it
finishes in seconds and against FP64 direct sums on sampled particles."""
import numpy as np
import pytest

import oracle
from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON, Points, datasets, direct

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel,n,leaf,theta", [("gravity", 262144, 64, 0.5), ("tsne", 200000, 16, 0.5)])
def test_large_tree_bit_exact_and_forces_match_oracle(kernel, n, leaf, theta):
    if kernel == "gravity":
        pos = datasets.two_disks(n, seed=3).astype(np.float64)
    else:
        pos = np.random.default_rng(4).normal(0.0, 20.0, (n, 2))
    mn, mx = pos.min(0), pos.max(0)
    k = oracle.KERNEL_GRAVITY if kernel == "gravity" else oracle.KERNEL_TSNE
    ref = oracle.sym_fmm(pos, kernel=k, eps=1e-3, max_children=leaf, theta=theta, mn=mn, mx=mx, want_nodes=False)
    s = NBodySolverFMM_SYM_MORTON(kernel, max_children=leaf, theta=theta, softening=1e-3)
    pts = Points.from_positions(pos)
    s.updateTree(pts, mn, mx)
    d = s.tree_dump()
    np.testing.assert_array_equal(d["codes"], ref["codes"])
    assert np.all(np.diff(d["codes"].astype(np.int64)) >= 0)
    np.testing.assert_array_equal(np.sort(d["perm"]), np.arange(n))
    np.testing.assert_array_equal(d["perm"], ref["ids"])
    total = s.solveNbody(0.0, pts)
    err = np.linalg.norm(pts.derivative - ref["grad"], axis=1) / np.linalg.norm(ref["grad"], axis=1)
    assert np.median(err) < 2e-6 and np.percentile(err, 99.9) < 1e-3, (np.median(err), err.max())
    assert total == pytest.approx(ref["total"], rel=2e-6)
    c = s.counters()
    assert c["p2p_pairs"] > 0 and c["m2l"] > 0


def test_error_against_fp64_direct_sum_shrinks_with_theta():
    n = 131072
    pos = datasets.two_disks(n, seed=9).astype(np.float64)
    rows = np.random.default_rng(1).choice(n, 2048, replace=False)
    fd, _ = direct(pos, kernel="gravity", softening=1e-3, precision="fp64", rows=rows)
    meds = []
    for theta in (0.6, 0.4, 0.25):
        s = NBodySolverFMM_SYM_MORTON("gravity", max_children=64, theta=theta, softening=1e-3)
        pts = Points.from_positions(pos)
        s.updateTree(pts, pos.min(0), pos.max(0))
        s.solveNbody(0.0, pts)
        g = np.zeros_like(pos)
        g[pts.ID] = pts.derivative
        e = np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1)
        meds.append(np.median(e))
    assert meds[0] > meds[1] > meds[2]
    assert meds[2] < 1e-4
