"""The order-p path's tree against the reference's updateTree.

The order-p solve (the path the benchmark times) keeps the reference's tree:
Morton codes (createMortonCode, nBodySolverFMM_SYM_MORTON.h:538-561), the
permutation of the code sort (:89; stable, so ties keep input order) and the
topology and boxes of createLeafNodes / bottomUpNodeConstruction (:328-470):
BBcentre, BBlength, firstChildIndex, firstParticleIndex, particleIndexAmount
and M0 bit-exact.  Its moments are the physical (mass-weighted) FP32 ones, so
centres of mass are checked to FP32 accuracy relative to the box size.

Cases: the 4,194,304-particle two-disk workload at the depth the benchmark
runs (11) and at the reference's own depth rule (9), through the host entry
point and through the device entry point with the box computed on the GPU;
a 70,000-point clustered embedding at leaf 16 (the t-SNE step's tree).
"""
import numpy as np
import pytest

import oracle
from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON, Points, datasets

pytestmark = pytest.mark.gpu


def _positions(case):
    if case == "two_disks_4m":
        return datasets.two_disks(4194304, seed=1000).astype(np.float64), "gravity", 64
    # a clustered 2D embedding of 70,000 points (10 clusters), the t-SNE step's input shape
    return 20.0 * datasets.gaussian_mixture(70000, k=10, seed=11).astype(np.float64), "tsne", 16


def _check(d, ref, depth):
    np.testing.assert_array_equal(d["codes"], ref["codes"])
    np.testing.assert_array_equal(d["perm"], ref["ids"])
    np.testing.assert_array_equal(d["pos"], ref["pos"])
    nodes = d["nodes"]
    rn = ref["nodes"]
    np.testing.assert_array_equal(nodes[:, 0:2], rn["bb_c"], err_msg="BBcentre")
    np.testing.assert_array_equal(nodes[:, 2], rn["bb_len"], err_msg="BBlength")
    np.testing.assert_array_equal(nodes[:, 3], rn["first_child"], err_msg="firstChildIndex")
    np.testing.assert_array_equal(nodes[:, 4], rn["first_part"], err_msg="firstParticleIndex")
    np.testing.assert_array_equal(nodes[:, 5], rn["count"], err_msg="particleIndexAmount")
    np.testing.assert_array_equal(nodes[:, 8], rn["m0"], err_msg="M0")
    nz = rn["count"] > 0
    # centre of mass: FP32 cell-relative sums, within 1e-5 of the node's box length
    dc = np.abs(nodes[nz, 6:8] - rn["com"][nz]).max(axis=1) / rn["bb_len"][nz]
    assert dc.max() < 1e-5, dc.max()


@pytest.mark.parametrize("case,depth,order", [("two_disks_4m", 11, 8), ("two_disks_4m", None, 12),
                                              ("tsne_70k", None, 8)])
def test_order_p_tree_bit_exact(case, depth, order):
    pos, kernel, leaf = _positions(case)
    mn, mx = pos.min(0), pos.max(0)
    s = NBodySolverFMM_SYM_MORTON(kernel, max_children=leaf, tree_depth=depth, theta=0.5, order=order,
                                  softening=1e-3)
    d_used = oracle.get_depth(leaf, len(pos)) if depth is None else depth
    ref = oracle.build_tree(pos, depth=d_used, mn=mn, mx=mx)
    pts = Points.from_positions(pos)
    s.updateTree(pts, mn, mx)
    assert s.depth() == d_used
    _check(s.tree_dump(), ref, d_used)
    np.testing.assert_array_equal(pts.ID, ref["ids"])
    s.close()


def test_order_p_tree_device_entry_box_on_gpu():
    """The benchmark's call: positions resident on the device, box computed there."""
    import torch
    pos, kernel, leaf = _positions("two_disks_4m")
    ref = oracle.build_tree(pos, depth=11)
    s = NBodySolverFMM_SYM_MORTON(kernel, max_children=leaf, tree_depth=11, theta=0.75, order=8, mac="bmax",
                                  softening=1e-3)
    s.update_tree_device(torch.from_numpy(pos).cuda())
    _check(s.tree_dump(), ref, 11)
    s.close()
