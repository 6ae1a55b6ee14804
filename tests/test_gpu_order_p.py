"""Order-p FMM: the error against FP64 direct sums falls with the expansion
order at a fixed opening angle, for both kernels (the only oracle at
arbitrary order is the direct sum; order 3 is the reference's truncation)."""
import numpy as np
import pytest

from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON, Points, datasets, direct

pytestmark = pytest.mark.gpu


def errors(pos, kernel, theta, orders, depth, rows, fd, leaf=16):
    out = {}
    for p in orders:
        s = NBodySolverFMM_SYM_MORTON(kernel, max_children=leaf, tree_depth=depth, theta=theta, softening=1e-3,
                                      order=p)
        pts = Points.from_positions(pos)
        s.updateTree(pts, pos.min(0), pos.max(0))
        total = s.solveNbody(0.0, pts)
        g = np.zeros_like(pos)
        g[pts.ID] = pts.derivative
        e = np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1)
        out[p] = (float(np.median(e)), total)
    return out


@pytest.mark.parametrize("kernel", ["gravity", "tsne"])
def test_error_falls_with_order(kernel):
    n = 65536
    if kernel == "gravity":
        pos = datasets.two_disks(n, seed=11).astype(np.float64)
    else:
        pos = np.random.default_rng(12).normal(0.0, 10.0, (n, 2))
    rows = np.random.default_rng(0).choice(n, 1024, replace=False)
    fd, _ = direct(pos, kernel=kernel, softening=1e-3, precision="fp64", rows=rows)
    _, ztot = direct(pos, kernel=kernel, softening=1e-3, precision="fp64")
    e = errors(pos, kernel, 0.6, (3, 4, 6, 8, 10, 12), 8, rows, fd)
    meds = [e[p][0] for p in (3, 4, 6, 8, 10, 12)]
    print(kernel, meds)
    assert meds[0] > meds[2] > meds[3] > meds[5]
    assert meds[5] < 1e-5
    # the pair sum converges to the direct one
    assert e[12][1] == pytest.approx(ztot, rel=1e-4)


def test_tsne_repulsion_order_p_normalised_gradient():
    n = 30000
    pos = np.random.default_rng(3).normal(0.0, 5.0, (n, 2))
    rows = np.arange(0, n, 37)
    fd, zd = direct(pos, kernel="tsne", precision="fp64", rows=rows)
    _, z_all = direct(pos, kernel="tsne", precision="fp64")
    s = NBodySolverFMM_SYM_MORTON("tsne", max_children=16, theta=0.5, order=8)
    pts = Points.from_positions(pos)
    s.updateTree(pts, pos.min(0), pos.max(0))
    z = s.solveNbody(0.0, pts)
    assert z == pytest.approx(z_all, rel=1e-5)
    g = np.zeros_like(pos)
    g[pts.ID] = pts.derivative
    e = np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1)
    assert np.median(e) < 1e-5


@pytest.mark.parametrize("kernel", ["gravity", "tsne"])
def test_bounding_radius_mac_converges(kernel):
    """TC_MAC_BMAX: (b_A + b_B)/theta < |dcom| with b the nodes' bounding
    radii about their COMs; the error falls with theta and with the order."""
    n = 65536
    if kernel == "gravity":
        pos = datasets.two_disks(n, seed=21).astype(np.float64)
    else:
        pos = np.random.default_rng(22).normal(0.0, 10.0, (n, 2))
    rows = np.random.default_rng(1).choice(n, 1024, replace=False)
    fd, _ = direct(pos, kernel=kernel, softening=1e-3, precision="fp64", rows=rows)
    meds = {}
    for theta, p in [(0.8, 8), (0.6, 8), (0.4, 8), (0.6, 12)]:
        s = NBodySolverFMM_SYM_MORTON(kernel, max_children=16, tree_depth=8, theta=theta, softening=1e-3, order=p,
                                      mac="bmax")
        pts = Points.from_positions(pos)
        s.updateTree(pts, pos.min(0), pos.max(0))
        s.solveNbody(0.0, pts)
        g = np.zeros_like(pos)
        g[pts.ID] = pts.derivative
        meds[(theta, p)] = float(np.median(np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1)))
        s.close()
    print(kernel, meds)
    assert meds[(0.8, 8)] > meds[(0.6, 8)] > meds[(0.4, 8)]
    assert meds[(0.6, 12)] < meds[(0.6, 8)]
    assert meds[(0.4, 8)] < 1e-5


def test_bounding_radius_mac_needs_order_p():
    from masterthesislucas_gb300._lib import TreecodeError
    with pytest.raises(TreecodeError):
        NBodySolverFMM_SYM_MORTON("tsne", mac="bmax")


@pytest.mark.parametrize("order", [8, 12])
def test_adaptive_order_keeps_the_error_of_fixed_order(order):
    """bmax_adaptive: accepted pairs at the lowest order whose bound stays
    below slack times the fixed-order one; at slack 0.01 the error stays
    within a small factor of the fixed-order error at the same theta."""
    n = 65536
    pos = datasets.two_disks(n, seed=31).astype(np.float64)
    rows = np.random.default_rng(2).choice(n, 1024, replace=False)
    fd, _ = direct(pos, kernel="gravity", softening=1e-3, precision="fp64", rows=rows)
    meds = {}
    for mac in ("bmax", "bmax_adaptive"):
        s = NBodySolverFMM_SYM_MORTON("gravity", max_children=16, tree_depth=8, theta=0.7, softening=1e-3,
                                      order=order, mac=mac, slack=0.01)
        pts = Points.from_positions(pos)
        s.updateTree(pts, pos.min(0), pos.max(0))
        s.solveNbody(0.0, pts)
        g = np.zeros_like(pos)
        g[pts.ID] = pts.derivative
        meds[mac] = float(np.median(np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1)))
        s.close()
    print(order, meds)
    assert meds["bmax_adaptive"] < 1.5 * meds["bmax"]


def test_leaf_p2p_switch_is_at_least_as_accurate():
    """tc_set_leaf_p2p: accepted leaf pairs with few particle pairs are summed
    directly; fewer M2L pairs, more P2P pairs, and no loss of accuracy."""
    n = 65536
    pos = datasets.two_disks(n, seed=41).astype(np.float64)
    rows = np.random.default_rng(3).choice(n, 1024, replace=False)
    fd, _ = direct(pos, kernel="gravity", softening=1e-3, precision="fp64", rows=rows)
    out = {}
    for cut in (0, 64):
        s = NBodySolverFMM_SYM_MORTON("gravity", max_children=16, tree_depth=9, theta=0.7, softening=1e-3, order=8,
                                      mac="bmax", leaf_p2p=cut)
        pts = Points.from_positions(pos)
        s.updateTree(pts, pos.min(0), pos.max(0))
        s.solveNbody(0.0, pts)
        g = np.zeros_like(pos)
        g[pts.ID] = pts.derivative
        out[cut] = (float(np.median(np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1))), s.counters())
        s.close()
    print(out)
    assert out[64][1]["m2l"] < out[0][1]["m2l"] and out[64][1]["p2p_pairs"] > out[0][1]["p2p_pairs"]
    assert out[64][0] <= out[0][0] * 1.05
    from masterthesislucas_gb300._lib import TreecodeError
    with pytest.raises(TreecodeError):
        NBodySolverFMM_SYM_MORTON("tsne", leaf_p2p=64)  # reference order keeps its interaction set


@pytest.mark.parametrize("mac", ["cell", "bmax"])
def test_deep_tree_uses_both_level_kernels(mac):
    """A depth-10 tree runs the coarse-level kernels (a warp per node for the
    lists and the M2L, four lanes per node for the M2M, levels <= 8) and the
    fine-level ones (a thread per node, levels 9-10) in one solve; the forces
    must meet the accuracy the same settings reach on shallow trees."""
    n = 262144
    pos = datasets.two_disks(n, seed=51).astype(np.float64)
    rows = np.random.default_rng(4).choice(n, 2048, replace=False)
    fd, _ = direct(pos, kernel="gravity", softening=1e-3, precision="fp64", rows=rows)
    theta = 1.0 if mac == "cell" else 0.7
    s = NBodySolverFMM_SYM_MORTON("gravity", max_children=16, tree_depth=10, theta=theta, softening=1e-3, order=10,
                                  mac=mac, leaf_p2p=64)
    pts = Points.from_positions(pos)
    s.updateTree(pts, pos.min(0), pos.max(0))
    s.solveNbody(0.0, pts)
    g = np.zeros_like(pos)
    g[pts.ID] = pts.derivative
    err = np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1)
    print(mac, np.median(err), np.percentile(err, 99))
    assert np.median(err) < 5e-5
    assert np.percentile(err, 99) < 2e-3
    c = s.counters()
    assert c["m2l"] > 0 and c["p2p_pairs"] > 0


@pytest.mark.parametrize("kernel", ["gravity", "tsne"])
def test_box_centred_expansions_converge(kernel):
    """Expansions about the cell centre (the dipole kept, the bounding-radius
    criterion measured from the cell centre): the error against the FP64
    direct sum falls with the order and the pair sum converges, as for the
    expansions about the centre of mass."""
    n = 65536
    if kernel == "gravity":
        pos = datasets.two_disks(n, seed=11).astype(np.float64)
    else:
        pos = np.random.default_rng(12).normal(0.0, 10.0, (n, 2))
    rows = np.random.default_rng(0).choice(n, 1024, replace=False)
    fd, _ = direct(pos, kernel=kernel, softening=1e-3, precision="fp64", rows=rows)
    _, ztot = direct(pos, kernel=kernel, softening=1e-3, precision="fp64")
    meds, tots = [], []
    for p in (4, 8, 12):
        s = NBodySolverFMM_SYM_MORTON(kernel, max_children=16, tree_depth=8, theta=0.6, softening=1e-3, order=p,
                                      mac="bmax", centre="box")
        pts = Points.from_positions(pos)
        s.updateTree(pts, pos.min(0), pos.max(0))
        tots.append(s.solveNbody(0.0, pts))
        g = np.zeros_like(pos)
        g[pts.ID] = pts.derivative
        meds.append(float(np.median(np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1))))
        s.close()
    print(kernel, meds)
    assert meds[0] > meds[1] > meds[2]
    assert meds[2] < 1e-5
    assert tots[2] == pytest.approx(ztot, rel=1e-4)
