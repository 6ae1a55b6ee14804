"""GPU parity of the symmetric Morton FMM (and of the non-symmetric
FMM_MORTON variant) against the reference's own outputs.

Golden fixtures come from the reference's CPU solvers compiled from their
sources (tests/golden/make_golden.py).  Contract:
* Morton codes, permutation, sorted positions and node topology, boxes and
  moments (BBcentre, BBlength, firstChildIndex, firstParticleIndex,
  particleIndexAmount, centreOfMass, M0, M2): bit-exact;
* forces and Z in FP64 mode: relative 1e-10 (only the summation order and
  FMA contraction differ; the interaction set is the reference's);
* forces in FP32 mode (the product precision): per-particle relative error
  |g - g_ref| / |g_ref| with median <= 2e-6 and max <= 1e-3, Z within 2e-6.
"""
import numpy as np
import pytest

from masterthesislucas_gb300 import NBodySolverFMM_MORTON, NBodySolverFMM_SYM_MORTON, Points, datasets, direct
from masterthesislucas_gb300._lib import TreecodeError

pytestmark = pytest.mark.gpu

SYM_CASES = ["sym_tsne_gauss_3000", "sym_grav_mixture_4096", "sym_tsne_ties_1000",
             "sym_tsne_deep_2000_theta1", "sym_grav_disks_3000_theta03", "sym_tsne_tiny_2",
             "sym_tsne_tiny_3", "sym_tsne_tiny_17", "sym_tsne_tiny_64"]

# the non-symmetric NBodySolverFMM_MORTON
ASYM_CASES = ["asym_tsne_gauss_3000", "asym_grav_mixture_4096", "asym_tsne_deep_2000_theta1",
              "asym_tsne_tiny_17"]
ALL_CASES = SYM_CASES + ASYM_CASES

FP32_MEDIAN = 2e-6
FP32_MAX = 1e-3


def run_case(g, precision, case=""):
    kernel = "tsne" if int(g["kernel"]) == 0 else "gravity"
    cls = NBodySolverFMM_MORTON if case.startswith("asym") else NBodySolverFMM_SYM_MORTON
    s = cls(kernel, max_children=int(g["max_children"]), tree_depth=int(g["depth"]),
                                  theta=float(g["theta"]), softening=float(g["eps"]) or 1e-3,
                                  precision=precision)
    pts = Points.from_positions(g["pos"])
    s.updateTree(pts, g["minmax"][:2], g["minmax"][2:])
    dump = s.tree_dump()
    total = s.solveNbody(0.0, pts)
    nodes = s.tree_dump()["nodes"]
    return s, pts, dump, nodes, total


def rel_err(a, b):
    nb = np.linalg.norm(b, axis=1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(nb, 1e-300)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("case", ALL_CASES)
def test_tree_bit_exact(golden, case, precision):
    g = golden(case)
    s, pts, dump, _, _ = run_case(g, precision, case)
    np.testing.assert_array_equal(dump["codes"], g["codes"])
    np.testing.assert_array_equal(dump["perm"], g["ids"])
    np.testing.assert_array_equal(pts.ID, g["ids"])
    np.testing.assert_array_equal(dump["pos"], g["pos_sorted"])
    np.testing.assert_array_equal(pts.position, g["pos_sorted"])
    # BBcentre BBlength firstChild firstParticle count com M0 M2
    np.testing.assert_array_equal(dump["nodes"][:, :13], g["nodes"][:, :13])


@pytest.mark.parametrize("case", ALL_CASES)
def test_forces_fp64_match_reference(golden, case):
    g = golden(case)
    s, pts, _, nodes, total = run_case(g, "fp64", case)
    err = rel_err(pts.derivative, g["grad"])
    assert err.max() < 1e-10, err.max()
    assert total == pytest.approx(float(g["total"]), rel=1e-10)
    # final local expansions of the non-empty nodes (C1, C2, C3)
    nz = g["nodes"][:, 5] > 0
    c_ref = g["nodes"][nz, 13:]
    c_gpu = nodes[nz, 13:]
    scale = np.abs(c_ref).max(axis=1, keepdims=True) + 1e-300
    assert np.abs(c_gpu - c_ref).max() <= 1e-9 * scale.max() or np.all(np.abs(c_gpu - c_ref) <= 1e-9 * scale)


@pytest.mark.parametrize("case", ALL_CASES)
def test_forces_fp32_match_reference(golden, case):
    g = golden(case)
    s, pts, _, _, total = run_case(g, "fp32", case)
    if len(pts) < 3:
        np.testing.assert_allclose(pts.derivative, g["grad"], rtol=1e-5)
    err = rel_err(pts.derivative, g["grad"])
    assert np.median(err) <= FP32_MEDIAN, np.median(err)
    assert err.max() <= FP32_MAX, err.max()
    assert total == pytest.approx(float(g["total"]), rel=2e-6)


@pytest.mark.parametrize("tag", ["tsne", "grav"])
def test_direct_sum_matches_reference_naive(golden, tag):
    g = golden(f"naive_{tag}_1500")
    kernel = "tsne" if tag == "tsne" else "gravity"
    grad, total = direct(g["pos"], kernel=kernel, softening=float(g["eps"]) or 1e-3, precision="fp64")
    assert rel_err(grad, g["grad"]).max() < 1e-11
    assert total == pytest.approx(float(g["total"]), rel=1e-11)
    grad32, total32 = direct(g["pos"], kernel=kernel, softening=float(g["eps"]) or 1e-3, precision="fp32")
    assert np.median(rel_err(grad32, g["grad"])) < 1e-4
    rows = np.array([0, 7, 1499, 500])
    gr, _ = direct(g["pos"], kernel=kernel, softening=float(g["eps"]) or 1e-3, precision="fp64", rows=rows)
    assert rel_err(gr, g["grad"][rows]).max() < 1e-11


def test_invalid_inputs_are_rejected():
    s = NBodySolverFMM_SYM_MORTON("tsne")
    pts = Points.from_positions(np.random.default_rng(0).normal(size=(100, 2)))
    with pytest.raises(TreecodeError) as e:
        s.solveNbody(0.0, pts)
    assert e.value.code == -4  # no tree yet
    bad = Points.from_positions(pts.position.copy())
    bad.position[5, 0] = np.nan
    with pytest.raises(TreecodeError) as e:
        s.updateTree(bad, [-5, -5], [5, 5])
    assert e.value.code == -1
    outside = Points.from_positions(pts.position.copy())
    with pytest.raises(TreecodeError) as e:
        s.updateTree(outside, outside.position.min(0) + 0.1, outside.position.max(0))
    assert e.value.code == -1
    with pytest.raises(TreecodeError):
        s.updateTree(pts, [0, 0], [0, 0])  # zero extent
    # the handle stays usable after rejected input
    s.updateTree(pts, pts.position.min(0), pts.position.max(0))
    s.solveNbody(0.0, pts)


def test_repeated_solves_are_deterministic():
    pos = np.random.default_rng(5).normal(0, 2, (20000, 2))
    s = NBodySolverFMM_SYM_MORTON("tsne", max_children=16, theta=0.5)
    outs = []
    for _ in range(2):
        pts = Points.from_positions(pos)
        s.updateTree(pts, pos.min(0), pos.max(0))
        t = s.solveNbody(0.0, pts)
        outs.append((pts.derivative.copy(), t))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    assert outs[0][1] == outs[1][1]


@pytest.mark.parametrize("tag", ["tsne", "grav"])
def test_barnes_hut_matches_reference(golden, tag):
    from masterthesislucas_gb300.solver import barnes_hut
    g = golden(f"bh_{tag}_3000")
    kernel = "tsne" if tag == "tsne" else "gravity"
    kw = dict(kernel=kernel, softening=float(g["eps"]) or 1e-3, max_children=int(g["max_children"]),
              theta=float(g["theta"]))
    grad, total = barnes_hut(g["pos"], precision="fp64", **kw)
    assert rel_err(grad, g["grad"]).max() < 1e-12
    assert total == pytest.approx(float(g["total"]), rel=1e-12)
    grad32, total32 = barnes_hut(g["pos"], precision="fp32", **kw)
    err = rel_err(grad32, g["grad"])
    assert np.median(err) < 1e-5 and err.max() < 1e-3
    assert total32 == pytest.approx(float(g["total"]), rel=1e-5)


@pytest.mark.parametrize("tag", ["tsne", "grav"])
def test_barnes_hut_multipole_matches_reference(golden, tag):
    from masterthesislucas_gb300.solver import barnes_hut
    g = golden(f"bhmp_{tag}_3000")
    kernel = "tsne" if tag == "tsne" else "gravity"
    kw = dict(kernel=kernel, softening=float(g["eps"]) or 1e-3, max_children=int(g["max_children"]),
              theta=float(g["theta"]), multipole=True)
    grad, total = barnes_hut(g["pos"], precision="fp64", **kw)
    assert rel_err(grad, g["grad"]).max() < 1e-12
    assert total == pytest.approx(float(g["total"]), rel=1e-12)
    grad32, total32 = barnes_hut(g["pos"], precision="fp32", **kw)
    err = rel_err(grad32, g["grad"])
    assert np.median(err) < 1e-5 and err.max() < 1e-3
    assert total32 == pytest.approx(float(g["total"]), rel=1e-5)
    # the quadrupole makes it more accurate than the monopole BH on the same tree
    bh, _ = barnes_hut(g["pos"], precision="fp64", **{**kw, "multipole": False})
    from masterthesislucas_gb300 import direct
    ref, _ = direct(g["pos"], kernel=kernel, softening=kw["softening"], precision="fp64")
    assert np.median(rel_err(grad, ref)) < np.median(rel_err(bh, ref))


def test_barnes_hut_large_matches_oracle():
    import oracle
    from masterthesislucas_gb300.solver import barnes_hut
    pos = datasets.gaussian_mixture(65536, seed=77).astype(np.float64)
    gref, tref = oracle.bh(pos, kernel=oracle.KERNEL_GRAVITY, eps=1e-3, max_children=16, theta=0.5)
    g, t = barnes_hut(pos, kernel="gravity", softening=1e-3, max_children=16, theta=0.5, precision="fp64")
    assert rel_err(g, gref).max() < 1e-11
    assert t == pytest.approx(tref, rel=1e-11)
