"""GPU particle-mesh (FFT-accelerated interpolation) t-SNE repulsion against the
reference's NBodySolverPM outputs (golden fixtures made by the reference built
with a plain-DFT stand-in for FFTW) and against the exact direct sum.

Contract: same grid (boxes, nodes, the reference's min/max quirk), so the
gradient and the pair sum agree with the reference to FFT rounding: relative
1e-10 of the largest gradient component, 1e-11 on the pair sum."""
import numpy as np
import pytest

from masterthesislucas_gb300 import NBodySolverPM, Points, direct, particle_mesh
from masterthesislucas_gb300._lib import TreecodeError

pytestmark = pytest.mark.gpu

CASES = ["pm_gauss_2000", "pm_wide_3000", "pm_small_cells_500", "pm_coarse_1000", "pm_tiny_17",
         "pm_first_min_800"]


@pytest.mark.parametrize("case", CASES)
def test_pm_matches_reference(golden, case):
    g = golden(case)
    grad, total = particle_mesh(g["pos"], n_interp=int(g["n_interp"]), cell_size=float(g["cell_size"]),
                                min_intervals=int(g["min_intervals"]))
    scale = np.abs(g["grad"]).max()
    assert np.abs(grad - g["grad"]).max() <= 1e-10 * scale
    assert total == pytest.approx(float(g["total"]), rel=1e-11)


def test_pm_interface_overwrites_like_the_reference(golden):
    g = golden("pm_gauss_2000")
    pts = Points.from_positions(g["pos"])
    pts.derivative[:] = 123.0  # overwritten, not accumulated
    s = NBodySolverPM(4, 1.0, 4)
    s.updateTree(pts)
    total = s.solveNbody(0.0, pts)
    assert np.abs(pts.derivative - g["grad"]).max() <= 1e-10 * np.abs(g["grad"]).max()
    assert total == pytest.approx(float(g["total"]), rel=1e-11)


def test_pm_accuracy_against_direct_sum():
    """The scheme's own error at the reference's settings (4 nodes, unit boxes)
    and its convergence with smaller boxes."""
    pos = np.random.default_rng(5).normal(0.0, 6.0, (20000, 2))
    rows = np.arange(0, 20000, 7)
    fd, _ = direct(pos, kernel="tsne", precision="fp64", rows=rows)
    _, zd = direct(pos, kernel="tsne", precision="fp64")
    meds = []
    for cell in (2.0, 1.0, 0.5):
        g, z = particle_mesh(pos, cell_size=cell)
        e = np.linalg.norm(g[rows] - fd, axis=1) / np.linalg.norm(fd, axis=1)
        meds.append(float(np.median(e)))
        assert z == pytest.approx(zd, rel=1e-3)
    print(meds)
    assert meds[0] > meds[1] > meds[2]
    assert meds[1] < 1e-2


def test_pm_rejects_bad_input():
    pos = np.random.default_rng(1).normal(size=(100, 2))
    with pytest.raises(TreecodeError):
        particle_mesh(pos, n_interp=0)
    with pytest.raises(TreecodeError):
        particle_mesh(pos, cell_size=0.0)
    bad = pos.copy()
    bad[3, 1] = np.inf
    with pytest.raises(TreecodeError):
        particle_mesh(bad)
    # usable afterwards
    g, _ = particle_mesh(pos)
    assert np.isfinite(g).all()


def test_tsne_step_with_particle_mesh_repulsion(golden):
    """The device t-SNE step with the reference's default repulsion (nBodySelect
    "PM"): gradient (4/Z) * repulsion + attraction and the momentum update,
    against the oracle's particle mesh and attractive term."""
    import oracle
    from masterthesislucas_gb300.tsne import TSNE
    g = golden("tsne_step_600")
    exag = float(g["exag_code"])
    lr = float(g["lr"])
    t = TSNE(g["row_ptr"], g["col"], g["val"], g["y0"], early_exaggeration=exag / 4.0, precision="fp64",
             learn_rate=lr, repulsion="pm", cell_size=1.0)
    z = t.time_step(with_z=True)
    y, yp, grad = t.embedding()
    rep, zr = oracle.pm(g["y0"], cell_size=1.0)
    expect = rep * (4.0 / zr)
    oracle.tsne_attractive(np.ascontiguousarray(g["row_ptr"], np.uint32), np.ascontiguousarray(g["col"], np.uint32),
                           np.ascontiguousarray(g["val"], np.float64), np.ascontiguousarray(g["y0"]), exag, expect)
    assert z == pytest.approx(zr, rel=1e-10)
    assert np.abs(grad - expect).max() <= 1e-8 * np.abs(expect).max()
    np.testing.assert_allclose(y, g["y0"] + lr * expect, rtol=0, atol=1e-8 * np.abs(g["y0"]).max())
    with pytest.raises(ValueError):
        TSNE(g["row_ptr"], g["col"], g["val"], g["y0"], repulsion="fmm")
