"""GPU t-SNE step (tree repulsion + CSR attractive term + Z + momentum update)
against the reference's composition (golden fixture from the reference's own
repulsion solver, tests/golden/make_golden.py)."""
import numpy as np
import pytest

from masterthesislucas_gb300.tsne import TSNE

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol_g,tol_y", [("fp64", 1e-10, 1e-12), ("fp32", 2e-5, 1e-6)])
def test_tsne_steps_match_reference(golden, precision, tol_g, tol_y):
    g = golden("tsne_step_600")
    t = TSNE(g["row_ptr"], g["col"], g["val"], g["y0"], early_exaggeration=float(g["exag_code"]) / 4.0,
             min_theta=float(g["theta"]), max_theta=float(g["theta"]), precision=precision,
             learn_rate=float(g["lr"]))
    for it in range(len(g["zs"])):
        z = t.time_step(with_z=True)
        y, yp, grad = t.embedding()
        assert z == pytest.approx(float(g["zs"][it]), rel=max(tol_g, 1e-12))
        gref = g["grads"][it]
        err = np.linalg.norm(grad - gref, axis=1) / np.linalg.norm(gref, axis=1)
        assert np.median(err) < tol_g and err.max() < 50 * tol_g, (np.median(err), err.max())
        scale = np.abs(g["ys"][it]).max()
        assert np.abs(y - g["ys"][it]).max() < tol_y * scale * 10 ** it
    assert t.launches() > 0
