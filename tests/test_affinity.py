"""The t-SNE affinity matrix builder (kNN + perplexity calibration +
symmetrisation, the openTSNE recipe the reference's P files come from)."""
import numpy as np
import pytest
import torch

from masterthesislucas_gb300 import affinity, datasets


def test_p_is_symmetric_normalised_and_sorted():
    x, _ = datasets.cluster_data(600, 8, k=4, seed=2)
    rp, col, val = affinity.build_p_csr(x, perplexity=10.0, device="cpu")
    n = len(x)
    assert rp[0] == 0 and rp[-1] == len(col) and np.all(np.diff(rp.astype(np.int64)) > 0)
    assert val.sum() == pytest.approx(1.0, rel=1e-12)
    dense = np.zeros((n, n))
    for i in range(n):
        cols = col[rp[i]:rp[i + 1]]
        assert np.all(np.diff(cols.astype(np.int64)) > 0)  # columns sorted within a row
        dense[i, cols] = val[rp[i]:rp[i + 1]]
    assert np.allclose(dense, dense.T, rtol=0, atol=1e-18)
    assert np.all(np.diag(dense) == 0.0)


def test_row_perplexity_is_calibrated():
    x, _ = datasets.cluster_data(800, 8, k=3, seed=4)
    d2, idx = affinity.knn(torch.from_numpy(x), 30)
    p = affinity.perplexity_rows(d2, 10.0).numpy()
    h = -(p * np.log(np.maximum(p, 1e-300))).sum(1)
    assert np.allclose(np.exp(h), 10.0, rtol=1e-3)


@pytest.mark.gpu
def test_device_symmetrisation_matches_host():
    x, _ = datasets.cluster_data(3000, 16, k=6, seed=7)
    xt = torch.from_numpy(x)
    d2, idx = affinity.knn(xt, 45)
    p = affinity.perplexity_rows(d2, 15.0)
    host = affinity._symmetrize_host(p.numpy(), idx.numpy(), len(x))
    dev = affinity._symmetrize_device(p.cuda(), idx.cuda(), len(x))
    for a, b in zip(host, dev):
        assert np.array_equal(a, b)
