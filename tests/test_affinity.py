"""The t-SNE affinity matrix: the CPU restatement in the oracle (the GPU
kernels are checked against it bit for bit in test_gpu_affinity.py) -- exact
kNN, perplexity calibration, the symmetric CSR layout of
setupEfficientPmatrix (rows sorted, columns sorted within a row), and the
oracle's own exp/log against the C library's."""
import ctypes
import math

import numpy as np
import pytest

import oracle
from masterthesislucas_gb300 import _lib, datasets


def test_series_exp_and_log_within_an_ulp_or_two():
    L = oracle.lib()
    xs = np.concatenate([-np.logspace(-12, 2.8, 500), np.linspace(-700.0, 5.0, 1001)])
    for x in xs:
        assert abs(L.orc_exp(float(x)) - math.exp(x)) <= 4.5e-16 * math.exp(x)
    for y in np.concatenate([np.logspace(-300, 300, 601), np.linspace(0.5, 3.0, 501)]):
        ref = math.log(y)
        assert abs(L.orc_log(float(y)) - ref) <= 4.5e-16 * max(abs(ref), 1.0)


def test_knn_matches_brute_force():
    x, _ = datasets.cluster_data(700, 12, k=4, seed=3)
    d, i = oracle.knn(x, 25)
    full = ((x[:, None, :].astype(np.float64) - x[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(full, np.inf)
    ref = np.sort(full, axis=1)[:, :25]
    np.testing.assert_allclose(d, ref, rtol=1e-5, atol=1e-6)
    assert np.all(np.diff(d, axis=1) >= 0)
    assert np.all(i != np.arange(len(x))[:, None])


def test_p_is_symmetric_normalised_and_sorted():
    x, _ = datasets.cluster_data(600, 8, k=4, seed=2)
    rp, col, val = oracle.affinity_csr(x, perplexity=10.0)
    n = len(x)
    assert rp[0] == 0 and rp[-1] == len(col) and np.all(np.diff(rp.astype(np.int64)) > 0)
    assert val.sum() == pytest.approx(1.0, rel=1e-12)
    dense = np.zeros((n, n))
    for r in range(n):
        cols = col[rp[r]:rp[r + 1]]
        assert np.all(np.diff(cols.astype(np.int64)) > 0)  # columns sorted within a row
        dense[r, cols] = val[rp[r]:rp[r + 1]]
    assert np.allclose(dense, dense.T, rtol=0, atol=1e-18)
    assert np.all(np.diag(dense) == 0.0)


def test_row_perplexity_is_calibrated():
    x, _ = datasets.cluster_data(800, 8, k=3, seed=4)
    d, _ = oracle.knn(x, 30)
    p = oracle.perplexity_rows(d, 10.0)
    assert np.allclose(p.sum(1), 1.0, rtol=1e-12)
    h = -(p * np.log(np.maximum(p, 1e-300))).sum(1)
    assert np.allclose(np.exp(h), 10.0, rtol=1e-3)


def test_entry_points_reject_invalid_arguments_before_any_launch():
    L = _lib.lib()
    fake = ctypes.c_void_p(256)
    assert L.tc_knn_device(fake, 100, 8, 129, fake, fake, None) == -1  # k above the kernel's 128
    assert L.tc_knn_device(fake, 10, 8, 10, fake, fake, None) == -1    # k must be below n
    assert L.tc_perplexity_device(fake, 100, 30, 1.0, 100, 1e-5, fake, None) == -1
    nnz = ctypes.c_int64(0)
    assert L.tc_symmetrize_device(None, fake, 100, 30, fake, fake, fake, ctypes.byref(nnz), None) == -1
