"""Matrix Market reader/writer for P against scipy's independent implementation."""
import os

import numpy as np
import pytest

import oracle
from masterthesislucas_gb300 import datasets, mtx


def dense(rp, col, val, n):
    d = np.zeros((n, n))
    for i in range(n):
        d[i, col[rp[i]:rp[i + 1]]] += val[rp[i]:rp[i + 1]]
    return d


def test_round_trip_is_exact(tmp_path):
    x, _ = datasets.cluster_data(400, 8, k=4, seed=3)
    rp, col, val = oracle.affinity_csr(x, perplexity=10.0)
    p = os.path.join(tmp_path, "P.mtx")
    mtx.write_p_matrix(p, rp, col, val, comment="test")
    rp2, col2, val2 = mtx.read_p_matrix(p)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2) and np.array_equal(val, val2)


def test_symmetric_file_expands_and_transposes(tmp_path):
    p = os.path.join(tmp_path, "S.mtx")
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n% lower triangle\n4 4 5\n")
        f.write("2 1 0.25\n3 1 0.125\n3 2 0.5\n4 4 0.75\n4 2 1.5\n")
    rp, col, val = mtx.read_p_matrix(p)
    d = dense(rp, col, val, 4)
    ref = np.zeros((4, 4))
    for r, c, v in [(1, 0, 0.25), (2, 0, 0.125), (2, 1, 0.5), (3, 3, 0.75), (3, 1, 1.5)]:
        ref[r, c] = v
        ref[c, r] = v
    assert np.array_equal(d, ref)
    for i in range(4):
        assert np.all(np.diff(col[rp[i]:rp[i + 1]].astype(np.int64)) > 0)


def test_general_file_matches_scipy_transpose(tmp_path):
    sio = pytest.importorskip("scipy.io")
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(0)
    a = sp.random(30, 30, density=0.2, random_state=1, format="coo")
    p = os.path.join(tmp_path, "G.mtx")
    sio.mmwrite(p, a, symmetry="general")
    rp, col, val = mtx.read_p_matrix(p)
    # setupEfficientPmatrix stores the transpose of what the file holds
    assert np.allclose(dense(rp, col, val, 30), a.toarray().T, rtol=0, atol=0)


def test_malformed_files_are_rejected(tmp_path):
    p = os.path.join(tmp_path, "bad.mtx")
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 0.5\n4 1 0.5\n")
    with pytest.raises(ValueError):
        mtx.read_p_matrix(p)
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(ValueError):
        mtx.read_p_matrix(p)
