"""The GPU affinity build (csrc/affinity.cu) against the oracle's CPU
restatement, bit for bit: kNN distances and indices, the calibrated rows
and the symmetric CSR (k = 90, perplexity 30 as openTSNE's defaults for the
reference's P files), including inputs with duplicate points (distance ties)."""
import numpy as np
import pytest
import torch

import oracle
from masterthesislucas_gb300 import affinity, datasets

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,dim,clusters,dups", [(3000, 64, 6, False), (1500, 784, 10, False), (1200, 16, 3, True)])
def test_affinity_bit_exact_against_oracle(n, dim, clusters, dups):
    x, _ = datasets.cluster_data(n, dim, k=clusters, seed=n)
    if dups:
        x[1::7] = x[0::7][: len(x[1::7])]  # exact duplicates: zero distances and ties
    xt = torch.from_numpy(x).cuda()
    d_g, i_g = affinity.knn(xt, 90)
    d_o, i_o = oracle.knn(x, 90)
    np.testing.assert_array_equal(d_g.cpu().numpy(), d_o)
    np.testing.assert_array_equal(i_g.cpu().numpy(), i_o)
    p_g = affinity.perplexity_rows(d_g, 30.0)
    p_o = oracle.perplexity_rows(d_o, 30.0)
    np.testing.assert_array_equal(p_g.cpu().numpy(), p_o)
    rp_g, col_g, val_g = affinity.symmetrize(i_g, p_g)
    rp_o, col_o, val_o = oracle.symmetrize(i_o, p_o)
    np.testing.assert_array_equal(rp_g, rp_o)
    np.testing.assert_array_equal(col_g, col_o)
    np.testing.assert_array_equal(val_g, val_o)


def test_build_p_csr_is_the_composition():
    x, _ = datasets.cluster_data(2000, 32, k=5, seed=9)
    rp, col, val = affinity.build_p_csr(x, perplexity=30.0)
    ro, co, vo = oracle.affinity_csr(x, perplexity=30.0)
    np.testing.assert_array_equal(rp, ro)
    np.testing.assert_array_equal(col, co)
    np.testing.assert_array_equal(val, vo)
    assert val.sum() == pytest.approx(1.0, rel=1e-12)
