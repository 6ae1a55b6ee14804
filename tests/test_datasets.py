"""The seeded synthetic workloads that stand in for the reference's datasets:
deterministic per seed, with the stated shapes and distributions."""
import numpy as np

from masterthesislucas_gb300 import datasets


def test_two_disks_is_seeded_and_has_the_stated_profile():
    n = 200000
    a = datasets.two_disks(n, seed=4)
    np.testing.assert_array_equal(a, datasets.two_disks(n, seed=4))
    assert not np.array_equal(a, datasets.two_disks(n, seed=5))
    assert a.shape == (n, 2) and a.dtype == np.float32
    p = datasets.two_disks(n, seed=4, dtype=np.float64)
    for half, scale, cx in ((p[: n // 2], 0.1, -0.3), (p[n // 2:], 0.05, 0.3)):
        r = np.hypot(half[:, 0] - cx, half[:, 1])
        # surface density ~ exp(-r/s): r ~ Gamma(2, s), mean 2s, variance 2s^2
        assert abs(r.mean() - 2 * scale) < 5 * scale * np.sqrt(2.0 / len(r))
        assert abs(half[:, 1].mean()) < 0.01


def test_gaussian_mixture_and_cluster_data():
    g = datasets.gaussian_mixture(50000, k=8, seed=1)
    np.testing.assert_array_equal(g, datasets.gaussian_mixture(50000, k=8, seed=1))
    assert g.shape == (50000, 2) and np.isfinite(g).all()
    assert np.abs(g).max() < 1.0 + 6 * 0.2  # centres in [-1, 1]^2, sigma <= 0.2
    x, lab = datasets.cluster_data(3000, 16, k=6, seed=2)
    assert x.shape == (3000, 16) and x.dtype == np.float32 and lab.dtype == np.uint8
    assert x.min() >= 0.0 and x.max() <= 1.0 and set(np.unique(lab)) <= set(range(6))


def test_tsne_init_matches_the_reference_scale():
    y = datasets.tsne_init(100000, seed=3)
    assert y.shape == (100000, 2)
    assert abs(y.std() - 0.01) < 1e-3 and abs(y.mean()) < 1e-3
