"""CPU oracle of the controller network: the numpy backward pass agrees with
central finite differences (FP64), which pins the reference the GPU training
kernels are checked against (tests/test_gpu_learned.py)."""
import numpy as np

from oracle.mlp_reference import NPARAM, reference_loss_grad


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, NPARAM)
    X = rng.normal(0, 1, (40, 16))
    T = rng.normal(0, 1, (40, 5))
    mean, std = np.zeros(16), np.ones(16)
    loss, g = reference_loss_grad(p, X, T, mean, std, round_weights=False)
    idx = rng.choice(NPARAM, 60, replace=False)
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (reference_loss_grad(pp, X, T, mean, std, round_weights=False)[0] -
              reference_loss_grad(pm, X, T, mean, std, round_weights=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
