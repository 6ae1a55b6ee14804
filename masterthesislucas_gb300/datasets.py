"""Seeded synthetic inputs with the shapes of the benchmark workloads.

The reference's datasets (MNIST digits/fashion, CIFAR10, 10x mouse brain) and
its openTSNE-built affinity files are not available, so every workload here is
generated from a seed:

* ``gaussian_mixture`` -- 2D mixture of ``k`` clusters, centres U[-1,1]^2,
  sigma ~ U[0.02, 0.2], equal weights (Barnes-Hut gravity workload).
* ``two_disks``        -- two exponential disks (scale lengths 0.1 and 0.05,
  centres 0.6 apart, half the particles each) (large FMM workload).
* ``cluster_data``     -- high-dimensional Gaussian clusters clipped to [0,1]
  (input of the t-SNE affinity build).
* ``tsne_init``        -- N(0, sigma^2) initial embedding, as
  ``TSNE::generateInitialPoints`` (src/nBodyInstances/tsne.h:522-562) draws it.
"""
from __future__ import annotations

import numpy as np


def gaussian_mixture(n: int, k: int = 8, seed: int = 0, dtype=np.float32) -> np.ndarray:
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-1.0, 1.0, (k, 2))
    sigmas = rng.uniform(0.02, 0.2, k)
    lab = rng.integers(0, k, n)
    pos = centres[lab] + rng.normal(size=(n, 2)) * sigmas[lab, None]
    return pos.astype(dtype)


def two_disks(n: int, seed: int = 0, scales=(0.1, 0.05), separation: float = 0.6,
              dtype=np.float32) -> np.ndarray:
    rng = np.random.default_rng(seed)
    n0 = n // 2
    out = np.empty((n, 2), np.float64)
    for (lo, hi), s, cx in (((0, n0), scales[0], -separation / 2),
                            ((n0, n), scales[1], separation / 2)):
        m = hi - lo
        r = rng.gamma(2.0, s, m)          # surface density ~ exp(-r/s)
        phi = rng.uniform(0.0, 2 * np.pi, m)
        out[lo:hi, 0] = cx + r * np.cos(phi)
        out[lo:hi, 1] = r * np.sin(phi)
    return out.astype(dtype)


def cluster_data(n: int, dim: int, k: int = 10, seed: int = 0, spread: float = 0.15) -> tuple:
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, (k, dim)).astype(np.float32)
    lab = rng.integers(0, k, n)
    x = centres[lab] + rng.normal(0.0, spread, (n, dim)).astype(np.float32)
    np.clip(x, 0.0, 1.0, out=x)
    return x.astype(np.float32), lab.astype(np.uint8)


def tsne_init(n: int, seed: int = 0, sigma: float = 0.01) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.normal(0.0, sigma, (n, 2))
