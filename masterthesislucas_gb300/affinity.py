"""Perplexity-calibrated kNN affinities (the t-SNE P matrix) as CSR.

The reference reads P from Matrix Market files written offline by openTSNE
(``MnistLoader.ipynb`` cell 14: PCA(50) -> PerplexityBasedNN(perplexity,
k = 3*perplexity, symmetrize=True) -> mmwrite) and converts them to CSR in
``TSNE::setupEfficientPmatrix`` (src/nBodyInstances/tsne.h:462-520: rows
sorted, columns sorted within a row).  openTSNE and the data files are not
available, so this module restates the published algorithm: exact kNN on
squared Euclidean distances, per-point binary search of the Gaussian
precision to the target perplexity, symmetrisation P = (P + P^T) / (2N).
The affinity values are therefore not pinned to the reference's files.

Setup code (not timed): it runs with torch on whatever device is given.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def knn(x: torch.Tensor, k: int, block: int = 4096):
    """Exact k nearest neighbours (self excluded) by blocked squared distances."""
    n = x.shape[0]
    x = x.float()
    sq = (x * x).sum(1)
    d_out = torch.empty(n, k, device=x.device)
    i_out = torch.empty(n, k, dtype=torch.int64, device=x.device)
    for s in range(0, n, block):
        e = min(n, s + block)
        d = sq[s:e, None] + sq[None, :] - 2.0 * (x[s:e] @ x.T)
        d[torch.arange(e - s, device=x.device), torch.arange(s, e, device=x.device)] = float("inf")
        vals, idx = torch.topk(d, k, dim=1, largest=False)
        d_out[s:e] = vals.clamp_min(0.0)
        i_out[s:e] = idx
    return d_out, i_out


def perplexity_rows(d2: torch.Tensor, perplexity: float, iters: int = 100, tol: float = 1e-5):
    """Binary search of beta_i so that H(P_i) = log(perplexity); rows sum to 1."""
    d2 = d2.double()
    n = d2.shape[0]
    target = math.log(perplexity)
    beta = torch.ones(n, dtype=torch.float64, device=d2.device)
    lo = torch.zeros_like(beta)
    hi = torch.full_like(beta, float("inf"))
    dmin = d2[:, :1]
    for _ in range(iters):
        w = torch.exp(-(d2 - dmin) * beta[:, None])
        s = w.sum(1)
        p = w / s[:, None]
        h = torch.log(s) + beta * ((d2 - dmin) * p).sum(1)
        diff = h - target
        if float(diff.abs().max()) < tol:
            break
        up = diff > 0
        lo = torch.where(up, beta, lo)
        hi = torch.where(up, hi, beta)
        beta = torch.where(torch.isinf(hi), beta * 2.0, (lo + hi) / 2.0)
    w = torch.exp(-(d2 - dmin) * beta[:, None])
    return w / w.sum(1, keepdim=True)


def build_p_csr(x, perplexity: float = 30.0, k: int | None = None, device=None):
    """Symmetric affinity matrix P (sums to 1) as CSR: (row_ptr u32, col u32, val f64)."""
    if k is None:
        k = int(3 * perplexity)
    xt = torch.as_tensor(np.asarray(x), device=device or "cpu")
    n = xt.shape[0]
    k = min(k, n - 1)
    d2, idx = knn(xt, k)
    if xt.is_cuda:
        return _symmetrize_device(perplexity_rows(d2, perplexity), idx, n)
    return _symmetrize_host(perplexity_rows(d2, perplexity).cpu().numpy(), idx.cpu().numpy(), n)


def _symmetrize_host(p: np.ndarray, idx: np.ndarray, n: int):
    """(P + P^T) / (2N) as CSR (rows and columns sorted), on the host."""
    k = idx.shape[1]
    rows = np.repeat(np.arange(n, dtype=np.int64), k)
    cols = idx.reshape(-1)
    vals = p.reshape(-1)
    # symmetrise: (P + P^T) / (2N)
    r2 = np.concatenate([rows, cols])
    c2 = np.concatenate([cols, rows])
    v2 = np.concatenate([vals, vals]) * (1.0 / (2.0 * n))  # as the device path scales
    key = r2 * n + c2
    order = np.argsort(key, kind="stable")
    key = key[order]
    v2 = v2[order]
    uniq, start = np.unique(key, return_index=True)
    vsum = np.add.reduceat(v2, start)
    r = (uniq // n).astype(np.int64)
    c = (uniq % n).astype(np.uint32)
    row_ptr = np.zeros(n + 1, np.uint32)
    np.add.at(row_ptr, r + 1, 1)
    row_ptr = np.cumsum(row_ptr).astype(np.uint32)
    return row_ptr, c, vsum.astype(np.float64)


def _symmetrize_device(p: torch.Tensor, idx: torch.Tensor, n: int):
    """(P + P^T) / (2N) as CSR, on the GPU (each entry sums at most two
    values, so the result does not depend on the summation order)."""
    k = idx.shape[1]
    dev = idx.device
    rows = torch.arange(n, device=dev, dtype=torch.int64).repeat_interleave(k)
    cols = idx.reshape(-1).to(torch.int64)
    vals = p.reshape(-1).to(torch.float64)
    key = torch.cat([rows * n + cols, cols * n + rows])
    v2 = torch.cat([vals, vals]) * (1.0 / (2.0 * n))
    key, order = torch.sort(key, stable=True)
    v2 = v2[order]
    uniq, counts = torch.unique_consecutive(key, return_counts=True)
    seg = torch.repeat_interleave(torch.arange(len(uniq), device=dev), counts)
    vsum = torch.zeros(len(uniq), dtype=torch.float64, device=dev).index_add_(0, seg, v2)
    r = uniq // n
    c = (uniq % n).to(torch.int32)
    row_ptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    row_ptr[1:] = torch.cumsum(torch.bincount(r, minlength=n), 0)
    return (row_ptr.cpu().numpy().astype(np.uint32), c.cpu().numpy().astype(np.uint32),
            vsum.cpu().numpy().astype(np.float64))
