"""Perplexity-calibrated kNN affinities (the t-SNE P matrix) as CSR, built on
the GPU by the library's kernels (csrc/affinity.cu).

The reference reads P from Matrix Market files written offline by openTSNE
(``MnistLoader.ipynb`` cell 14: PCA(50) -> PerplexityBasedNN(perplexity,
k = 3*perplexity, symmetrize=True) -> mmwrite) and converts them to CSR in
``TSNE::setupEfficientPmatrix`` (src/nBodyInstances/tsne.h:462-520: rows
sorted, columns sorted within a row).  openTSNE and the data files are not
available, so the published algorithm is restated: exact kNN on squared
Euclidean distances (FP32, summed over the dimensions in order), a per-point
bisection of the Gaussian precision to the target perplexity (FP64), and the
symmetrisation P = (P + P^T) / (2N).  The affinity values are therefore not
pinned to the reference's files; the kernels are pinned bit for bit to the
CPU restatement in the oracle.

Setup code (not timed): inputs are copied to the device with torch, which is
used for memory only.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib, ptr

MAX_K = 128


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the affinity build runs on the GPU (no CUDA device)")
    return torch


def knn(x, k: int, stream=None):
    """Exact k nearest neighbours (self excluded) of device float32 rows x (n x
    dim): (dist n x k float32, idx n x k int32) on the device, each row
    ordered by (squared distance, index)."""
    torch = _torch()
    x = x.contiguous()
    n, dim = x.shape
    d = torch.empty((n, k), dtype=torch.float32, device=x.device)
    i = torch.empty((n, k), dtype=torch.int32, device=x.device)
    check(lib().tc_knn_device(ptr(x), n, dim, k, ptr(d), ptr(i), stream))
    return d, i


def perplexity_rows(dist, perplexity: float, max_iter: int = 100, tol: float = 1e-5, stream=None):
    """Row-normalised Gaussian affinities (FP64, device) whose entropy is
    log(perplexity) to within tol, from the kNN distances."""
    torch = _torch()
    n, k = dist.shape
    p = torch.empty((n, k), dtype=torch.float64, device=dist.device)
    check(lib().tc_perplexity_device(ptr(dist.contiguous()), n, k, float(perplexity), int(max_iter), float(tol),
                                     ptr(p), stream))
    return p


def symmetrize(idx, p, stream=None):
    """(P + P^T) / (2N) as CSR on the host: (row_ptr u32, col u32, val f64)."""
    torch = _torch()
    n, k = idx.shape
    rp = torch.empty(n + 1, dtype=torch.int32, device=idx.device)
    col = torch.empty(2 * n * k, dtype=torch.int32, device=idx.device)
    val = torch.empty(2 * n * k, dtype=torch.float64, device=idx.device)
    nnz = ctypes.c_int64(0)
    check(lib().tc_symmetrize_device(ptr(idx.contiguous()), ptr(p.contiguous()), n, k, ptr(rp), ptr(col), ptr(val),
                                     ctypes.byref(nnz), stream))
    m = nnz.value
    return (rp.cpu().numpy().view(np.uint32).copy(), col[:m].cpu().numpy().view(np.uint32).copy(),
            val[:m].cpu().numpy().copy())


def build_p_csr(x, perplexity: float = 30.0, k: int | None = None, device="cuda", max_iter: int = 100,
                tol: float = 1e-5):
    """Symmetric affinity matrix P (sums to 1) as CSR: (row_ptr u32, col u32, val f64).

    x: n x dim input points (host array or device tensor).  k defaults to
    3 * perplexity, as openTSNE's PerplexityBasedNN."""
    torch = _torch()
    if k is None:
        k = int(3 * perplexity)
    xt = torch.as_tensor(np.asarray(x, np.float32) if not torch.is_tensor(x) else x, device=device)
    xt = xt.to(torch.float32).contiguous()
    n = xt.shape[0]
    k = min(k, n - 1)
    if k > MAX_K:
        raise ValueError(f"k = {k} exceeds the kNN kernel's {MAX_K} neighbours")
    d, i = knn(xt, k)
    p = perplexity_rows(d, perplexity, max_iter, tol)
    return symmetrize(i, p)
