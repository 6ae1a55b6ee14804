"""Regenerates the golden fixtures in this folder from the reference itself.

The reference's CPU solvers are compiled from the reference sources by
oracle/Makefile.ref (oracle/_ref/libref_oracle.so) and run here on seeded
synthetic inputs; their outputs are the fixtures.  The reference's ``TSNE``
class cannot be linked (it constructs the FFTW-based PM solver), so the t-SNE
step fixture composes the reference's own repulsion solver with a numpy
restatement of updateRepulsive / updateAttractive / updatePoints
(src/nBodyInstances/tsne.h:287-301, :356-381, :179-206).

Run from the repo root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from masterthesislucas_gb300 import datasets  # noqa: E402
from masterthesislucas_gb300.affinity import build_p_csr  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"{name}: {os.path.getsize(path) / 1024:.1f} KiB")


def sym_case(name, pos, *, kernel=0, eps=0.0, max_children=16, depth=-1, theta=0.5, symmetric=True):
    pos = np.ascontiguousarray(pos, np.float64)
    mn, mx = oracle.bbox(pos)
    r = oracle.ref_sym_fmm(pos, kernel=kernel, eps=eps, max_children=max_children, depth=depth,
                           theta=theta, mn=mn, mx=mx, symmetric=symmetric)
    save(name, pos=pos, minmax=np.concatenate([mn, mx]), kernel=kernel, eps=eps,
         max_children=max_children, depth=r["depth"], theta=theta, codes=r["codes"], ids=r["ids"],
         pos_sorted=r["pos"], grad=r["grad"], total=r["total"], nodes=r["nodes"])


def tsne_step_case(name, n=600, dim=16, steps=3, seed=21, theta=0.5, exag_code=16.0, perplexity=10.0):
    x, _ = datasets.cluster_data(n, dim, k=5, seed=seed)
    row_ptr, col, val = build_p_csr(x, perplexity=perplexity)
    y0 = datasets.tsne_init(n, seed=seed)
    lr = n / 15.0
    ys = [y0, y0]  # y_prev, y
    grads, zs = [], []
    for it in range(steps):
        y_prev, y = ys[-2], ys[-1]
        mn, mx = oracle.bbox(y)
        r = oracle.ref_sym_fmm(y, kernel=0, max_children=16, depth=-1, theta=theta, mn=mn, mx=mx)
        z = r["total"]
        g = np.zeros_like(y)
        g[r["ids"]] = r["grad"] * (4.0 / z)
        for i in range(n):  # updateAttractive
            ax = ay = 0.0
            for k in range(row_ptr[i], row_ptr[i + 1]):
                c = col[k]
                dx = y[c, 0] - y[i, 0]
                dy = y[c, 1] - y[i, 1]
                q = 1.0 / (1.0 + (dx * dx + dy * dy))
                ax += exag_code * val[k] * q * dx
                ay += exag_code * val[k] * q * dy
            g[i, 0] += ax
            g[i, 1] += ay
        mom = 0.5
        ys.append(y + lr * g + mom * (y - y_prev))
        grads.append(g)
        zs.append(z)
    save(name, row_ptr=row_ptr, col=col, val=val, y0=y0, ys=np.stack(ys[2:]), grads=np.stack(grads),
         zs=np.array(zs), theta=theta, exag_code=exag_code, lr=lr, momentum=0.5,
         perplexity=perplexity)


def asym_cases():
    """The non-symmetric NBodySolverFMM_MORTON (gravity put in its kernel slots)."""
    sym_case("asym_grav_mixture_4096", datasets.gaussian_mixture(4096, seed=6), kernel=1, eps=1e-3,
             symmetric=False)
    sym_case("asym_tsne_deep_2000_theta1", np.random.default_rng(15).uniform(-5, 5, (2000, 2)), depth=5,
             theta=1.0, symmetric=False)
    sym_case("asym_tsne_tiny_17", np.random.default_rng(117).normal(0, 1, (17, 2)), symmetric=False)


def bhmp_cases():
    """NBodySolverBHMP: Barnes-Hut with quadrupoles (gravity put in its slots)."""
    for kernel, eps, tag in ((0, 0.0, "tsne"), (1, 1e-3, "grav")):
        pos = datasets.gaussian_mixture(3000, seed=33).astype(np.float64)
        g, t = oracle.ref_bhmp(pos, kernel=kernel, eps=eps, max_children=16, theta=0.5)
        save(f"bhmp_{tag}_3000", pos=pos, grad=g, total=t, kernel=kernel, eps=eps, max_children=16, theta=0.5)


def pm_cases():
    """NBodySolverPM: FFT-accelerated interpolation repulsion (the reference built with
    oracle/fftw_stub.cpp in place of FFTW).  The first point of pm_first_min_800 is the
    smallest coordinate, which the reference's min/max pass never takes for the minimum."""
    rng = np.random.default_rng(21)
    cases = [("pm_gauss_2000", rng.normal(0, 3, (2000, 2)), 1.0, 4),
             ("pm_wide_3000", rng.normal(0, 8, (3000, 2)), 1.0, 4),
             ("pm_small_cells_500", rng.normal(0, 1, (500, 2)), 0.3, 4),
             ("pm_coarse_1000", rng.normal(0, 20, (1000, 2)), 2.0, 4),
             ("pm_tiny_17", rng.normal(0, 0.5, (17, 2)), 1.0, 4)]
    first_min = rng.normal(0, 2, (800, 2))
    first_min[0] = first_min.min() - 1.0
    cases.append(("pm_first_min_800", first_min, 1.0, 4))
    for name, pos, cell, mn in cases:
        pos = np.ascontiguousarray(pos, np.float64)
        g, t = oracle.ref_pm(pos, n_interp=4, cell_size=cell, min_intervals=mn)
        save(name, pos=pos, grad=g, total=t, n_interp=4, cell_size=cell, min_intervals=mn)


def main():
    if oracle.build_ref() is None:
        raise SystemExit("reference sources not found; fixtures cannot be regenerated")
    rng = np.random.default_rng(11)
    sym_case("sym_tsne_gauss_3000", rng.normal(0, 3, (3000, 2)))
    sym_case("sym_grav_mixture_4096", datasets.gaussian_mixture(4096, seed=5), kernel=1, eps=1e-3)
    base = np.random.default_rng(12).normal(0, 1, (600, 2))
    ties = np.concatenate([base, base[:400]])
    sym_case("sym_tsne_ties_1000", ties)
    sym_case("sym_tsne_deep_2000_theta1", np.random.default_rng(13).uniform(-5, 5, (2000, 2)),
             depth=5, theta=1.0)
    sym_case("sym_grav_disks_3000_theta03", datasets.two_disks(3000, seed=14), kernel=1, eps=1e-3,
             theta=0.3, max_children=8)
    for n in (2, 3, 17, 64):
        sym_case(f"sym_tsne_tiny_{n}", np.random.default_rng(100 + n).normal(0, 1, (n, 2)))
    sym_case("asym_tsne_gauss_3000", rng.normal(0, 3, (3000, 2)), symmetric=False)
    asym_cases()
    for kernel, eps, tag in ((0, 0.0, "tsne"), (1, 1e-3, "grav")):
        pos = datasets.gaussian_mixture(1500, seed=31).astype(np.float64)
        g, t = oracle.ref_naive(pos, kernel=kernel, eps=eps)
        save(f"naive_{tag}_1500", pos=pos, grad=g, total=t, kernel=kernel, eps=eps)
        pos = datasets.gaussian_mixture(3000, seed=32).astype(np.float64)
        g, t = oracle.ref_bh(pos, kernel=kernel, eps=eps, max_children=16, theta=0.5)
        save(f"bh_{tag}_3000", pos=pos, grad=g, total=t, kernel=kernel, eps=eps, max_children=16,
             theta=0.5)
    bhmp_cases()
    pm_cases()
    tsne_step_case("tsne_step_600")


if __name__ == "__main__":
    main()
