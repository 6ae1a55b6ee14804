"""Learned expansion-order controller: data generation and training (host side).

The network and its training run in libtreecode's own kernels (csrc/mlp.cu);
the error samples come from the method itself (csrc/learned.cu): for node
pairs drawn from the candidate lists of order-12 solves on independently
seeded systems, the pair's far-field force error at orders 4, 6, 8, 10, 12 is
measured against the direct sum over the source node's particles.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import datasets
from ._lib import check, lib, ptr
from .solver import NBodySolverFMM_SYM_MORTON

ORDERS = (4, 6, 8, 10, 12)
NPARAM = 5573


class OrderController:
    """The 16 -> 64 -> 64 -> 5 MLP (BF16 weights, FP32 accumulation) on the GPU."""

    def __init__(self, seed: int = 0):
        self._m = ctypes.c_void_p()
        check(lib().tc_mlp_create(ctypes.c_uint64(seed), ctypes.byref(self._m)))
        self.mean = np.zeros(16, np.float32)
        self.std = np.ones(16, np.float32)

    def close(self):
        if self._m:
            lib().tc_mlp_destroy(self._m)
            self._m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_normalization(self, mean, std):
        self.mean = np.ascontiguousarray(mean, np.float32)
        self.std = np.ascontiguousarray(np.maximum(std, 1e-6), np.float32)
        check(lib().tc_mlp_set_normalization(self._m, ptr(self.mean), ptr(self.std)))

    def params(self) -> np.ndarray:
        p = np.zeros(NPARAM, np.float32)
        check(lib().tc_mlp_get_params(self._m, ptr(p), None, None))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().tc_mlp_set_params(self._m, ptr(p)))

    def gradient(self, X_d, T_d):
        g = np.zeros(NPARAM, np.float32)
        loss = ctypes.c_float(0)
        check(lib().tc_mlp_gradient(self._m, ptr(X_d), ptr(T_d), X_d.shape[0], ptr(g), ctypes.byref(loss)))
        return g, float(loss.value)

    def train(self, X_d, T_d, steps: int, batch: int = 4096, lr: float = 2e-3, seed: int = 0) -> float:
        loss = ctypes.c_float(0)
        check(lib().tc_mlp_train(self._m, ptr(X_d), ptr(T_d), X_d.shape[0], steps, batch, ctypes.c_float(lr),
                                 ctypes.c_uint64(seed), ctypes.byref(loss)))
        return float(loss.value) / (batch * len(ORDERS))

    def predict_tc(self, X_d):
        """The list builder's tensor-core evaluation (BF16 inputs and activations)."""
        import torch
        Y = torch.empty((X_d.shape[0], len(ORDERS)), dtype=torch.float32, device=X_d.device)
        check(lib().tc_mlp_forward_tc(self._m, ptr(X_d), X_d.shape[0], ptr(Y)))
        return Y

    def predict(self, X_d):
        import torch
        Y = torch.empty((X_d.shape[0], len(ORDERS)), dtype=torch.float32, device=X_d.device)
        check(lib().tc_mlp_forward(self._m, ptr(X_d), X_d.shape[0], ptr(Y)))
        return Y

    def save(self, path):
        np.savez(path, params=self.params(), mean=self.mean, std=self.std, orders=np.array(ORDERS))

    @classmethod
    def load(cls, path):
        z = np.load(path)
        c = cls()
        c.set_params(z["params"])
        c.set_normalization(z["mean"], z["std"])
        return c


def sample_pairs(solver: NBodySolverFMM_SYM_MORTON, per_level: int, rng, min_level: int = 2):
    """Candidate pairs (level, sink, source) drawn from the accepted and near lists."""
    out = []
    d = solver.depth()
    for level in range(min_level, d + 1):
        nl = 4 ** level
        for kind in (0, 1):
            ptr_h = np.zeros(nl + 1, np.uint32)
            tot = ctypes.c_int64(0)
            check(lib().tc_get_list(solver._h, level, kind, ptr(ptr_h), None, ctypes.byref(tot)))
            if tot.value == 0:
                continue
            idx_h = np.zeros(tot.value, np.uint32)
            check(lib().tc_get_list(solver._h, level, kind, ptr(ptr_h), ptr(idx_h), ctypes.byref(tot)))
            k = min(per_level, tot.value)
            e = rng.choice(tot.value, k, replace=False)
            sink = np.searchsorted(ptr_h, e, side="right") - 1
            src = idx_h[e]
            keep = sink != src
            out.append(np.stack([np.full(keep.sum(), level), sink[keep], src[keep]], 1))
    return np.concatenate(out).astype(np.int32) if out else np.zeros((0, 3), np.int32)


def generate(n_systems: int = 4, n_particles: int = 1 << 20, kernel: str = "gravity", per_level: int = 20000,
             theta_gen: float = 1.6, seed: int = 0, depth_offset: int = 2, leaf: int = 64):
    """Features and log10 errors from independently seeded systems (GPU)."""
    import torch

    rng = np.random.default_rng(seed)
    feats, errs = [], []
    for k in range(n_systems):
        sd = int(rng.integers(1 << 30))
        if kernel == "gravity":
            pos = (datasets.two_disks(n_particles, seed=sd) if k % 2 == 0 else
                   datasets.gaussian_mixture(n_particles, seed=sd)).astype(np.float64)
        else:
            pos = np.random.default_rng(sd).normal(0.0, 10.0 * (1 + k), (n_particles, 2))
        from .solver import get_depth
        depth = min(14, get_depth(leaf, n_particles) + depth_offset)
        s = NBodySolverFMM_SYM_MORTON(kernel, max_children=leaf, tree_depth=depth, theta=theta_gen,
                                      softening=1e-3, order=12)
        pos_d = torch.from_numpy(pos).cuda()
        g = torch.zeros_like(pos_d)
        t = torch.zeros(1, dtype=torch.float64, device="cuda")
        s.update_tree_device(pos_d)
        s.solve_device(g, t)
        pairs = sample_pairs(s, per_level, rng)
        pd = torch.from_numpy(pairs).cuda()
        F = torch.zeros((len(pairs), 16), dtype=torch.float32, device="cuda")
        E = torch.zeros((len(pairs), 5), dtype=torch.float32, device="cuda")
        check(lib().tc_lc_pair_errors(s._h, ptr(pd), len(pairs), ptr(F), ptr(E)))
        feats.append(F.cpu().numpy())
        errs.append(E.cpu().numpy())
        s.close()
    return np.concatenate(feats), np.concatenate(errs)


def fit(X, T, *, steps=3000, batch=4096, lr=2e-3, seed=0, holdout=0.1):
    """Trains an OrderController; returns it with train/holdout mean-squared errors."""
    import torch

    rng = np.random.default_rng(seed)
    n = len(X)
    perm = rng.permutation(n)
    nh = int(n * holdout)
    hold, tr = perm[:nh], perm[nh:]
    c = OrderController(seed)
    c.set_normalization(X[tr].mean(0), X[tr].std(0))
    Xd = torch.from_numpy(np.ascontiguousarray(X[tr])).cuda()
    Td = torch.from_numpy(np.ascontiguousarray(T[tr])).cuda()
    c.train(Xd, Td, steps=steps, batch=batch, lr=lr, seed=seed)
    ph = c.predict(torch.from_numpy(np.ascontiguousarray(X[hold])).cuda()).cpu().numpy()
    pt = c.predict(Xd[:200000]).cpu().numpy()
    mse_h = float(((ph - T[hold]) ** 2).mean()) if nh else float("nan")
    mse_t = float(((pt - T[tr][:200000]) ** 2).mean())
    return c, {"train_mse": mse_t, "holdout_mse": mse_h, "n_train": len(tr), "n_holdout": nh}


class CheckedSolve:
    """The learned-order solve with the plain fixed-order FMM as fallback and
    judge.  After each learned solve the forces on n_check seeded sample
    particles are compared with an FP32 direct sum over all particles (the
    library's tc_direct_device); when their median relative error exceeds tol
    the step is recomputed by the plain solver into the same outputs.  Both
    solvers must use the same kernel and softening; they run on their own
    streams, and step() synchronises the device before it decides.

    step() returns the sampled median error of the learned solve; `recomputed`
    counts the steps the plain FMM redid.  The median over n_check samples is
    an estimate: at 4M particles 32 samples misjudged a solve of median error
    8.8e-5 as above 1e-4; 64 cost 0.55 ms per check on a GB300."""

    def __init__(self, learned_solver, plain_solver, n, *, kernel="gravity", softening=1e-3, tol=1e-4,
                 n_check=256, seed=0, device=0):
        import torch
        self.learned, self.plain = learned_solver, plain_solver
        self.kernel = 1 if kernel == "gravity" else 0
        self.softening, self.tol = float(softening), float(tol)
        rows = np.sort(np.random.default_rng(seed).choice(n, min(n_check, n), replace=False)).astype(np.int64)
        self.rows = torch.from_numpy(rows).to(torch.device("cuda", device))
        self.ref = torch.zeros((len(rows), 2), dtype=torch.float64, device=self.rows.device)
        self.n = n
        self.recomputed = 0
        self.steps = 0

    def sampled_error(self, pos_d, grad_d) -> float:
        import torch
        check(lib().tc_direct_device(self.kernel, self.softening, 0, ptr(pos_d), self.n, ptr(self.rows),
                                     len(self.rows), ptr(self.ref), None, None))
        torch.cuda.synchronize()
        g = grad_d[self.rows]
        e = torch.linalg.norm(g - self.ref, dim=1) / torch.linalg.norm(self.ref, dim=1)
        return float(torch.median(e).item())

    def check_async(self, pos_d, grad_d, err_out, stream):
        """Enqueues the sampled-error check of a learned solve on `stream`
        (a torch.cuda.Stream) without synchronising the host: the median
        relative error lands in the device scalar err_out.  The caller reads
        the errors later and redoes the failed steps with the plain FMM."""
        import torch
        check(lib().tc_direct_device(self.kernel, self.softening, 0, ptr(pos_d), self.n, ptr(self.rows),
                                     len(self.rows), ptr(self.ref), None, ctypes.c_void_p(stream.cuda_stream)))
        with torch.cuda.stream(stream):
            g = grad_d[self.rows]
            e = torch.linalg.norm(g - self.ref, dim=1) / torch.linalg.norm(self.ref, dim=1)
            err_out.copy_(torch.median(e))

    def judge(self, pos_d, grad_d, tot_d) -> float:
        """Checks a learned solve already written to grad_d / tot_d (for
        instance by a captured step) and redoes it with the plain FMM when the
        sampled error exceeds the tolerance; returns the sampled error."""
        import torch
        self.steps += 1
        torch.cuda.synchronize()
        err = self.sampled_error(pos_d, grad_d)
        if not err <= self.tol:  # NaN recomputes too
            self.plain.update_tree_device(pos_d)
            self.plain.solve_device(grad_d, tot_d, accumulate=False, scatter=True)
            torch.cuda.synchronize()
            self.recomputed += 1
        return err

    def step(self, pos_d, grad_d, tot_d) -> float:
        """One learned solve, judged."""
        self.learned.update_tree_device(pos_d)
        self.learned.solve_device(grad_d, tot_d, accumulate=False, scatter=True)
        return self.judge(pos_d, grad_d, tot_d)
