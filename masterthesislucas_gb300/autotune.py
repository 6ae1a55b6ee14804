"""Autotuner for the order-p FMM: opening criterion, tree depth, opening angle
and expansion order (and, for the learned-order controller, tree depth and
tolerance tau).

For a given particle set (device-resident) it measures, for each candidate
(depth, theta, order), the device time of one updateTree + solveNbody (CUDA
events, after one warm-up) and the median relative force error against an
FP64 direct sum on sampled sinks, and returns the fastest candidate whose
error meets the target.  Candidates are visited from cheap to expensive and a
theta/order line stops once the error target is met (larger orders at the same
theta only cost more).
"""
from __future__ import annotations

import numpy as np

from .solver import NBodySolverFMM_SYM_MORTON, get_depth

ORDERS = (4, 6, 8, 10, 12)
THETAS = (1.6, 1.4, 1.3, 1.2, 1.1, 1.0, 0.9, 0.8, 0.7, 0.6, 0.5, 0.4)
# the bounding-radius criterion compares radii, not cell sizes: the expansions
# converge only below 1
THETAS_BMAX = (0.95, 0.9, 0.85, 0.8, 0.75, 0.7, 0.65, 0.6, 0.55, 0.5, 0.45, 0.4, 0.35, 0.3)
TAUS = (3e-3, 2e-3, 1e-3, 7e-4, 5e-4, 3e-4, 2e-4, 1e-4, 5e-5)


def median_error(grad_rows: np.ndarray, ref_rows: np.ndarray) -> float:
    e = np.linalg.norm(grad_rows - ref_rows, axis=1) / np.linalg.norm(ref_rows, axis=1)
    return float(np.median(e))


def tune(pos_d, ref_rows, rows_d, *, kernel: str, softening: float, leaf: int, target: float,
         stream=None, depths=None, thetas=None, orders=ORDERS, device: int = 0, log=None, macs=("cell",),
         leaf_p2p: int = 0, centre: str = "com", m2l: str = "simt"):
    """Returns (best, trials).  best = dict(mac, depth, theta, order, ms, err) or None."""
    import torch

    n = pos_d.shape[0]
    d0 = get_depth(leaf, n)
    depths = depths or (d0 + 1, d0 + 2, d0 + 3)
    grad_d = torch.zeros((n, 2), dtype=torch.float64, device=pos_d.device)
    tot_d = torch.zeros(1, dtype=torch.float64, device=pos_d.device)
    s_torch = torch.cuda.Stream(device=pos_d.device) if stream is None else stream
    trials = []
    best = None
    for mac, depth, order in [(m, d, o) for m in macs for d in depths for o in orders]:
        if depth > 15:
            continue
        # "bmax_adaptive:<slack>": the per-pair order rule with that slack
        kind, _, slack = mac.partition(":")
        if kind == "bmax_adaptive" and order < 6:
            continue
        for theta in thetas or (THETAS_BMAX if kind.startswith("bmax") else THETAS):
            s = NBodySolverFMM_SYM_MORTON(kernel, max_children=leaf, tree_depth=depth, theta=theta,
                                          softening=softening, precision="fp32", order=order,
                                          device=device, stream=s_torch.cuda_stream, mac=kind,
                                          slack=float(slack or 1.0), leaf_p2p=leaf_p2p, centre=centre, m2l=m2l)
            try:
                s.update_tree_device(pos_d)
                s.solve_device(grad_d, tot_d)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(s_torch)
                s.update_tree_device(pos_d)
                s.solve_device(grad_d, tot_d)
                e1.record(s_torch)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                err = median_error(grad_d[rows_d].cpu().numpy(), ref_rows)
            finally:
                s.close()
            t = dict(mac=mac, depth=depth, theta=theta, order=order, ms=ms, err=err, centre=centre, m2l=m2l)
            trials.append(t)
            if log:
                log(t)
            if err <= target:
                if best is None or ms < best["ms"]:
                    best = t
                break  # smaller theta at this order only costs more
    return best, trials


LEAF_P2P = (0, 16, 32, 64, 128, 256)


def refine_leaf_p2p(best, pos_d, ref_rows, rows_d, *, kernel: str, softening: float, leaf: int, target: float,
                    stream=None, device: int = 0, values=LEAF_P2P):
    """Second pass over the leaf-pair threshold at the chosen configuration:
    accepted leaf pairs with at most that many particle pairs are summed
    directly (trading M2L + L2P work for near-field pairs, which moves the
    balance between the tensor-free FP32 near field and the expansions).
    Returns (best with its leaf_p2p, trials)."""
    import torch

    n = pos_d.shape[0]
    grad_d = torch.zeros((n, 2), dtype=torch.float64, device=pos_d.device)
    tot_d = torch.zeros(1, dtype=torch.float64, device=pos_d.device)
    s_torch = torch.cuda.Stream(device=pos_d.device) if stream is None else stream
    kind, _, slack = best["mac"].partition(":")
    out, trials = dict(best), []
    for v in values:
        s = NBodySolverFMM_SYM_MORTON(kernel, max_children=leaf, tree_depth=best["depth"], theta=best["theta"],
                                      softening=softening, precision="fp32", order=best["order"], device=device,
                                      stream=s_torch.cuda_stream, mac=kind, slack=float(slack or 1.0), leaf_p2p=v,
                                      centre=best.get("centre", "com"), m2l=best.get("m2l", "simt"))
        try:
            ms = _time_step(s, pos_d, grad_d, tot_d, s_torch)
            err = median_error(grad_d[rows_d].cpu().numpy(), ref_rows)
        finally:
            s.close()
        t = dict(best, leaf_p2p=v, ms=ms, err=err)
        trials.append(t)
        if err <= target and ms < out["ms"]:
            out = t
    return out, trials


def _time_step(s, pos_d, grad_d, tot_d, s_torch):
    import torch
    s.update_tree_device(pos_d)
    s.solve_device(grad_d, tot_d)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s_torch)
    s.update_tree_device(pos_d)
    s.solve_device(grad_d, tot_d)
    e1.record(s_torch)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def tune_learned(pos_d, ref_rows, rows_d, controller, *, kernel: str, softening: float, leaf: int, target: float,
                 stream=None, depths=None, taus=TAUS, device: int = 0, log=None):
    """The learned-order controller's knobs: for each depth the largest tau
    (loosest tolerance) whose measured median error meets the target.
    Returns (best, trials); best = dict(depth, tau, ms, err) or None."""
    import torch

    n = pos_d.shape[0]
    d0 = get_depth(leaf, n)
    depths = depths or (d0 + 1, d0 + 2)
    grad_d = torch.zeros((n, 2), dtype=torch.float64, device=pos_d.device)
    tot_d = torch.zeros(1, dtype=torch.float64, device=pos_d.device)
    s_torch = torch.cuda.Stream(device=pos_d.device) if stream is None else stream
    trials, best = [], None
    for depth in depths:
        if depth > 15:
            continue
        for tau in taus:
            s = NBodySolverFMM_SYM_MORTON(kernel, max_children=leaf, tree_depth=depth, theta=1.0,
                                          softening=softening, precision="fp32", order=12, device=device,
                                          stream=s_torch.cuda_stream)
            try:
                s.set_controller(controller, tau)
                ms = _time_step(s, pos_d, grad_d, tot_d, s_torch)
                err = median_error(grad_d[rows_d].cpu().numpy(), ref_rows)
            finally:
                s.close()
            t = dict(depth=depth, tau=tau, ms=ms, err=err)
            trials.append(t)
            if log:
                log(t)
            if err <= target:
                if best is None or ms < best["ms"]:
                    best = t
                break  # smaller tau at this depth only costs more
    return best, trials
