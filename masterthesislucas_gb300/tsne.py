"""Host-side mirror of the reference's ``TSNE`` driver over the device step.

``TSNE`` keeps the schedule of src/nBodyInstances/tsne.h: learning rate N/15
(:90), early exaggeration for the first 250 iterations (:358), momentum 0.5
then 0.8 (:186), and the cosine theta schedule of ``thetaFunction``
(:208-233).  The code's attractive factor is 4 x exaggeration (the gradient's
factor 4 folded in, 16 = 4 x 4 early and 4 late in the reference); the
benchmark workload uses an early exaggeration of 12 (factor 48).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import check, lib, ptr


class TSNE:
    def __init__(self, row_ptr, col, val, y0, *, early_exaggeration: float = 4.0, min_theta: float = 0.5,
                 max_theta: float = 0.5, max_children: int = 16, precision: str = "fp32", device: int = 0,
                 learn_rate: float | None = None, order: int = 0, depth: int = -1, repulsion: str = "tree",
                 cell_size: float = 1.0):
        """repulsion: "tree" (the handle's FMM) or "pm", the reference's particle-mesh solver
        (TSNE with nBodySelect "PM": 4 nodes per box, boxes of side cell_size)."""
        if repulsion not in ("tree", "pm"):
            raise ValueError("repulsion must be 'tree' or 'pm'")
        y0 = np.ascontiguousarray(y0, np.float64)
        self.n = len(y0)
        self.row_ptr = np.ascontiguousarray(row_ptr, np.uint32)
        self.col = np.ascontiguousarray(col, np.uint32)
        self.val = np.ascontiguousarray(val, np.float64)
        cfg = _lib.TcConfig()
        check(lib().tc_config_init(ctypes.byref(cfg)))
        cfg.kernel = _lib.TC_KERNEL_TSNE
        cfg.max_children = max_children
        cfg.theta = max_theta
        cfg.precision = {"fp32": _lib.TC_PREC_FP32, "fp64": _lib.TC_PREC_FP64}[precision]
        cfg.order = order
        cfg.depth = depth
        cfg.device = device
        self._t = ctypes.c_void_p()
        check(lib().tc_tsne_create(ctypes.byref(cfg), self.n, ptr(self.row_ptr), ptr(self.col), ptr(self.val),
                                   ptr(y0), ctypes.byref(self._t)))
        self.repulsion = repulsion
        self.cell_size = float(cell_size)
        if repulsion == "pm":
            check(lib().tc_tsne_set_repulsion(self._t, _lib.TC_REPULSION_PM, self.cell_size))
        self.order = order
        self.max_children = max_children
        self.learnRate = self.n / 15.0 if learn_rate is None else learn_rate
        self.early_exaggeration = early_exaggeration
        self.min_theta = min_theta
        self.max_theta = max_theta
        self.iteration_counter = 0
        self.last_z = None

    def close(self):
        if self._t:
            lib().tc_tsne_destroy(self._t)
            self._t = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def theta_for(self, it: int) -> float:
        """thetaFunction (tsne.h:208-233): cosine from max_theta to min_theta over 1000 iterations."""
        r = 0.5 + 0.5 * math.cos(math.pi * min((it / 999.0) ** 1.0, 1.0))
        return self.min_theta + r * (self.max_theta - self.min_theta)

    def time_step(self, with_z: bool = False):
        """One TSNE_buffers::timeStep: derivative at the current embedding, then the momentum step."""
        it = self.iteration_counter
        exag = 4.0 * (self.early_exaggeration if it < 250 else 1.0)
        mom = 0.5 if it < 250 else 0.8
        if self.min_theta != self.max_theta:
            check(lib().tc_tsne_set_theta(self._t, self.theta_for(it)))
        z = ctypes.c_double(0.0)
        check(lib().tc_tsne_step(self._t, exag, mom, self.learnRate, ctypes.byref(z) if with_z else None))
        self.iteration_counter += 1
        if with_z:
            self.last_z = z.value
        return self.last_z

    def embedding(self):
        y = np.empty((self.n, 2))
        yp = np.empty((self.n, 2))
        g = np.empty((self.n, 2))
        check(lib().tc_tsne_get(self._t, ptr(y), ptr(yp), ptr(g)))
        return y, yp, g

    def launches(self) -> int:
        return int(lib().tc_tsne_last_launch_count(self._t))

    def set_depth(self, depth: int):
        check(lib().tc_tsne_set_depth(self._t, int(depth)))
        self.depth = int(depth)


def tune_depth(system: TSNE, offsets=(0, 1, 2, 3), theta: float = 0.5, reps: int = 2) -> dict:
    """Autotunes one embedding's tree depth on its current positions: the
    device time of updateTree + solveNbody (CUDA events) at getDepth + each
    offset, with a separate solver on a copy of the embedding; the fastest
    depth is set on the system."""
    import torch
    from .solver import NBodySolverFMM_SYM_MORTON, get_depth
    y = torch.from_numpy(np.ascontiguousarray(system.embedding()[0])).cuda()
    g = torch.zeros_like(y)
    tot = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    leaf, order = system.max_children, system.order
    d0 = get_depth(leaf, system.n)
    trials = []
    for off in offsets:
        d = d0 + off
        if d > 15:
            continue
        s = NBodySolverFMM_SYM_MORTON("tsne", max_children=leaf, tree_depth=d, theta=theta, order=order,
                                      stream=stream.cuda_stream)
        s.update_tree_device(y)
        s.solve_device(g, tot)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            s.update_tree_device(y)
            s.solve_device(g, tot)
        e1.record(stream)
        torch.cuda.synchronize()
        trials.append((e0.elapsed_time(e1) / reps, d))
        s.close()
    ms, best = min(trials)
    system.set_depth(best)
    return {"depth": best, "ms": ms, "trials": trials}


class TSNEBatch:
    """Independent embeddings advanced in lockstep, one CUDA graph launch per
    step (``tc_tsne_batch_*``).  ``systems`` are ``TSNE`` objects (FP32,
    order > 0, not stepped on their own afterwards); they share the
    schedule: exaggeration for the first 250 iterations, momentum 0.5 then
    0.8, learning rate n/15 per system."""

    def __init__(self, systems, margin: float = 0.5, capture: bool = True):
        self.systems = list(systems)
        arr = (ctypes.c_void_p * len(self.systems))(*[s._t.value for s in self.systems])
        self._b = ctypes.c_void_p()
        check(lib().tc_tsne_batch_create(arr, len(self.systems), float(margin), ctypes.byref(self._b)))
        if not capture:
            check(lib().tc_tsne_batch_set_capture(self._b, 0))
        self.early_exaggeration = self.systems[0].early_exaggeration
        self.iteration_counter = self.systems[0].iteration_counter

    def time_step(self):
        it = self.iteration_counter
        exag = 4.0 * (self.early_exaggeration if it < 250 else 1.0)
        mom = 0.5 if it < 250 else 0.8
        check(lib().tc_tsne_batch_step(self._b, exag, mom, 1.0 / 15.0))
        self.iteration_counter += 1
        for s in self.systems:
            s.iteration_counter = self.iteration_counter

    def stats(self) -> dict:
        out = np.zeros(8, np.int64)
        check(lib().tc_tsne_batch_stats(self._b, ptr(out)))
        return dict(graph_launches=int(out[0]), captures=int(out[1]), restepped=int(out[2]),
                    graph_nodes=int(out[3]), particles=int(out[4]), kernels_per_launch=int(out[5]),
                    graph_ms=out[6] / 1e3, restep_ms=out[7] / 1e3)

    def close(self):
        if self._b:
            lib().tc_tsne_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
