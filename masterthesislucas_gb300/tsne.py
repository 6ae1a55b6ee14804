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
                 learn_rate: float | None = None, order: int = 0, depth: int = -1):
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
