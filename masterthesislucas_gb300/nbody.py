"""N-body time stepping over the FMM force (device resident).

``LeapfrogNBody`` advances equal-mass particles (G = 1) with the
kick-drift-kick leapfrog of ``tc_leapfrog_step``; the reference's N-body
scenes step kick-then-drift around their solver call
(src/nBodyInstances/gravitysim.h:99-127, nbodySim.h:215-240).  Energy and
momentum are summed in FP64 on the device after every step.
"""
from __future__ import annotations

import numpy as np

from ._lib import check, lib, ptr
from .solver import NBodySolverFMM_SYM_MORTON


class LeapfrogNBody:
    def __init__(self, pos, vel=None, *, mass=None, dt=1e-4, softening=1e-3, max_children=64, tree_depth=None,
                 theta=1.0, order=8, device=0):
        import torch
        self.dev = torch.device("cuda", device)
        self.x = torch.as_tensor(np.ascontiguousarray(pos, np.float64), device=self.dev).clone()
        n = self.x.shape[0]
        self.v = (torch.zeros_like(self.x) if vel is None else
                  torch.as_tensor(np.ascontiguousarray(vel, np.float64), device=self.dev).clone())
        self.a = torch.zeros_like(self.x)
        self.diag = torch.zeros(4, dtype=torch.float64, device=self.dev)
        self.n = n
        self.mass = float(mass if mass is not None else 1.0 / n)
        self.dt = float(dt)
        self.solver = NBodySolverFMM_SYM_MORTON("gravity", max_children=max_children, tree_depth=tree_depth,
                                                theta=theta, softening=softening, order=order, device=device)
        self._init = True
        self.steps = 0

    def _call(self, dt, init):
        check(lib().tc_leapfrog_step(self.solver._h, ptr(self.x), ptr(self.v), ptr(self.a), self.n, dt, self.mass,
                                     int(init), ptr(self.diag)))

    def step(self, k: int = 1):
        for _ in range(k):
            self._call(self.dt, self._init)
            self._init = False
            self.steps += 1

    def reverse(self):
        """Negate the velocities (time reversal of the leapfrog)."""
        import torch
        torch.cuda.synchronize(self.dev)
        self.v.neg_()
        torch.cuda.synchronize(self.dev)

    def diagnostics(self) -> dict:
        """{kinetic, potential, energy, px, py} after the last step (evaluates at t = 0)."""
        import torch
        if self._init:
            self._call(0.0, True)
            self._init = False
        torch.cuda.synchronize(self.dev)
        k, u, px, py = self.diag.cpu().numpy().tolist()
        return {"kinetic": k, "potential": u, "energy": k + u, "px": px, "py": py}

    def state(self):
        import torch
        torch.cuda.synchronize(self.dev)
        return self.x.cpu().numpy(), self.v.cpu().numpy()

    def close(self):
        self.solver.close()


def circular_velocities(pos, mass, softening=1e-3, centres=None):
    """Rotation about each disk centre from the enclosed mass (a cold start
    when ``centres`` is None)."""
    pos = np.asarray(pos, np.float64)
    if centres is None:
        return np.zeros_like(pos)
    v = np.zeros_like(pos)
    c = np.asarray(centres, np.float64)
    owner = np.argmin(((pos[:, None, :] - c[None]) ** 2).sum(-1), axis=1)
    for k in range(len(c)):
        sel = owner == k
        d = pos[sel] - c[k]
        r = np.sqrt((d ** 2).sum(1))
        order = np.argsort(r)
        m_enc = np.empty(len(r))
        m_enc[order] = np.arange(1, len(r) + 1) * mass
        vc = np.sqrt(m_enc * r ** 2 / (r ** 2 + softening ** 2) ** 1.5)
        v[sel, 0] = -vc * d[:, 1] / np.maximum(r, 1e-12)
        v[sel, 1] = vc * d[:, 0] / np.maximum(r, 1e-12)
    return v
