"""Leapfrog N-body steps over the FMM force: trajectories against an FP64
leapfrog on the oracle's direct-sum forces, energy and momentum
conservation, and time reversibility."""
import numpy as np
import pytest

import oracle
from masterthesislucas_gb300 import datasets
from masterthesislucas_gb300.nbody import LeapfrogNBody, circular_velocities

pytestmark = pytest.mark.gpu

EPS = 1e-3


def oracle_leapfrog(x, v, m, dt, steps):
    """KDK leapfrog with the oracle's FP64 direct sum (unit-mass field * m)."""
    x, v = x.copy(), v.copy()
    a = oracle.naive(x, kernel=oracle.KERNEL_GRAVITY, eps=EPS)[0] * m
    for _ in range(steps):
        v += 0.5 * dt * a
        x += dt * v
        g, tot = oracle.naive(x, kernel=oracle.KERNEL_GRAVITY, eps=EPS)
        a = g * m
        v += 0.5 * dt * a
    k = 0.5 * m * (v ** 2).sum()
    u = 0.5 * m * m * tot
    return x, v, k + u


def test_trajectory_matches_fp64_direct_leapfrog():
    n = 3000
    x0 = datasets.two_disks(n, seed=11).astype(np.float64)
    m = 1.0 / n
    v0 = circular_velocities(x0, m, EPS, centres=[[-0.3, 0.0], [0.3, 0.0]])
    sim = LeapfrogNBody(x0, v0, mass=m, dt=1e-4, max_children=16, theta=0.5, order=12)
    sim.step(20)
    x, v = sim.state()
    e = sim.diagnostics()["energy"]
    xr, vr, er = oracle_leapfrog(x0, v0, m, 1e-4, 20)
    span = np.abs(x0).max()
    assert np.abs(x - xr).max() < 1e-8 * span
    assert np.abs(v - vr).max() < 1e-6 * np.abs(vr).max()
    assert e == pytest.approx(er, rel=1e-5)
    sim.close()


def test_energy_and_momentum_are_conserved():
    n = 65536
    x0 = datasets.two_disks(n, seed=5).astype(np.float64)
    m = 1.0 / n
    sim = LeapfrogNBody(x0, None, mass=m, dt=1e-4, theta=0.8, order=10)
    d0 = sim.diagnostics()
    sim.step(100)
    d1 = sim.diagnostics()
    drift = abs(d1["energy"] - d0["energy"]) / abs(d0["energy"])
    assert d1["kinetic"] > 0.0
    assert drift < 1e-4, (d0, d1)
    # momentum starts at zero; the symmetric pair interactions keep it small
    pscale = m * n * np.sqrt(2.0 * d1["kinetic"] / (m * n))
    assert np.hypot(d1["px"], d1["py"]) < 1e-4 * pscale
    sim.close()


def test_time_reversal_returns_to_the_start():
    n = 20000
    x0 = datasets.two_disks(n, seed=8).astype(np.float64)
    sim = LeapfrogNBody(x0, None, mass=1.0 / n, dt=1e-4, theta=0.8, order=10)
    sim.step(10)
    sim.reverse()
    sim.step(10)
    x, v = sim.state()
    # the force is a deterministic function of the positions, so KDK retraces
    # its path up to rounding (FP32 expansions, FP64 state)
    assert np.abs(x - x0).max() < 1e-9
    sim.close()


def test_invalid_arguments_are_rejected():
    from masterthesislucas_gb300._lib import TreecodeError, lib, check, ptr
    sim = LeapfrogNBody(datasets.two_disks(1000, seed=1).astype(np.float64), dt=1e-4)
    with pytest.raises(TreecodeError):
        check(lib().tc_leapfrog_step(sim.solver._h, None, ptr(sim.v), ptr(sim.a), sim.n, 1e-4, 1e-3, 1,
                                     ptr(sim.diag)))
    with pytest.raises(TreecodeError):
        check(lib().tc_leapfrog_step(sim.solver._h, ptr(sim.x), ptr(sim.v), ptr(sim.a), sim.n, 1e-4, -1.0, 1,
                                     ptr(sim.diag)))
    sim.close()
