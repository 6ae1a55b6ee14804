"""The host-buffer entry points through the C ABI, with the reference's
semantics: updateTree sorts the caller's whole records in place (the sort
moves each TsnePoint2D with its ID, nBodySolverFMM_SYM_MORTON.h:89), and
solveNbody adds the force into each point's derivative (applyForces,
nBodySolverFMM_SYM_MORTON.h:533, `derivative +=`) and the pair sum into the
caller's total.  The IDs are permuted and the sum is taken on the device; both
must equal the host-side composition bit for bit."""
import ctypes

import numpy as np
import pytest

from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON, datasets
from masterthesislucas_gb300._lib import check, lib, ptr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["fp64", "fp32", "order8"])
def test_update_tree_moves_ids_and_solve_adds(mode):
    n = 5000
    pos = datasets.two_disks(n, seed=9).astype(np.float64)
    ids = np.random.default_rng(2).permutation(n).astype(np.int32) * 3 + 7  # arbitrary distinct IDs
    if mode == "order8":
        s = NBodySolverFMM_SYM_MORTON("gravity", max_children=16, theta=0.75, softening=1e-3, order=8,
                                      mac="bmax", leaf_p2p=64)
    else:
        s = NBodySolverFMM_SYM_MORTON("tsne", max_children=16, theta=0.5, precision=mode)
    L = lib()
    mn, mx = pos.min(0), pos.max(0)
    p = pos.copy()
    i = ids.copy()
    check(L.tc_update_tree(s._h, ptr(p), ptr(i), n, ptr(mn), ptr(mx)))
    perm = np.empty(n, np.int32)
    check(L.tc_get_tree(s._h, None, ptr(perm), None, None))
    assert np.array_equal(np.sort(perm), np.arange(n))
    np.testing.assert_array_equal(p, pos[perm])
    np.testing.assert_array_equal(i, ids[perm])
    # without IDs the positions are sorted the same way
    p2 = pos.copy()
    check(L.tc_update_tree(s._h, ptr(p2), None, n, ptr(mn), ptr(mx)))
    np.testing.assert_array_equal(p2, p)

    g0 = np.zeros((n, 2))
    t0 = ctypes.c_double(0.0)
    check(L.tc_solve(s._h, ctypes.byref(t0), None, ptr(g0), n))
    assert np.isfinite(g0).all() and np.abs(g0).max() > 0
    base = np.random.default_rng(5).normal(size=(n, 2))
    g1 = base.copy()
    t1 = ctypes.c_double(2.5)
    check(L.tc_solve(s._h, ctypes.byref(t1), None, ptr(g1), n))
    np.testing.assert_array_equal(g1, base + g0)  # one FP64 add per component, as on the host
    assert t1.value == 2.5 + t0.value
    s.close()
