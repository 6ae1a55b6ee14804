"""The FP32 fast path of the Morton quantisation (csrc/tree.cu: k_morton_fast)
restated in numpy float32 arithmetic (IEEE round-to-nearest, as on the GPU):
wherever it does not queue a point for the FP64 path, its cell index equals
the reference's createMortonCode (nBodySolverFMM_SYM_MORTON.h:545-549, the
oracle's FP64 restatement), on random points and on points placed within a
few ulps of cell edges."""
import numpy as np

import oracle


def fast_path(pos, mn, mx):
    L = max(mx[0] - mn[0], mx[1] - mn[1])
    s = np.float32(65536.0 / L)
    q = np.zeros(pos.shape, np.int64)
    exact = np.zeros(len(pos), bool)
    for c in range(2):
        v = (pos[:, c] - mn[c]).astype(np.float32) * s  # float32 product, rounded once
        assert v.dtype == np.float32
        top = v >= np.float32(65535.0 + 1.0 / 64.0)
        f = v - np.floor(v)
        exact |= ~top & ~((f >= np.float32(1.0 / 64.0)) & (f < np.float32(63.0 / 64.0)))
        q[:, c] = np.where(top, 65535, np.where(v > 0, np.floor(v), 0)).astype(np.int64)
    return q, exact


def ref_cells(pos, mn, mx):
    codes = oracle.morton_codes(pos, mn, mx).astype(np.int64)
    def compact(x):
        x &= 0x55555555
        x = (x | (x >> 1)) & 0x33333333
        x = (x | (x >> 2)) & 0x0F0F0F0F
        x = (x | (x >> 4)) & 0x00FF00FF
        x = (x | (x >> 8)) & 0x0000FFFF
        return x
    return np.stack([compact(codes.copy()), compact(codes >> 1)], axis=1)


def test_fast_path_agrees_where_it_does_not_defer():
    rng = np.random.default_rng(0)
    mn, mx = np.array([-1.3, -0.7]), np.array([1.1, 2.9])
    L = max(mx - mn)
    rnd = mn + rng.uniform(0.0, 1.0, (1 << 20, 2)) * (mx - mn)
    # points within a few ulps of cell edges at every level of the grid
    cells = rng.integers(0, 65536, (1 << 19, 2)).astype(np.float64)
    edge = mn + cells / 65536.0 * L
    edge = edge + rng.integers(-4, 5, edge.shape) * np.spacing(np.abs(edge) + 1.0)
    pos = np.clip(np.concatenate([rnd, edge, [mn, mx]]), mn, mx)
    q, exact = fast_path(pos, mn, mx)
    ref = ref_cells(pos, mn, mx)
    ok = ~exact
    assert ok[:len(rnd)].mean() > 0.9  # most random points take the fast path
    np.testing.assert_array_equal(q[ok], ref[ok])
    # the edge points are the ones the FP64 path takes
    assert exact[len(rnd):len(rnd) + len(edge)].mean() > 0.9
