"""Host-side mirror of the reference's solver interface over the C ABI.

``NBodySolverFMM_SYM_MORTON`` keeps the names and argument meaning of
``NBodySolver<T>`` (src/nbodysolvers/cpu/nBodySolver.h:9-23) as implemented by
``NBodySolverFMM_SYM_MORTON<TsnePoint2D>``
(src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:29-614):

* ``updateTree(points, minPos, maxPos)`` sorts ``points`` into Morton order in
  place (positions, derivatives, labels and IDs move together, as the
  reference's AoS sort moves whole ``TsnePoint2D`` records);
* ``solveNbody(total, points)`` adds the repulsive force into
  ``points.derivative`` and returns ``total`` plus the kernel's pair sum (the
  reference's ``double& total`` argument);
* ``getNodesBufferData(level)`` returns the boxes of the non-empty nodes.

``Points`` is the structure-of-arrays form of ``std::vector<TsnePoint2D>``
(src/particles/tsnePoint2D.h:6-37).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, lib, ptr


@dataclass
class Points:
    position: np.ndarray               # (n, 2) float64
    derivative: np.ndarray             # (n, 2) float64
    ID: np.ndarray                     # (n,) int32
    label: np.ndarray | None = None    # (n,) int32

    @classmethod
    def from_positions(cls, pos) -> "Points":
        pos = np.ascontiguousarray(pos, np.float64)
        n = len(pos)
        return cls(pos.copy(), np.zeros((n, 2)), np.arange(n, dtype=np.int32), np.zeros(n, np.int32))

    def __len__(self):
        return len(self.position)


KERNELS = {"tsne": _lib.TC_KERNEL_TSNE, "gravity": _lib.TC_KERNEL_GRAVITY}
PRECISIONS = {"fp32": _lib.TC_PREC_FP32, "fp64": _lib.TC_PREC_FP64}


def get_depth(max_children: int, n: int) -> int:
    d = ctypes.c_uint32(0)
    check(lib().tc_get_depth(max_children, n, ctypes.byref(d)))
    return int(d.value)


def node_count(depth: int) -> int:
    c = ctypes.c_int64(0)
    check(lib().tc_node_count(depth, ctypes.byref(c)))
    return int(c.value)


class NBodySolverFMM_SYM_MORTON:
    """GPU symmetric Morton FMM behind the reference's solver interface."""

    def __init__(self, kernel: str = "tsne", max_children: int = 16, tree_depth: int | None = None,
                 theta: float = 0.5, softening: float = 1e-3, precision: str = "fp32", device: int = 0,
                 stream=None, order: int = 0, mac: str = "cell", slack: float = 1.0, leaf_p2p: int = 0,
                 centre: str = "com", m2l: str = "simt", near_overlap: bool = True):
        """mac (order p only): "cell", the reference's (L_A + L_B)/theta <
        |dcom| with cell sizes L; "bmax", (b_A + b_B)/theta < |dcom| with b
        the largest distance of a node's particles from its COM;
        "bmax_adaptive", the same with each accepted pair evaluated at the
        lowest order in {4, 6, ..., order} whose bound ((b_A + b_B)/|dcom|)^(q+1)
        stays below slack * theta^(order+1).
        leaf_p2p (order p): accepted leaf pairs with at most this many
        particle pairs are summed directly instead of by an M2L.
        centre (order p, fp32): "com" expands about each node's centre of
        mass; "box" about its cell centre (M2L operators then depend only on
        the level and the grid offset of a pair).
        m2l (centre "box"): "simt" FP32 kernels, or "tensor" the tensor-core
        M2L (BF16 hi/lo split, FP32 accumulation) on the levels with enough
        nodes to fill the GPU, or "tensor_all" on every level.
        near_overlap (order p): the near field runs on a second stream beside
        the far field (False: in sequence; the results are identical)."""
        if centre not in ("com", "box"):
            raise ValueError("centre must be 'com' or 'box'")
        if m2l not in ("simt", "tensor", "tensor_all"):
            raise ValueError("m2l must be 'simt', 'tensor' or 'tensor_all'")
        if mac not in ("cell", "bmax", "bmax_adaptive"):
            raise ValueError("mac must be 'cell', 'bmax' or 'bmax_adaptive'")
        cfg = _lib.TcConfig()
        check(lib().tc_config_init(ctypes.byref(cfg)))
        cfg.kernel = KERNELS[kernel]
        cfg.max_children = max_children
        cfg.depth = -1 if tree_depth is None else int(tree_depth)
        cfg.theta = theta
        cfg.softening = softening
        cfg.precision = PRECISIONS[precision]
        cfg.device = device
        cfg.stream = stream
        cfg.order = order
        self.order = order
        self._h = ctypes.c_void_p()
        check(lib().tc_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self.mac = mac
        if mac.startswith("bmax"):
            check(lib().tc_set_mac(self._h, _lib.TC_MAC_BMAX))
        if mac == "bmax_adaptive":
            check(lib().tc_set_adaptive_order(self._h, float(slack)))
        if leaf_p2p:
            check(lib().tc_set_leaf_p2p(self._h, int(leaf_p2p)))
        if centre == "box":
            check(lib().tc_set_expansion_centre(self._h, _lib.TC_CENTRE_BOX))
        if m2l != "simt":
            check(lib().tc_set_m2l_engine(self._h, _lib.TC_M2L_TENSOR if m2l == "tensor"
                                          else _lib.TC_M2L_TENSOR_ALL))
        if not near_overlap:
            check(lib().tc_set_near_overlap(self._h, 0))
        self.centre = centre
        self.m2l = m2l
        self.near_overlap = near_overlap
        self.maxChildren = max_children
        self._cfg_depth = cfg.depth
        self._theta = theta
        self.kernel = kernel
        self.precision = precision
        self.treeDepth = None
        self.n = 0

    # -- NBodySolver fields
    @property
    def theta(self) -> float:
        return self._theta

    @theta.setter
    def theta(self, v: float):
        check(lib().tc_set_theta(self._h, float(v)))
        self._theta = float(v)

    def close(self):
        if self._h:
            lib().tc_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- NBodySolver methods
    def updateTree(self, points: Points, minPos, maxPos):
        n = len(points)
        pos = np.ascontiguousarray(points.position, np.float64)
        ids = np.ascontiguousarray(points.ID, np.int32)
        mn = np.asarray(minPos, np.float64)
        mx = np.asarray(maxPos, np.float64)
        check(lib().tc_update_tree(self._h, ptr(pos), None, n, ptr(mn), ptr(mx)))
        perm = np.empty(n, np.int32)
        check(lib().tc_get_tree(self._h, None, ptr(perm), None, None))
        points.position[...] = pos
        points.ID[...] = ids[perm]
        points.derivative[...] = points.derivative[perm]
        if points.label is not None:
            points.label[...] = points.label[perm]
        self.n = n
        self.treeDepth = get_depth(self.maxChildren, n) if self._depth_cfg() < 0 else self._depth_cfg()
        return perm

    def _depth_cfg(self):
        return -1 if not hasattr(self, "_cfg_depth") else self._cfg_depth

    def solveNbody(self, total: float, points: Points) -> float:
        tot = ctypes.c_double(total)
        grad = np.ascontiguousarray(points.derivative, np.float64)
        check(lib().tc_solve(self._h, ctypes.byref(tot), None, ptr(grad), len(points)))
        points.derivative[...] = grad
        return float(tot.value)

    def getNodesBufferData(self, level: int = -1) -> np.ndarray:
        cnt = ctypes.c_int64(0)
        check(lib().tc_get_node_boxes(self._h, level, None, 0, ctypes.byref(cnt)))
        boxes = np.zeros((cnt.value, 3))
        check(lib().tc_get_node_boxes(self._h, level, ptr(boxes), cnt.value, ctypes.byref(cnt)))
        return boxes

    # -- extras used by the tests and the benchmark
    def tree_dump(self):
        """Morton codes, permutation, sorted positions and the 27-double node rows."""
        n = self.n
        codes = np.empty(n, np.uint32)
        perm = np.empty(n, np.int32)
        pos = np.empty((n, 2))
        nodes = np.empty((node_count(self.depth()), 27))
        check(lib().tc_get_tree(self._h, ptr(codes), ptr(perm), ptr(pos), ptr(nodes)))
        return dict(codes=codes, perm=perm, pos=pos, nodes=nodes)

    def depth(self) -> int:
        return self.treeDepth

    def list_stats(self):
        d = self.depth()
        nn = np.zeros(d + 1, np.uint32)
        nr = np.zeros(d + 1, np.uint32)
        check(lib().tc_get_list_stats(self._h, ptr(nn), ptr(nr)))
        return nn, nr

    def launches(self) -> int:
        return int(lib().tc_last_launch_count(self._h))

    STAGES = ("sort", "build", "lists", "far", "near", "l2p", "reduce")

    def stage_times(self) -> dict:
        """Device milliseconds per stage of the last update + solve (CUDA events)."""
        ms = np.zeros(len(self.STAGES))
        check(lib().tc_get_stage_times(self._h, ptr(ms)))
        return dict(zip(self.STAGES, ms.tolist()))

    def counters(self) -> dict:
        c = np.zeros(4, np.uint64)
        check(lib().tc_get_counters(self._h, ptr(c)))
        return dict(p2p_pairs=int(c[0]), m2p=int(c[1]), p2l=int(c[2]), m2l=int(c[3]))

    def capture_step(self, pos, grad, total, box=None, scatter: bool = True):
        """Captures updateTree + solveNbody on device tensors as one CUDA graph
        (after an ordinary update_tree_device of the same positions' size)."""
        import numpy as _np
        if box is None:
            mn = pos.min(0).values.cpu().numpy()
            mx = pos.max(0).values.cpu().numpy()
            box = _np.concatenate([mn, mx])
        self._box = _np.ascontiguousarray(box, _np.float64)
        check(lib().tc_step_capture(self._h, ptr(pos), pos.shape[0], ptr(self._box), ptr(grad), ptr(total),
                                    int(scatter)))

    def launch_step(self):
        """Replays the captured step (asynchronous on the handle's stream)."""
        check(lib().tc_step_launch(self._h))

    def async_status(self) -> int:
        """After synchronising a replay: 0 valid, bit 0 a point left the box, bit 1 a list overflowed."""
        return int(lib().tc_async_status(self._h))

    def set_controller(self, controller, tau: float = 1e-4):
        """Accept pairs by a learned order controller (FP32, order 12 handles);
        None restores the MAC.  Takes effect at the next updateTree."""
        check(lib().tc_set_controller(self._h, None if controller is None else controller._m, float(tau)))

    def list_orders(self, level: int) -> np.ndarray:
        """Order bucket (0..4 for orders 4, 6, 8, 10, 12) of each accepted pair of a level."""
        tot = ctypes.c_int64(0)
        check(lib().tc_get_list(self._h, level, 0, None, None, ctypes.byref(tot)))
        out = np.zeros(max(tot.value, 1), np.uint8)
        check(lib().tc_get_list(self._h, level, 2, None, ptr(out), ctypes.byref(tot)))
        return out[:tot.value]

    # device-resident entry points (torch tensors on the handle's device)
    def update_tree_device(self, pos, minPos=None, maxPos=None):
        mn = None if minPos is None else np.asarray(minPos, np.float64)
        mx = None if maxPos is None else np.asarray(maxPos, np.float64)
        check(lib().tc_update_tree_device(self._h, ptr(pos), pos.shape[0], ptr(mn), ptr(mx)))
        self.n = pos.shape[0]
        self.treeDepth = get_depth(self.maxChildren, self.n) if self._depth_cfg() < 0 else self._depth_cfg()

    def solve_device(self, grad, total, accumulate: bool = False, scatter: bool = True):
        check(lib().tc_solve_device(self._h, ptr(grad), ptr(total), int(accumulate), int(scatter)))


class NBodySolverFMM_MORTON(NBodySolverFMM_SYM_MORTON):
    """The reference's non-symmetric Morton FMM (src/nbodysolvers/cpu/
    nBodySolverFMM_MORTON.h): the same tree, ordered (sink, source) pairs,
    kernels applied to the sink only, M2P/P2P per sink point at the leaves.
    Runs at the reference's expansion order."""

    def __init__(self, kernel: str = "tsne", max_children: int = 16, tree_depth: int | None = None,
                 theta: float = 0.5, **kw):
        if kw.get("order", 0):
            raise ValueError("NBodySolverFMM_MORTON runs at the reference's expansion order (order 0)")
        super().__init__(kernel, max_children=max_children, tree_depth=tree_depth, theta=theta, **kw)
        check(lib().tc_set_variant(self._h, _lib.TC_VARIANT_MORTON))


def direct(pos, *, kernel="tsne", softening=1e-3, precision="fp64", rows=None):
    """O(N^2) force on `rows` (all points when None) on the GPU."""
    pos = np.ascontiguousarray(pos, np.float64)
    n = len(pos)
    r = None if rows is None else np.ascontiguousarray(rows, np.int64)
    m = n if r is None else len(r)
    g = np.zeros((m, 2))
    tot = ctypes.c_double(0.0)
    check(lib().tc_direct(KERNELS[kernel], softening, PRECISIONS[precision], ptr(pos), n, ptr(r), m, ptr(g),
                          ctypes.byref(tot)))
    return g, float(tot.value)


def barnes_hut(pos, *, kernel="tsne", softening=1e-3, max_children=16, theta=0.5, precision="fp32",
               multipole=False):
    """NBodySolverBH on the GPU (NBodySolverBHMP with multipole=True): forces
    in input order and the pair sum."""
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = ctypes.c_double(0.0)
    fn = lib().tc_bhmp_solve if multipole else lib().tc_bh_solve
    check(fn(KERNELS[kernel], softening, max_children, theta, PRECISIONS[precision], ptr(pos), len(pos), ptr(g),
             ctypes.byref(tot)))
    return g, float(tot.value)


def particle_mesh(pos, *, n_interp: int = 4, cell_size: float = 1.0, min_intervals: int = 4):
    """NBodySolverPM::solveNbody on the GPU (FFT-accelerated interpolation
    t-SNE repulsion, FP64): the reference's derivative sum_j q_ij^2 (y_i - y_j)
    in input order and the pair sum over i != j of q_ij."""
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = ctypes.c_double(0.0)
    check(lib().tc_pm_solve(int(n_interp), float(cell_size), int(min_intervals), ptr(pos), len(pos), ptr(g),
                            ctypes.byref(tot)))
    return g, float(tot.value)


class NBodySolverPM:
    """The reference's NBodySolverPM interface (nBodySolverPM.h:93-305): the
    constructor takes the interpolation points per box, the box side
    (cell_size) and the minimum number of boxes per dimension; updateTree does
    nothing; solveNbody overwrites the points' derivatives and returns the
    pair sum (the reference overwrites both)."""

    def __init__(self, n_interpolation_points: int = 4, cell_size: float = 1.0, min_num_intervals: int = 4):
        self.n_interpolation_points = int(n_interpolation_points)
        self.cell_size = float(cell_size)
        self.min_num_intervals = int(min_num_intervals)

    def updateTree(self, points, min_pos=None, max_pos=None):
        pass

    def solveNbody(self, total: float, points: "Points") -> float:
        g, t = particle_mesh(points.position, n_interp=self.n_interpolation_points, cell_size=self.cell_size,
                             min_intervals=self.min_num_intervals)
        points.derivative[:] = g
        return t
