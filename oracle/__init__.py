"""TEST INFRASTRUCTURE -- the CPU oracle, never the product.

ctypes bindings for the plain-C FP64 restatement of the reference's tree-code
path (``oracle/treecode_oracle.c``) and, when it has been built in this
container, for the reference's own solvers compiled from its sources
(``oracle/_ref/libref_oracle.so``).  Only the tests, the smoke check and the
CPU-baseline leg of ``bench.py`` use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_oracle.so")

KERNEL_TSNE = 0
KERNEL_GRAVITY = 1

# orc_node in treecode_oracle.h (NodeFMM_MORTON_2D flattened), 208 bytes
NODE_DTYPE = np.dtype([
    ("bb_c", "f8", 2), ("bb_len", "f8"),
    ("first_child", "u4"), ("first_part", "u4"), ("count", "u4"), ("pad", "u4"),
    ("com", "f8", 2), ("m0", "f8"), ("m2", "f8", 4),
    ("c1", "f8", 2), ("c2", "f8", 4), ("c3", "f8", 8),
])
assert NODE_DTYPE.itemsize == 208


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc (FP contraction off: same bits on x86 and Arm)."""
    src = os.path.join(HERE, "treecode_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "treecode_oracle.h"))):
        subprocess.check_call(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                               "-o", LIB_PATH, src, "-lm", "-lpthread"])
    return LIB_PATH


def build_ref(ref_root: str = "/root/reference") -> str | None:
    """Compile the reference's own solvers (only where the reference sources exist)."""
    if not os.path.isdir(os.path.join(ref_root, "src")):
        return None
    repo = os.path.dirname(HERE)
    subprocess.check_call(["make", "-s", "-f", "oracle/Makefile.ref", f"REF={ref_root}"], cwd=repo)
    return REF_PATH


_lib = None
_ref = None
P = ctypes.c_void_p
I64 = ctypes.c_int64
D = ctypes.c_double
I = ctypes.c_int


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_get_depth.restype = ctypes.c_uint32
        L.orc_get_depth.argtypes = [I, I64]
        L.orc_node_count.restype = I64
        L.orc_node_count.argtypes = [ctypes.c_uint32]
        L.orc_morton_codes.argtypes = [I64, P, P, P, P]
        L.orc_sort_perm.argtypes = [I64, P, P]
        L.orc_build_tree.argtypes = [ctypes.c_uint32, I64, P, P, P, P]
        L.orc_sym_fmm_solve.argtypes = [I, D, ctypes.c_uint32, D, I64, P, P, P, P]
        L.orc_sym_fmm.argtypes = [I, D, I, I, D, I64, P, P, P, P, P, P, P, P, P]
        L.orc_fmm_morton_solve.argtypes = [I, D, D, P, P, P, P]
        L.orc_fmm_morton.argtypes = [I, D, I, I, D, I64, P, P, P, P, P, P, P, P, P]
        L.orc_naive.argtypes = [I, D, I64, P, P, P, I]
        L.orc_direct_rows.argtypes = [I, D, I64, P, I64, P, P, I]
        L.orc_bh.argtypes = [I, D, I, D, I64, P, P, P]
        L.orc_bhmp.argtypes = [I, D, I, D, I64, P, P, P]
        L.orc_pm.argtypes = [I, D, I, I64, P, P, P]
        L.orc_bh.restype = I
        L.orc_tsne_attractive.argtypes = [I64, P, P, P, P, D, P]
        L.orc_tsne_step.argtypes = [I64, P, P, P, P, P, I, I, D, D, D, D, P, P, P]
        L.orc_knn.argtypes = [I64, I, P, I, P, P]
        L.orc_exp.argtypes = [D]
        L.orc_exp.restype = D
        L.orc_log.argtypes = [D]
        L.orc_log.restype = D
        L.orc_perplexity.argtypes = [I64, I, P, D, I, D, P]
        L.orc_symmetrize.argtypes = [I64, I, P, P, P, P, P]
        L.orc_symmetrize.restype = I64
        _lib = L
    return _lib


def ref_lib():
    """The reference's own solvers, or None where they were not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = ctypes.CDLL(REF_PATH)
        R.ref_get_depth.restype = ctypes.c_uint
        R.ref_get_depth.argtypes = [I, I]
        R.ref_sym_fmm.argtypes = [I, D, I, I, D, I64] + [P] * 9 + [I]
        R.ref_naive.argtypes = [I, D, I64, P, P, P]
        R.ref_bh.argtypes = [I, D, I, D, I64, P, P, P, P]
        R.ref_bhmp.argtypes = [I, D, I, D, I64, P, P, P]
        R.ref_pm.argtypes = [I, D, I, I64, P, P, P]
        _ref = R
    return _ref


def get_depth(max_children: int, n: int) -> int:
    return int(lib().orc_get_depth(max_children, n))


def node_count(depth: int) -> int:
    return int(lib().orc_node_count(depth))


def bbox(pos: np.ndarray):
    return pos.min(0).astype(np.float64), pos.max(0).astype(np.float64)


def morton_codes(pos, mn, mx):
    pos = np.ascontiguousarray(pos, np.float64)
    out = np.empty(len(pos), np.uint32)
    lib().orc_morton_codes(len(pos), _p(pos), _p(np.asarray(mn, np.float64)),
                           _p(np.asarray(mx, np.float64)), _p(out))
    return out


def sort_perm(codes):
    codes = np.ascontiguousarray(codes, np.uint32)
    perm = np.empty(len(codes), np.int32)
    lib().orc_sort_perm(len(codes), _p(codes), _p(perm))
    return perm


def build_tree(pos, *, depth, mn=None, mx=None):
    """updateTree alone (createMortonCode, the stable code sort,
    createLeafNodes, bottomUpNodeConstruction): sorted codes, permutation,
    sorted positions and the node records (NODE_DTYPE; the C fields zero)."""
    pos = np.ascontiguousarray(pos, np.float64)
    if mn is None:
        mn, mx = bbox(pos)
    mn = np.ascontiguousarray(mn, np.float64)
    mx = np.ascontiguousarray(mx, np.float64)
    codes = morton_codes(pos, mn, mx)
    perm = sort_perm(codes)
    ps = np.ascontiguousarray(pos[perm])
    nodes = np.zeros(node_count(depth), NODE_DTYPE)
    lib().orc_build_tree(depth, len(pos), _p(ps), _p(mn), _p(mx), _p(nodes))
    return dict(codes=codes[perm], ids=perm, pos=ps, nodes=nodes)


def sym_fmm(pos, *, kernel=KERNEL_TSNE, eps=0.0, max_children=16, depth=-1, theta=0.5,
            mn=None, mx=None, want_nodes=True, symmetric=True):
    """updateTree + solveNbody of the symmetric Morton FMM (sorted-order
    outputs); symmetric=False runs the non-symmetric FMM_MORTON instead."""
    pos = np.ascontiguousarray(pos, np.float64)
    n = len(pos)
    if mn is None:
        mn, mx = bbox(pos)
    d = depth if depth >= 0 else get_depth(max_children, n)
    codes = np.empty(n, np.uint32)
    ids = np.empty(n, np.int32)
    ps = np.empty((n, 2))
    g = np.zeros((n, 2))
    tot = np.zeros(1)
    nodes = np.zeros(node_count(d), NODE_DTYPE) if want_nodes else None
    fn = lib().orc_sym_fmm if symmetric else lib().orc_fmm_morton
    fn(kernel, eps, max_children, d, theta, n, _p(pos), _p(np.asarray(mn, np.float64)),
       _p(np.asarray(mx, np.float64)), _p(codes), _p(ids), _p(ps), _p(g), _p(tot), _p(nodes))
    return dict(codes=codes, ids=ids, pos=ps, grad=g, total=float(tot[0]), nodes=nodes, depth=d)


def knn(x, k):
    """Exact k nearest neighbours (FP32 distances summed in dimension order,
    ties by index, self excluded): (dist n x k float32, idx n x k int32)."""
    x = np.ascontiguousarray(x, np.float32)
    n, dim = x.shape
    d = np.empty((n, k), np.float32)
    i = np.empty((n, k), np.int32)
    lib().orc_knn(n, dim, _p(x), k, _p(d), _p(i))
    return d, i


def perplexity_rows(dist, perplexity, max_iter=100, tol=1e-5):
    """Row-normalised Gaussian affinities calibrated to the perplexity (FP64)."""
    dist = np.ascontiguousarray(dist, np.float32)
    n, k = dist.shape
    p = np.empty((n, k))
    lib().orc_perplexity(n, k, _p(dist), perplexity, max_iter, tol, _p(p))
    return p


def symmetrize(idx, p):
    """(P + P^T) / (2N) as CSR (row_ptr u32, col u32, val f64)."""
    idx = np.ascontiguousarray(idx, np.int32)
    p = np.ascontiguousarray(p, np.float64)
    n, k = idx.shape
    rp = np.empty(n + 1, np.uint32)
    col = np.empty(2 * n * k, np.uint32)
    val = np.empty(2 * n * k)
    nnz = lib().orc_symmetrize(n, k, _p(idx), _p(p), _p(rp), _p(col), _p(val))
    return rp, col[:nnz].copy(), val[:nnz].copy()


def affinity_csr(x, perplexity=30.0, k=None, max_iter=100, tol=1e-5):
    """The whole affinity build: kNN, bandwidths, symmetrisation."""
    k = int(3 * perplexity) if k is None else k
    d, i = knn(x, min(k, len(x) - 1))
    return symmetrize(i, perplexity_rows(d, perplexity, max_iter, tol))


def bhmp(pos, *, kernel=KERNEL_TSNE, eps=0.0, max_children=16, theta=0.5):
    """NBodySolverBHMP (Barnes-Hut with quadrupoles), input order."""
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = np.zeros(1)
    lib().orc_bhmp(kernel, eps, max_children, theta, len(pos), _p(pos), _p(g), _p(tot))
    return g, float(tot[0])


def pm(pos, *, n_interp=4, cell_size=1.0, min_intervals=4):
    """NBodySolverPM (FFT-accelerated interpolation t-SNE repulsion), input order."""
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = np.zeros(1)
    rc = lib().orc_pm(n_interp, cell_size, min_intervals, len(pos), _p(pos), _p(g), _p(tot))
    if rc != 0:
        raise ValueError("orc_pm: invalid arguments")
    return g, float(tot[0])


def pm_numpy(pos, *, n_interp=4, cell_size=1.0, min_intervals=4):
    """The same NBodySolverPM restatement vectorised with numpy (pocketfft for the
    transforms): the CPU baseline of the particle-mesh workload.  Same grid and
    node sums as orc_pm; differs only in FFT rounding."""
    pos = np.ascontiguousarray(pos, np.float64)
    n, p = len(pos), int(n_interp)
    v = pos.reshape(-1)
    prefix = np.concatenate([[-np.inf], np.maximum.accumulate(v)[:-1]])
    record = v > prefix                       # the reference's `if (v > max)` branch
    mx = float(v.max())
    rest = v[~record]
    mn = float(rest.min()) if rest.size else float("inf")
    nb = max(int(min_intervals), int((mx - mn) / cell_size))
    bw = (mx - mn) / nb
    hs = 1.0 / p
    sp = [hs / 2]
    for _ in range(1, p):
        sp.append(sp[-1] + hs)
    sp = np.array(sp)
    den = np.array([np.prod([sp[i] - sp[j] for j in range(p) if j != i]) for i in range(p)])
    n1, nf = p * nb, 2 * p * nb
    xt = [mn + hs * bw / 2]
    for _ in range(1, n1):
        xt.append(xt[-1] + hs * bw)
    xt = np.array(xt)
    d = xt[0] - xt
    ker = (1.0 + d[:, None] ** 2 + d[None, :] ** 2) ** -2
    kt = np.zeros((nf, nf))
    kt[n1:, n1:] = ker
    kt[n1:0:-1, n1:] = ker[: n1]
    kt[n1:, n1:0:-1] = ker[:, : n1]
    kt[n1:0:-1, n1:0:-1] = ker[: n1, : n1]
    kf = np.fft.rfft2(kt)
    ix = np.clip(((pos[:, 0] - mn) / bw).astype(np.int64), 0, nb - 1)
    iy = np.clip(((pos[:, 1] - mn) / bw).astype(np.int64), 0, nb - 1)

    def lagrange(t):
        out = np.ones((len(t), p))
        for j in range(p):
            for k in range(p):
                if j != k:
                    out[:, j] *= t - sp[k]
            out[:, j] /= den[j]
        return out

    wx = lagrange((pos[:, 0] - (ix * bw + mn)) / bw)
    wy = lagrange((pos[:, 1] - (iy * bw + mn)) / bw)
    q = [np.ones(n), pos[:, 0], pos[:, 1], pos[:, 0] * pos[:, 0] + pos[:, 1] * pos[:, 1]]
    phi = np.zeros((4, n))
    for dd in range(4):
        grid = np.zeros((n1, n1))
        for a in range(p):
            for b in range(p):
                np.add.at(grid, (ix * p + a, iy * p + b), wy[:, b] * wx[:, a] * q[dd])
        fin = np.zeros((nf, nf))
        fin[:n1, :n1] = grid
        pot = np.fft.irfft2(np.fft.rfft2(fin) * kf, s=(nf, nf))[n1:, n1:]
        for a in range(p):
            for b in range(p):
                phi[dd] += wx[:, a] * wy[:, b] * pot[ix * p + a, iy * p + b]
    x, y = pos[:, 0], pos[:, 1]
    grad = np.stack([x * phi[0] - phi[1], y * phi[0] - phi[2]], axis=1)
    total = float(np.sum((1 + x * x + y * y) * phi[0] - 2 * (x * phi[1] + y * phi[2]) + phi[3]) - n)
    return grad, total


def ref_pm(pos, *, n_interp=4, cell_size=1.0, min_intervals=4):
    """The reference's own NBodySolverPM (oracle/_ref), or None where it was not built."""
    R = ref_lib()
    if R is None:
        return None
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = np.zeros(1)
    R.ref_pm(n_interp, cell_size, min_intervals, len(pos), _p(pos), _p(g), _p(tot))
    return g, float(tot[0])


def naive(pos, *, kernel=KERNEL_TSNE, eps=0.0, nthreads=None):
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = np.zeros(1)
    lib().orc_naive(kernel, eps, len(pos), _p(pos), _p(g), _p(tot), nthreads or os.cpu_count() or 1)
    return g, float(tot[0])


def direct_rows(pos, rows, *, kernel=KERNEL_TSNE, eps=0.0, nthreads=None):
    pos = np.ascontiguousarray(pos, np.float64)
    rows = np.ascontiguousarray(rows, np.int64)
    g = np.zeros((len(rows), 2))
    lib().orc_direct_rows(kernel, eps, len(pos), _p(pos), len(rows), _p(rows), _p(g),
                          nthreads or os.cpu_count() or 1)
    return g


def bh(pos, *, kernel=KERNEL_TSNE, eps=0.0, max_children=16, theta=0.5):
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = np.zeros(1)
    lib().orc_bh(kernel, eps, max_children, theta, len(pos), _p(pos), _p(g), _p(tot))
    return g, float(tot[0])


def tsne_attractive(row_ptr, col, val, pos, exag, grad):
    lib().orc_tsne_attractive(len(pos), _p(row_ptr), _p(col), _p(val), _p(pos), exag, _p(grad))


def tsne_step(y, y_prev, row_ptr, col, val, *, max_children=16, depth=-1, theta=0.5,
              exag_code=16.0, lr=None, momentum=0.5):
    y = np.ascontiguousarray(y, np.float64)
    y_prev = np.ascontiguousarray(y_prev, np.float64)
    n = len(y)
    d = depth if depth >= 0 else get_depth(max_children, n)
    lr = n / 15.0 if lr is None else lr
    yn = np.empty_like(y)
    g = np.zeros_like(y)
    z = np.zeros(1)
    lib().orc_tsne_step(n, _p(y), _p(y_prev), _p(np.ascontiguousarray(row_ptr, np.uint32)),
                        _p(np.ascontiguousarray(col, np.uint32)),
                        _p(np.ascontiguousarray(val, np.float64)), max_children, d, theta,
                        exag_code, lr, momentum, _p(yn), _p(g), _p(z))
    return yn, g, float(z[0])


# ---------------------------------------------------------------- reference
def ref_sym_fmm(pos, *, kernel=KERNEL_TSNE, eps=0.0, max_children=16, depth=-1, theta=0.5,
                mn=None, mx=None, symmetric=True):
    R = ref_lib()
    if R is None:
        return None
    pos = np.ascontiguousarray(pos, np.float64)
    n = len(pos)
    if mn is None:
        mn, mx = bbox(pos)
    d = depth if depth >= 0 else int(R.ref_get_depth(max_children, n))
    mm = np.array([mn[0], mn[1], mx[0], mx[1]], np.float64)
    codes = np.empty(n, np.uint32)
    ids = np.empty(n, np.int32)
    ps = np.empty((n, 2))
    g = np.zeros((n, 2))
    tot = np.zeros(1)
    nodes = np.zeros((node_count(d), 27))
    tm = np.zeros(2)
    R.ref_sym_fmm(kernel, eps, max_children, d, theta, n, _p(pos), _p(mm), _p(codes), _p(ids),
                  _p(ps), _p(g), _p(tot), _p(nodes), _p(tm), 1 if symmetric else 0)
    return dict(codes=codes, ids=ids, pos=ps, grad=g, total=float(tot[0]), nodes=nodes,
                depth=d, times=tm)


def ref_naive(pos, *, kernel=KERNEL_TSNE, eps=0.0):
    R = ref_lib()
    if R is None:
        return None
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = np.zeros(1)
    R.ref_naive(kernel, eps, len(pos), _p(pos), _p(g), _p(tot))
    return g, float(tot[0])


def ref_bh(pos, *, kernel=KERNEL_TSNE, eps=0.0, max_children=16, theta=0.5):
    R = ref_lib()
    if R is None:
        return None
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = np.zeros(1)
    tm = np.zeros(2)
    R.ref_bh(kernel, eps, max_children, theta, len(pos), _p(pos), _p(g), _p(tot), _p(tm))
    return g, float(tot[0])


def ref_bhmp(pos, *, kernel=KERNEL_TSNE, eps=0.0, max_children=16, theta=0.5):
    R = ref_lib()
    if R is None:
        return None
    pos = np.ascontiguousarray(pos, np.float64)
    g = np.zeros_like(pos)
    tot = np.zeros(1)
    R.ref_bhmp(kernel, eps, max_children, theta, len(pos), _p(pos), _p(g), _p(tot))
    return g, float(tot[0])


def ref_nodes_to_struct(ref_nodes: np.ndarray) -> np.ndarray:
    """Map the reference harness's 27-double node rows onto NODE_DTYPE."""
    out = np.zeros(len(ref_nodes), NODE_DTYPE)
    out["bb_c"] = ref_nodes[:, 0:2]
    out["bb_len"] = ref_nodes[:, 2]
    out["first_child"] = ref_nodes[:, 3].astype(np.uint32)
    out["first_part"] = ref_nodes[:, 4].astype(np.uint32)
    out["count"] = ref_nodes[:, 5].astype(np.uint32)
    out["com"] = ref_nodes[:, 6:8]
    out["m0"] = ref_nodes[:, 8]
    out["m2"] = ref_nodes[:, 9:13]
    out["c1"] = ref_nodes[:, 13:15]
    out["c2"] = ref_nodes[:, 15:19]
    out["c3"] = ref_nodes[:, 19:27]
    return out
