"""Matrix Market files for the t-SNE affinity matrix P.

The reference reads P from Matrix Market files written offline by openTSNE
(``MnistLoader.ipynb`` cell 14, via scipy's ``mmwrite``) with Eigen's
``loadMarket`` (src/dataLoaders/loader.h:56-75), then builds row-sorted CSR
in ``TSNE::setupEfficientPmatrix`` (src/nBodyInstances/tsne.h:462-520),
taking each stored entry (r, c) as (c, r) -- the transpose, equal to P for a
symmetric P -- and sorting by row, then column.

``read_p_matrix`` accepts ``coordinate real general`` and ``coordinate real
symmetric`` files (the symmetric form stores one triangle; it is expanded),
sums duplicate entries as Eigen's triplet assembly does, and returns the same
CSR (row_ptr u32, col u32, val f64).  ``write_p_matrix`` writes a
``coordinate real general`` file (1-based indices, 17 significant digits, so
values round-trip exactly).
"""
from __future__ import annotations

import numpy as np


def _header(f):
    first = f.readline()
    if not first.lower().startswith("%%matrixmarket"):
        raise ValueError("not a Matrix Market file")
    tok = first.split()
    if len(tok) < 5 or tok[1].lower() != "matrix" or tok[2].lower() != "coordinate":
        raise ValueError("only coordinate matrices are supported")
    field, sym = tok[3].lower(), tok[4].lower()
    if field not in ("real", "double", "integer"):
        raise ValueError(f"unsupported field {field!r}")
    if sym not in ("general", "symmetric"):
        raise ValueError(f"unsupported symmetry {sym!r}")
    line = f.readline()
    while line.startswith("%") or not line.strip():
        line = f.readline()
        if not line:
            raise ValueError("missing size line")
    nr, nc, nnz = (int(v) for v in line.split())
    return sym, nr, nc, nnz


def read_p_matrix(path):
    with open(path, "r") as f:
        sym, nr, nc, nnz = _header(f)
        body = np.array(f.read().split(), dtype=np.float64)
    if nr != nc:
        raise ValueError("P must be square")
    if body.size != 3 * nnz:
        raise ValueError(f"expected {nnz} entries, found {body.size / 3:g}")
    e = body.reshape(nnz, 3)
    r = e[:, 0].astype(np.int64) - 1
    c = e[:, 1].astype(np.int64) - 1
    v = e[:, 2]
    if nnz and (r.min() < 0 or c.min() < 0 or r.max() >= nr or c.max() >= nc):
        raise ValueError("index out of range")
    if sym == "symmetric":
        off = r != c
        r, c, v = np.concatenate([r, c[off]]), np.concatenate([c, r[off]]), np.concatenate([v, v[off]])
    # setupEfficientPmatrix: entry (r, c) becomes row c, column r; rows then columns sorted
    rows, cols = c, r
    key = rows * nc + cols
    order = np.argsort(key, kind="stable")
    key, v = key[order], v[order]
    uniq, start = np.unique(key, return_index=True)
    vals = np.add.reduceat(v, start) if len(v) else v
    rr = uniq // nc
    row_ptr = np.zeros(nr + 1, np.int64)
    np.add.at(row_ptr, rr + 1, 1)
    return np.cumsum(row_ptr).astype(np.uint32), (uniq % nc).astype(np.uint32), vals.astype(np.float64)


def write_p_matrix(path, row_ptr, col, val, comment: str = ""):
    row_ptr = np.asarray(row_ptr, np.int64)
    n = len(row_ptr) - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(row_ptr))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        if comment:
            for line in comment.splitlines():
                f.write(f"% {line}\n")
        f.write(f"{n} {n} {len(col)}\n")
        # stored as (column, row) so that reading takes the transpose back
        data = np.column_stack([np.asarray(col, np.int64) + 1, rows + 1])
        for (a, b), x in zip(data.tolist(), np.asarray(val, np.float64).tolist()):
            f.write(f"{a} {b} {x!r}\n")
