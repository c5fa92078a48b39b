"""MatrixMarket ingestion as RACE's example driver does it
(examples/src/helpers/sparsemat.cpp: readFile :108-279, makeDiagFirst
:431-546; examples/src/helpers/mmio.cpp: mm_read_unsymmetric_sparse :15-105).

Host code: it runs once per matrix and hands the engine host CRS arrays.

* Accepted: ``coordinate`` (sparse) ``real`` or ``pattern`` matrices,
  ``general`` or ``symmetric``, square. Pattern entries get the value 0.01.
* A symmetric file is expanded: every off-diagonal entry (r, c) is followed
  by its mirror (c, r).
* Entries are stably sorted by row, so within a row they keep the file order.
* ``.gz`` files are read transparently (the reference reads plain files).
"""
from __future__ import annotations

import gzip
import pathlib

import numpy as np

from .matgen import Csr

PATTERN_VALUE = 0.01  # mmio.cpp:68-76


def _open(path):
    path = pathlib.Path(path)
    return gzip.open(path, "rt") if path.suffix == ".gz" else open(path, "r")


def read_matrix_market(path) -> Csr:
    """sparsemat::readFile: the CRS matrix of a MatrixMarket file (see the
    module docstring for what is accepted). Raises ValueError otherwise."""
    with _open(path) as f:
        banner = f.readline().split()
        if len(banner) < 5 or banner[0].lower() != "%%matrixmarket" or banner[1].lower() != "matrix":
            raise ValueError("not a MatrixMarket matrix file")
        fmt, field, symm = (b.lower() for b in banner[2:5])
        if fmt != "coordinate" or field not in ("real", "pattern") or symm not in ("general", "symmetric"):
            raise ValueError(f"unsupported MatrixMarket type: {fmt} {field} {symm} (needs coordinate, real or "
                             "pattern, general or symmetric)")
        line = f.readline()
        while line.startswith("%") or not line.strip():
            line = f.readline()
        nrows, ncols, nnz = (int(v) for v in line.split()[:3])
        data = np.array(f.read().split(), dtype=np.float64)
    width = 2 if field == "pattern" else 3
    if data.size < nnz * width:
        raise ValueError("premature end of the MatrixMarket file")
    data = data[: nnz * width].reshape(nnz, width)
    if nrows != ncols:
        raise ValueError("matrix not square")
    row = data[:, 0].astype(np.int64) - 1
    col = data[:, 1].astype(np.int64) - 1
    val = np.full(nnz, PATTERN_VALUE) if field == "pattern" else data[:, 2].copy()
    if symm == "symmetric":
        # each entry, then its mirror right after it when off the diagonal
        off = row != col
        rep = np.where(off, 2, 1)
        pos = np.concatenate([[0], np.cumsum(rep)[:-1]])
        total = int(rep.sum())
        r2, c2, v2 = np.empty(total, np.int64), np.empty(total, np.int64), np.empty(total)
        r2[pos], c2[pos], v2[pos] = row, col, val
        r2[pos[off] + 1], c2[pos[off] + 1], v2[pos[off] + 1] = col[off], row[off], val[off]
        row, col, val = r2, c2, v2
    order = np.argsort(row, kind="stable")
    row, col, val = row[order], col[order], val[order]
    rp = np.zeros(nrows + 1, np.int64)
    np.cumsum(np.bincount(row, minlength=nrows), out=rp[1:])
    return Csr(nrows, rp.astype(np.int32), col.astype(np.int32), val, pathlib.Path(path).name)


def make_diag_first(csr: Csr, missing_diag_value: float = 0.0, rewrite_all_diag_with_max_row_sum: bool = False) -> Csr:
    """sparsemat::makeDiagFirst, for Gauss-Seidel-like kernels: rows without
    a diagonal entry get one (value missing_diag_value) at their end, then
    each row's diagonal entry moves to its first slot, the entries before it
    shifting one slot right (a row is assumed to hold one diagonal entry, as
    MatrixMarket files do not repeat entries). With rewrite_all_diag_with_max_row_sum
    every diagonal becomes the largest |row sum| (row sums taken left to
    right after the insertion)."""
    n = csr.n
    lens = np.diff(csr.row_ptr).astype(np.int64)
    rows = np.repeat(np.arange(n), lens)
    is_diag = csr.col == rows
    missing = np.ones(n, bool)
    missing[rows[is_diag]] = False
    # append the missing diagonals at the end of their rows
    lens2 = lens + missing
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(lens2, out=rp[1:])
    col = np.empty(int(rp[-1]), np.int64)
    val = np.empty(int(rp[-1]))
    local = np.arange(rows.size) - csr.row_ptr[:-1][rows]
    col[rp[rows] + local] = csr.col
    val[rp[rows] + local] = csr.val
    mrows = np.flatnonzero(missing)
    col[rp[mrows + 1] - 1] = mrows
    val[rp[mrows + 1] - 1] = missing_diag_value
    max_row_sum = 0.0
    if rewrite_all_diag_with_max_row_sum:
        for r in range(n):
            row_sum = 0.0
            for x in val[rp[r]:rp[r + 1]]:
                row_sum += x
            max_row_sum = max(max_row_sum, abs(row_sum))
    # move each row's first diagonal entry to the front
    rows2 = np.repeat(np.arange(n), lens2)
    local2 = np.arange(rows2.size) - rp[rows2]
    hits = np.flatnonzero(col == rows2)
    hit_rows, first = np.unique(rows2[hits], return_index=True)  # every row has one now
    diag_at = np.empty(n, np.int64)
    diag_at[hit_rows] = local2[hits[first]]
    d = diag_at[rows2]
    new_local = np.where(local2 == d, 0, np.where(local2 < d, local2 + 1, local2))
    col_out = np.empty_like(col)
    val_out = np.empty_like(val)
    col_out[rp[rows2] + new_local] = col
    val_out[rp[rows2] + new_local] = val
    if rewrite_all_diag_with_max_row_sum:
        val_out[rp[:-1]] = max_row_sum
    return Csr(n, rp.astype(np.int32), col_out.astype(np.int32), val_out, csr.name)


def rcm_perm(csr):
    """A reverse Cuthill-McKee ordering to pass as the Interface's initPerm
    (new row i = old row perm[i]) with its inverse. The reference's examples
    take RCM from SpMP (CMakeLists.txt:294-323), a third-party library that
    is not part of RACE; this one is SciPy's, so the ordering itself can
    differ from SpMP's. The pattern is symmetrised first."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee

    n = csr.n
    S = sp.csr_matrix((np.ones(len(csr.col)), np.asarray(csr.col), np.asarray(csr.row_ptr)), shape=(n, n))
    perm = np.asarray(reverse_cuthill_mckee((S + S.T).tocsr(), symmetric_mode=True), np.int32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(n, dtype=np.int32)
    return perm, inv
