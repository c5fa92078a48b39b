"""Seeded synthetic sparse matrices in RACE's input layout.

Every generator returns a :class:`Csr` with int32 ``row_ptr``/``col`` and float64
``val``, the diagonal entry first in each row and the remaining columns in
ascending order (the layout RACE's Gauss-Seidel and SymmSpMV kernels assume
after ``makeDiagFirst``, examples/src/helpers/sparsemat.cpp:432-546). Random
numbers come from ``numpy.random.Generator(PCG64(seed))`` so x86 and Arm hosts
produce identical matrices.

Workloads (the public suite matrices the reference measured on are not
available; these stand in with the same shapes and value distributions):

* ``laplace3d_7pt(32)``: 3D 7-point Laplacian, diagonal 6, off-diagonals -1.
* ``stencil3d_27pt(128)``: 27-point stencil on 128^3 (the HPCG-128 shape),
  symmetric off-diagonals U[-1,0), diagonal = sum|off| + 1.
* ``powerlaw_chung_lu(n)``: symmetric Chung-Lu graph, Pareto(2.1) weights with
  mean degree 16, off-diagonals N(0,1) mirrored, diagonal = sum|off| + 1.
* ``aniso2d(nx, ny, points, ratio)``: 2D 5/9-point anisotropic stencil.
* ``banded_scrambled(n, bw)``: random banded symmetric matrix whose rows are
  scrambled by a random permutation.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Csr:
    n: int
    row_ptr: np.ndarray  # int32 [n+1]
    col: np.ndarray  # int32 [nnz]
    val: np.ndarray  # float64 [nnz]
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1])

    def upper(self) -> "Csr":
        """Upper triangle including the diagonal, diagonal first
        (``computeSymmData``, examples/src/helpers/sparsemat.cpp:581-632)."""
        rows = np.repeat(np.arange(self.n, dtype=np.int64), np.diff(self.row_ptr))
        keep = self.col >= rows
        counts = np.bincount(rows[keep], minlength=self.n)
        rp = np.zeros(self.n + 1, dtype=np.int32)
        np.cumsum(counts, out=rp[1:])
        return Csr(self.n, rp, self.col[keep].copy(), self.val[keep].copy(), self.name + "_upper")

    def permuted(self, perm: np.ndarray, inv_perm: np.ndarray) -> "Csr":
        """Symmetric permutation the way RACE's users apply it
        (``sparsemat::permute``, examples/src/helpers/sparsemat.cpp:990-1078):
        new row i is old row perm[i]; each column c becomes inv_perm[c]; the
        order of entries inside a row is kept."""
        perm = np.asarray(perm, dtype=np.int64)
        lens = np.diff(self.row_ptr)[perm]
        rp = np.zeros(self.n + 1, dtype=np.int32)
        np.cumsum(lens, out=rp[1:])
        starts = self.row_ptr[:-1][perm].astype(np.int64)
        idx = np.repeat(starts - rp[:-1], lens) + np.arange(rp[-1], dtype=np.int64)
        col = np.asarray(inv_perm, dtype=np.int32)[self.col[idx]]
        return Csr(self.n, rp, col.astype(np.int32), self.val[idx].copy(), self.name + "_perm")

    def to_dense(self) -> np.ndarray:
        a = np.zeros((self.n, self.n))
        rows = np.repeat(np.arange(self.n), np.diff(self.row_ptr))
        np.add.at(a, (rows, self.col), self.val)
        return a


def _assemble(n: int, rows: np.ndarray, cols: np.ndarray, vals: np.ndarray, diag: np.ndarray, name: str) -> Csr:
    """Build a diagonal-first CRS from off-diagonal triplets (no duplicates)."""
    rows = rows.astype(np.int64)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    counts = np.bincount(rows, minlength=n) + 1
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    nnz = int(rp[-1])
    col = np.empty(nnz, dtype=np.int32)
    val = np.empty(nnz, dtype=np.float64)
    col[rp[:-1]] = np.arange(n, dtype=np.int32)
    val[rp[:-1]] = diag
    # position of each off-diagonal: row start + 1 + rank within its row
    first = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts - 1, out=first[1:])
    rank = np.arange(rows.size, dtype=np.int64) - first[rows]
    pos = rp[rows] + 1 + rank
    col[pos] = cols
    val[pos] = vals
    if rp[-1] >= 2**31:
        raise ValueError("matrix too large for int32 indices")
    return Csr(n, rp.astype(np.int32), col, val, name)


def _grid_offsets(dim: int, points: int):
    if dim == 3 and points == 7:
        return [(dx, dy, dz) for dx, dy, dz in
                [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)]]
    if dim == 3 and points == 27:
        return [(dx, dy, dz) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)
                if (dx, dy, dz) != (0, 0, 0)]
    raise ValueError("unsupported stencil")


def _stencil3d_pairs(nx: int, ny: int, nz: int, points: int):
    """Upper (c > r) neighbour pairs of a 3D stencil; r = x + nx*(y + ny*z)."""
    n = nx * ny * nz
    idx = np.arange(n, dtype=np.int64)
    x = idx % nx
    y = (idx // nx) % ny
    z = idx // (nx * ny)
    rs, cs = [], []
    for dx, dy, dz in _grid_offsets(3, points):
        off = dx + nx * (dy + ny * dz)
        if off <= 0:
            continue
        ok = (x + dx >= 0) & (x + dx < nx) & (y + dy >= 0) & (y + dy < ny) & (z + dz >= 0) & (z + dz < nz)
        r = idx[ok]
        rs.append(r)
        cs.append(r + off)
    return n, np.concatenate(rs), np.concatenate(cs)


def laplace3d_7pt(nx: int, ny: int | None = None, nz: int | None = None) -> Csr:
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n, r, c = _stencil3d_pairs(nx, ny, nz, 7)
    rows = np.concatenate([r, c])
    cols = np.concatenate([c, r]).astype(np.int32)
    vals = np.full(rows.size, -1.0)
    return _assemble(n, rows, cols, vals, np.full(n, 6.0), f"lap7_{nx}x{ny}x{nz}")


def stencil3d_27pt(nx: int, ny: int | None = None, nz: int | None = None, seed: int = 0) -> Csr:
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n, r, c = _stencil3d_pairs(nx, ny, nz, 27)
    rng = np.random.Generator(np.random.PCG64(seed))
    v = -rng.random(r.size)  # U[-1, 0)
    v = np.where(v == 0.0, -0.5, v)
    rows = np.concatenate([r, c])
    cols = np.concatenate([c, r]).astype(np.int32)
    vals = np.concatenate([v, v])
    absum = np.bincount(rows, weights=np.abs(vals), minlength=n)
    return _assemble(n, rows, cols, vals, absum + 1.0, f"st27_{nx}x{ny}x{nz}")


def powerlaw_chung_lu(n: int, mean_degree: float = 16.0, alpha: float = 2.1, seed: int = 0) -> Csr:
    """Symmetric Chung-Lu graph: edge (i,j) present with p = min(1, w_i w_j / S).
    Sampled by drawing ~n*mean/2 endpoint pairs proportionally to the weights
    (the standard fast Chung-Lu approximation), then removing self loops and
    duplicates."""
    rng = np.random.Generator(np.random.PCG64(seed))
    w = rng.pareto(alpha - 1.0, n) + 1.0
    w *= mean_degree / w.mean()
    m = int(n * mean_degree / 2)
    p = w / w.sum()
    cdf = np.cumsum(p)
    cdf[-1] = 1.0
    a = np.searchsorted(cdf, rng.random(m), side="right").astype(np.int64)
    b = np.searchsorted(cdf, rng.random(m), side="right").astype(np.int64)
    a = np.minimum(a, n - 1)
    b = np.minimum(b, n - 1)
    keep = a != b
    a, b = a[keep], b[keep]
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = np.unique(lo * n + hi)
    lo, hi = key // n, key % n
    v = rng.standard_normal(lo.size)
    rows = np.concatenate([lo, hi])
    cols = np.concatenate([hi, lo]).astype(np.int32)
    vals = np.concatenate([v, v])
    absum = np.bincount(rows, weights=np.abs(vals), minlength=n)
    return _assemble(n, rows, cols, vals, absum + 1.0, f"plaw_{n}")


def aniso2d(nx: int, ny: int, points: int = 5, ratio: float = 10.0) -> Csr:
    """2D anisotropic diffusion stencil: coupling -1 in x and -ratio in y
    (5-point), plus -sqrt(ratio)/2 on the diagonals (9-point); diagonal =
    sum|off| (+ 1e-3 for strict dominance)."""
    n = nx * ny
    idx = np.arange(n, dtype=np.int64)
    x = idx % nx
    y = idx // nx
    offs = [(1, 0, 1.0), (0, 1, ratio)]
    if points == 9:
        d = 0.5 * np.sqrt(ratio)
        offs += [(1, 1, d), (-1, 1, d)]
    elif points != 5:
        raise ValueError("points must be 5 or 9")
    rs, cs, vs = [], [], []
    for dx, dy, coef in offs:
        ok = (x + dx >= 0) & (x + dx < nx) & (y + dy < ny)
        r = idx[ok]
        rs.append(r)
        cs.append(r + dx + nx * dy)
        vs.append(np.full(r.size, -coef))
    r, c, v = np.concatenate(rs), np.concatenate(cs), np.concatenate(vs)
    rows = np.concatenate([r, c])
    cols = np.concatenate([c, r]).astype(np.int32)
    vals = np.concatenate([v, v])
    absum = np.bincount(rows, weights=np.abs(vals), minlength=n)
    return _assemble(n, rows, cols, vals, absum + 1e-3, f"aniso{points}_{nx}x{ny}_{ratio:g}")


def banded_scrambled(n: int, bandwidth: int, seed: int = 0, fill: float = 0.5) -> Csr:
    """Random symmetric banded matrix (each offset 1..bandwidth kept with
    probability ``fill``), rows then scrambled by a random permutation."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rs, cs = [], []
    base = np.arange(n, dtype=np.int64)
    for off in range(1, bandwidth + 1):
        r = base[: n - off]
        keep = rng.random(r.size) < fill
        rs.append(r[keep])
        cs.append(r[keep] + off)
    r, c = np.concatenate(rs), np.concatenate(cs)
    v = rng.standard_normal(r.size)
    perm = rng.permutation(n)
    r, c = perm[r], perm[c]
    rows = np.concatenate([r, c])
    cols = np.concatenate([c, r]).astype(np.int32)
    vals = np.concatenate([v, v])
    absum = np.bincount(rows, weights=np.abs(vals), minlength=n)
    return _assemble(n, rows, cols, vals, absum + 1.0, f"band{bandwidth}_{n}")


def uniform_vector(n: int, seed: int = 0, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(lo, hi, n)


def aniso2d_batch(count: int, seed: int = 0, lo: int = 100, hi: int = 700):
    """``count`` 2D anisotropic stencils of uneven size: grid nx, ny drawn
    from U{lo..hi}, 5- or 9-point with equal odds, coefficient ratio
    log-uniform on [1, 100] (PCG64 seeded)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mats = []
    for _ in range(count):
        nx, ny = (int(v) for v in rng.integers(lo, hi + 1, size=2))
        pts = 5 if rng.random() < 0.5 else 9
        ratio = float(np.exp(rng.uniform(0.0, np.log(100.0))))
        mats.append(aniso2d(nx, ny, pts, ratio))
    return mats


def uniform_block(n: int, nrhs: int, seed: int = 0) -> np.ndarray:
    """n x nrhs right-hand sides, U[-1,1] (PCG64 seeded), row-major."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(-1.0, 1.0, size=(n, nrhs))


def islands(seed: int = 0) -> Csr:
    """Disconnected pieces with isolated rows: a 6^3 7-point Laplacian (216
    rows), a 12 x 9 anisotropic 5-point stencil (108 rows) and 6 rows holding
    only their diagonal, rows scrambled by a seeded permutation (330 rows)."""
    parts = [laplace3d_7pt(6), aniso2d(12, 9, 5, 4.0)]
    rows, cols, vals, diag, off = [], [], [], [], 0
    for P in parts:
        r = np.repeat(np.arange(P.n), np.diff(P.row_ptr))
        keep = r != P.col
        rows.append(r[keep] + off)
        cols.append(P.col[keep].astype(np.int64) + off)
        vals.append(P.val[keep])
        d = np.zeros(P.n)
        dm = ~keep
        d[r[dm]] = P.val[dm]
        diag.append(d)
        off += P.n
    diag.append(np.full(6, 2.0))
    n = off + 6
    rows, cols, vals, diag = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals), np.concatenate(diag)
    perm = np.random.Generator(np.random.PCG64(seed)).permutation(n)  # new index of old row i
    return _assemble(n, perm[rows], perm[cols].astype(np.int32), vals, diag[np.argsort(perm)], "islands_330")


def chain_with_empty_rows(n: int = 300, empty=(0, 150, 299)) -> Csr:
    """1D Laplacian chain whose rows in `empty` hold no entry at all (not
    even a diagonal): edge cases for traversal and the matrix power."""
    r = np.arange(n - 1)
    rows = np.concatenate([r, r + 1])
    cols = np.concatenate([r + 1, r])
    e = np.asarray(empty)
    keep = ~(np.isin(rows, e) | np.isin(cols, e))
    rows, cols = rows[keep], cols[keep].astype(np.int32)
    vals = np.full(rows.size, -1.0)
    B = _assemble(n, rows, cols, vals, np.full(n, 2.0), f"chain{n}_empty")
    # drop the diagonal of the empty rows
    rl = np.diff(B.row_ptr)
    r_of = np.repeat(np.arange(n), rl)
    keep = ~np.isin(r_of, e)
    rp = np.zeros(n + 1, np.int32)
    np.cumsum(np.bincount(r_of[keep], minlength=n), out=rp[1:])
    return Csr(n, rp, B.col[keep].astype(np.int32), B.val[keep].copy(), B.name)
