"""Seeded synthetic sparse matrices for the SpGEMM workloads (int32 CSR, FP64).

The reference measures on SuiteSparse matrices that are not available here;
these generators stand in for them with the shapes, sizes and value
distributions of the measured workloads:

* ``laplacian2d(256, seed=0)`` -- 5-point stencil on a 256x256 grid,
  n = 65,536, nnz = 326,656, values uniform(-1, 1).
* ``stencil27(40, dof=3, seed=1)`` -- 27-point stencil on a 40^3 grid with
  full 3x3 node blocks, n = 192,000, nnz = 14,787,288, values uniform(-1, 1).
* ``rmat(18, 16, seed=2)`` -- R-MAT graph, 2^18 rows, 16 * 2^18 sampled edges,
  quadrant probabilities (0.57, 0.19, 0.19, 0.05), duplicate edges merged,
  values uniform(0, 1).
* ``poisson_random`` -- rows with Poisson(lambda) uniformly placed columns.
* ``poisson7`` / ``aggregation_prolongator`` -- 7-point Poisson matrix on a
  cubic grid and the piecewise-constant 2x2x2 aggregation prolongator of an
  AMG Galerkin product P^T (A P).

Every matrix is returned as a :class:`CSR` with strictly increasing column
indices in each row (the canonical form the engine requires).  numpy's PCG64
generator gives identical streams on x86_64 and aarch64, so a seed names the
same matrix on every machine.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class CSR:
    """Host CSR matrix: int32 row_ptr/col, float64 val, shape (M, N)."""

    M: int
    N: int
    row_ptr: np.ndarray
    col: np.ndarray
    val: np.ndarray

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1])

    def row_nnz(self) -> np.ndarray:
        return np.diff(self.row_ptr)

    def check(self) -> None:
        """Raise ValueError unless this is canonical int32 CSR."""
        rp, c = self.row_ptr, self.col
        if rp.dtype != np.int32 or c.dtype != np.int32 or self.val.dtype != np.float64:
            raise ValueError("CSR must be int32/int32/float64")
        if rp.shape != (self.M + 1,) or rp[0] != 0 or np.any(np.diff(rp) < 0):
            raise ValueError("bad row_ptr")
        if c.shape != (self.nnz,) or self.val.shape != (self.nnz,):
            raise ValueError("col/val length != nnz")
        if self.nnz and (c.min() < 0 or c.max() >= self.N):
            raise ValueError("column index out of range")
        if self.nnz > 1:
            d = np.diff(c.astype(np.int64))
            starts = rp[1:-1]
            boundary = np.zeros(self.nnz - 1, dtype=bool)
            boundary[starts[(starts > 0) & (starts < self.nnz)] - 1] = True
            if np.any(~boundary & (d <= 0)):
                raise ValueError("columns not strictly increasing within a row")

    def to_scipy(self):
        import scipy.sparse as sp

        return sp.csr_matrix((self.val, self.col, self.row_ptr), shape=(self.M, self.N))


def _from_coo_sorted_unique(M: int, N: int, key: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """key = row * N + col, sorted and unique -> (row_ptr, col) int32."""
    rows = (key // N).astype(np.int64)
    cols = (key % N).astype(np.int32)
    counts = np.bincount(rows, minlength=M)
    rp = np.zeros(M + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    if rp[-1] > np.iinfo(np.int32).max:
        raise ValueError("nnz does not fit int32")
    return rp.astype(np.int32), cols


def _sorted_unique(key: np.ndarray) -> np.ndarray:
    """np.unique of an int64 array by an in-place sort and a neighbour test (the
    same result; np.unique measured ~80x slower on 16M keys)."""
    key.sort()
    if key.size < 2:
        return key
    keep = np.empty(key.size, dtype=bool)
    keep[0] = True
    np.not_equal(key[1:], key[:-1], out=keep[1:])
    return key[keep]


def laplacian2d(side: int, seed: int = 0, lo: float = -1.0, hi: float = 1.0) -> CSR:
    """5-point stencil on a side x side grid, natural ordering."""
    n = side * side
    idx = np.arange(n, dtype=np.int64)
    x, y = idx % side, idx // side
    keys = [idx * n + idx]
    for dx, dy in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        ok = (x + dx >= 0) & (x + dx < side) & (y + dy >= 0) & (y + dy < side)
        keys.append(idx[ok] * n + (idx[ok] + dx + dy * side))
    key = np.sort(np.concatenate(keys))
    rp, col = _from_coo_sorted_unique(n, n, key)
    val = np.random.default_rng(seed).uniform(lo, hi, size=col.shape[0])
    return CSR(n, n, rp, col, val)


def stencil27(side: int, dof: int = 3, seed: int = 1, lo: float = -1.0, hi: float = 1.0) -> CSR:
    """27-point stencil on a side^3 grid with full dof x dof node blocks.

    Row r = node * dof + d; node = x + side * (y + side * z).  Every pair of
    neighbouring nodes (including a node with itself) contributes a dense
    dof x dof block.
    """
    nodes = side ** 3
    n = nodes * dof
    nid = np.arange(nodes, dtype=np.int64)
    x, y, z = nid % side, (nid // side) % side, nid // (side * side)
    # neighbour offsets in increasing node-index order: dz major, then dy, dx
    nbr_lists = []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                ok = ((x + dx >= 0) & (x + dx < side) & (y + dy >= 0) & (y + dy < side)
                      & (z + dz >= 0) & (z + dz < side))
                nb = np.where(ok, nid + dx + side * (dy + side * dz), -1)
                nbr_lists.append(nb)
    nbr = np.stack(nbr_lists, axis=1)  # (nodes, 27): ascending node ids, -1 where absent
    # per node: its column list nb*dof + e (ascending), padded with -1
    cols_node = np.where(nbr[:, :, None] >= 0, nbr[:, :, None] * dof + np.arange(dof)[None, None, :], -1)
    cols_node = cols_node.reshape(nodes, 27 * dof)
    cnt = (nbr >= 0).sum(axis=1) * dof
    rows = np.repeat(cols_node, dof, axis=0).reshape(-1)  # each node's list once per dof row
    col = rows[rows >= 0].astype(np.int32)
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.repeat(cnt, dof), out=rp[1:])
    if rp[-1] > np.iinfo(np.int32).max:
        raise ValueError("nnz does not fit int32")
    val = np.random.default_rng(seed).uniform(lo, hi, size=col.shape[0])
    return CSR(n, n, rp.astype(np.int32), col, val)


def rmat(scale: int, edge_factor: int = 16, seed: int = 2,
         probs: tuple[float, float, float, float] = (0.57, 0.19, 0.19, 0.05),
         lo: float = 0.0, hi: float = 1.0) -> CSR:
    """R-MAT graph with duplicate edges merged.

    For each of the scale bit levels (most significant first) every edge picks
    a quadrant with probabilities (a, b, c, d): a = (row bit 0, col bit 0),
    b = (0, 1), c = (1, 0), d = (1, 1).  Values are drawn after merging, in
    CSR order.
    """
    n = 1 << scale
    ne = n * edge_factor
    a, b, c, _ = probs
    rng = np.random.default_rng(seed)
    row = np.zeros(ne, dtype=np.int64)
    col = np.zeros(ne, dtype=np.int64)
    for lev in range(scale):
        r = rng.random(ne)
        bit = 1 << (scale - 1 - lev)
        rbit = r >= a + b                       # quadrants c, d
        cbit = ((r >= a) & (r < a + b)) | (r >= a + b + c)  # quadrants b, d
        row += rbit * bit
        col += cbit * bit
    row *= n
    row += col
    del col
    key = _sorted_unique(row)
    del row
    rp, cidx = _from_coo_sorted_unique(n, n, key)
    val = rng.uniform(lo, hi, size=cidx.shape[0])
    return CSR(n, n, rp, cidx, val)


def poisson_random(n: int, lam: float, seed: int, ncols: int | None = None,
                   lo: float = -1.0, hi: float = 1.0) -> CSR:
    """n rows, nnz per row ~ Poisson(lam), columns uniform without repeats."""
    ncols = n if ncols is None else ncols
    rng = np.random.default_rng(seed)
    k = np.minimum(rng.poisson(lam, size=n), ncols).astype(np.int64)
    rows = np.repeat(np.arange(n, dtype=np.int64), k)
    cols = rng.integers(0, ncols, size=rows.shape[0], dtype=np.int64)
    key = _sorted_unique(rows * ncols + cols)
    rp, cidx = _from_coo_sorted_unique(n, ncols, key)
    val = rng.uniform(lo, hi, size=cidx.shape[0])
    return CSR(n, ncols, rp, cidx, val)


def poisson7(side: int, seed: int | None = None) -> CSR:
    """7-point Poisson matrix on a side^3 grid: 6 on the diagonal, -1 off it.

    With a seed, values are uniform(-1, 1) instead (same structure)."""
    n = side ** 3
    nid = np.arange(n, dtype=np.int64)
    x, y, z = nid % side, (nid // side) % side, nid // (side * side)
    keys = [nid * n + nid]
    for off, ok in ((-side * side, z > 0), (-side, y > 0), (-1, x > 0),
                    (1, x < side - 1), (side, y < side - 1), (side * side, z < side - 1)):
        keys.append(nid[ok] * n + nid[ok] + off)
    key = np.sort(np.concatenate(keys))
    rp, col = _from_coo_sorted_unique(n, n, key)
    if seed is None:
        rows = np.repeat(np.arange(n), np.diff(rp))
        val = np.where(col == rows, 6.0, -1.0)
    else:
        val = np.random.default_rng(seed).uniform(-1.0, 1.0, size=col.shape[0])
    return CSR(n, n, rp, col, val)


def aggregation_prolongator(side: int) -> CSR:
    """Piecewise-constant prolongator for 2x2x2 aggregation of a side^3 grid.

    Fine node (x, y, z) maps to coarse node (x//2, y//2, z//2) of a
    ceil(side/2)^3 grid with weight 1.0; one entry per row."""
    n = side ** 3
    cs = (side + 1) // 2
    nid = np.arange(n, dtype=np.int64)
    x, y, z = nid % side, (nid // side) % side, nid // (side * side)
    col = (x // 2 + cs * (y // 2 + cs * (z // 2))).astype(np.int32)
    rp = np.arange(n + 1, dtype=np.int32)
    return CSR(n, cs ** 3, rp, col, np.ones(n, dtype=np.float64))


def transpose(A: CSR) -> CSR:
    """A^T with sorted columns (stable counting sort)."""
    rows = np.repeat(np.arange(A.M, dtype=np.int64), np.diff(A.row_ptr))
    order = np.argsort(A.col, kind="stable")
    counts = np.bincount(A.col, minlength=A.N)
    rp = np.zeros(A.N + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    return CSR(A.N, A.M, rp.astype(np.int32), rows[order].astype(np.int32), A.val[order].copy())


def products(A: CSR, B: CSR) -> int:
    """Intermediate products sum_{(i,k) in A} nnz(B(k,:)) (64-bit)."""
    blen = np.diff(B.row_ptr).astype(np.int64)
    return int(blen[A.col].sum())


def compulsory_bytes(A: CSR, B: CSR, c_nnz: int, c_rows: int) -> int:
    """Algorithmic bytes: read A and B once, write C once (int32 + FP64)."""
    return (4 * (A.M + 1) + 12 * A.nnz) + (4 * (B.M + 1) + 12 * B.nnz) + (4 * (c_rows + 1) + 12 * c_nnz)


WORKLOADS = {
    "laplacian2d_256": lambda: (laplacian2d(256, seed=0),) * 2,
    "stencil27_40_dof3": lambda: (stencil27(40, 3, seed=1),) * 2,
    "rmat18_AA": lambda: (lambda A: (A, A))(rmat(18, 16, seed=2)),
    "rmat18_AAt": lambda: (lambda A: (A, transpose(A)))(rmat(18, 16, seed=2)),
}
