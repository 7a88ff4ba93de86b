"""Matrix Market (coordinate) reader producing the engine's canonical CSR.

Reads the same files as the reference's loader (mmio_allinone,
src/mmio_highlevel.h:18-193) with the same value rules: `real` values as
written, `integer` converted to double, `pattern` entries as 1.0, `complex`
entries by their real part, and `symmetric` / `hermitian` matrices expanded
by mirroring every off-diagonal entry (same value).  Indices are 1-based in
the file.  Unlike the reference, which keeps each row in file order, the
result is canonical -- columns strictly increasing within each row, duplicate
entries of one position summed in file order -- because the engine's kernels
need sorted rows.
"""
from __future__ import annotations

import numpy as np

from .gen import CSR

_FIELDS = ("real", "integer", "pattern", "complex", "double")
_SYMMETRY = ("general", "symmetric", "hermitian", "skew-symmetric")


def _banner(line: str):
    parts = line.strip().split()
    if len(parts) < 5 or parts[0].lower() != "%%matrixmarket" or parts[1].lower() != "matrix":
        raise ValueError("not a Matrix Market matrix file: %r" % line.strip())
    fmt, field, symmetry = (p.lower() for p in parts[2:5])
    if fmt != "coordinate":
        raise ValueError("only coordinate (sparse) Matrix Market files are supported, got %r" % fmt)
    if field not in _FIELDS:
        raise ValueError("unsupported Matrix Market field %r" % field)
    if symmetry not in _SYMMETRY:
        raise ValueError("unsupported Matrix Market symmetry %r" % symmetry)
    return field, symmetry


def _parse_numbers(text: str) -> np.ndarray:
    """whitespace-separated numbers of the entry lines as float64"""
    return np.array(text.split(), dtype=np.float64)


def read_mtx(path: str) -> CSR:
    """Canonical CSR (int32 row pointers and columns, float64 values) of a .mtx file."""
    with open(path, "r") as f:
        field, symmetry = _banner(f.readline())
        line = f.readline()
        while line and (line.startswith("%") or not line.strip()):
            line = f.readline()
        if not line:
            raise ValueError("missing size line")
        M, N, nnz = (int(x) for x in line.split()[:3])
        data = _parse_numbers(f.read()) if nnz else np.zeros(0)
    per = {"pattern": 2, "complex": 4}.get(field, 3)
    if data.size < per * nnz:
        raise ValueError("file holds %d numbers, %d entries of %d expected" % (data.size, nnz, per))
    data = data[: per * nnz].reshape(nnz, per)
    rows = data[:, 0].astype(np.int64) - 1
    cols = data[:, 1].astype(np.int64) - 1
    vals = np.ones(nnz) if field == "pattern" else data[:, 2].astype(np.float64)
    if nnz and (rows.min() < 0 or cols.min() < 0 or rows.max() >= M or cols.max() >= N):
        raise ValueError("entry index outside the %d x %d matrix" % (M, N))
    if symmetry in ("symmetric", "hermitian"):
        off = rows != cols
        rows, cols, vals = (np.concatenate([rows, cols[off]]), np.concatenate([cols, rows[off]]),
                            np.concatenate([vals, vals[off]]))
    return coo_to_csr(M, N, rows, cols, vals)


def coo_to_csr(M: int, N: int, rows, cols, vals) -> CSR:
    """Canonical CSR from coordinate triplets; duplicates summed in input order."""
    rows = np.asarray(rows, np.int64)
    cols = np.asarray(cols, np.int64)
    vals = np.asarray(vals, np.float64)
    key = rows * N + cols
    order = np.argsort(key, kind="stable")
    key, vals = key[order], vals[order]
    if key.size:
        head = np.empty(key.size, bool)
        head[0] = True
        head[1:] = key[1:] != key[:-1]
        starts = np.flatnonzero(head)
        ends = np.append(starts[1:], key.size)
        summed = vals[starts].copy()
        for r in np.flatnonzero(ends - starts > 1):  # duplicates (rare): left to right, in input order
            acc = 0.0
            for v in vals[starts[r]:ends[r]]:
                acc = acc + float(v)
            summed[r] = acc
        key, vals = key[starts], summed
    r = (key // N).astype(np.int64) if N else np.zeros(0, np.int64)
    c = (key % N).astype(np.int32) if N else np.zeros(0, np.int32)
    rp = np.zeros(M + 1, np.int64)
    np.add.at(rp, r + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    return CSR(M, N, rp, c, vals)


def write_mtx(path: str, A: CSR, symmetric: bool = False) -> None:
    """Write A as a `coordinate real general` file (or `symmetric`: lower triangle only)."""
    rows = np.repeat(np.arange(A.M, dtype=np.int64), np.diff(A.row_ptr))
    cols = A.col.astype(np.int64)
    vals = A.val
    if symmetric:
        keep = rows >= cols
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
    with open(path, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate real %s\n" % ("symmetric" if symmetric else "general"))
        f.write("%d %d %d\n" % (A.M, A.N, rows.size))
        for i, j, v in zip(rows, cols, vals):
            f.write("%d %d %.17g\n" % (i + 1, j + 1, v))
