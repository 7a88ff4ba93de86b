"""Sampled-row parity checks of products too large to check in full --
TEST INFRASTRUCTURE ONLY (tests/ and bench.py's output self-check).

A product of the stated workload sizes (R-MAT scale 18: 1.28e9 entries,
15 GB; R-MAT scale 20: ~1e10 entries) is checked on a sample of its rows:
random blocks of consecutive rows, the rows with the most intermediate
products (they take the engine's large-row window path, the counterpart of
the reference's bin-13 dense accumulator, src/external/spECK/dense_acc.cu
:122-243), and the first and last rows.  Each sampled row is compared with
the host Gustavson oracle (gustavson.c) on exactly those rows: columns
identical, values bit for bit (the engine adds in the oracle's order), and
within the stated tolerance 1e-12 * max(|c|, sum |a||b|).
"""
from __future__ import annotations

import numpy as np

from . import spgemm

RTOL = 1e-12


def row_products(A, B) -> np.ndarray:
    """Intermediate products of every row of A*B (int64)."""
    blen = np.diff(B.row_ptr).astype(np.int64)
    cs = np.zeros(A.nnz + 1, dtype=np.int64)
    np.cumsum(blen[A.col], out=cs[1:])
    return cs[A.row_ptr[1:]] - cs[A.row_ptr[:-1]]


def sample_rows(A, B, blocks: int = 48, block: int = 32, heavy: int = 48, seed: int = 0,
                max_products: float = 4e8) -> np.ndarray:
    """Sorted unique row ids: `blocks` random runs of `block` consecutive rows,
    the `heavy` rows with the most products (while their sum stays within
    max_products, so the oracle finishes in seconds), and rows 0 and M-1."""
    M = A.M
    if M == 0:
        return np.zeros(0, dtype=np.int32)
    rng = np.random.default_rng(seed)
    parts = [np.array([0, M - 1], dtype=np.int64)]
    if M > block:
        starts = rng.integers(0, M - block + 1, size=blocks)
        parts.append((starts[:, None] + np.arange(block)[None, :]).reshape(-1))
    else:
        parts.append(np.arange(M))
    prod = row_products(A, B)
    order = np.argsort(prod, kind="stable")[::-1][:heavy]
    keep = np.cumsum(prod[order]) <= max_products
    keep[0] = True
    parts.append(order[keep])
    return np.unique(np.concatenate(parts)).astype(np.int32)


def check_rows(got, A, B, rows, fma: bool = False) -> dict:
    """got = (local row_ptr[k+1], col, val) of the sampled rows (the order of
    `rows`).  Raises AssertionError on any structural difference or a value
    beyond the tolerance; returns a summary (rows, entries, bitwise, max
    relative error)."""
    rows = np.asarray(rows, dtype=np.int32)
    grp, gcol, gval = got
    rp, col, val, absv = spgemm(A, B, rows=rows, with_abs=True, fma=fma)
    grp = np.asarray(grp, dtype=np.int64)
    if not np.array_equal(grp, rp):
        bad = np.flatnonzero(np.diff(grp) != np.diff(rp))[:5]
        raise AssertionError("row lengths differ from the oracle at sampled rows %s" % rows[bad])
    if not np.array_equal(gcol, col):
        i = int(np.flatnonzero(gcol != col)[0])
        r = int(np.searchsorted(rp, i, side="right") - 1)
        raise AssertionError("columns differ from the oracle in row %d" % rows[r])
    scale = np.maximum(np.abs(val), absv)
    err = np.abs(gval - val)
    ok = err <= RTOL * scale
    if not np.all(ok):
        i = np.flatnonzero(~ok)[:3]
        raise AssertionError("value error above %g at %d sampled entries (e.g. %r vs %r)"
                             % (RTOL, int((~ok).sum()), gval[i], val[i]))
    nz = scale > 0
    rel = float(np.max(err[nz] / scale[nz])) if np.any(nz) else 0.0
    bitwise = bool(np.array_equal(gval.view(np.int64), val.view(np.int64)))
    return {"rows": int(rows.size), "entries": int(col.size), "bitwise": bitwise, "max_rel_err": rel}
