"""Row-block sharding of C = A*B over several GPUs (one process per GPU).

Rows of A -- and with them rows of C -- are independent: row i of C needs
row i of A and the B rows it references.  A product is therefore split into
contiguous row blocks of A, balanced by intermediate products (the work of a
row), and every GPU computes C for its block against its own full copy of B
(no peer memory access, no remote loads).  The only exchange is the number
of entries of each shard: an all-gather of one int64 per rank gives every
rank where its rows start in the global C, which is all a caller needs to
place the shards in one CSR (stitch below does it on the host).

The reference runs on one GPU only (src/NHC_spgemm.cuh:7; its 14 streams
all live on one device, src/loading.cuh:55-59); this is the partition that
its row-independent stages admit.
"""
from __future__ import annotations

import numpy as np

from .gen import CSR


def row_products(A: CSR, B: CSR) -> np.ndarray:
    """intermediate products of every row of A*B (int64)"""
    blen = np.diff(B.row_ptr).astype(np.int64)
    cs = np.zeros(A.nnz + 1, dtype=np.int64)
    np.cumsum(blen[A.col], out=cs[1:])
    return cs[A.row_ptr[1:]] - cs[A.row_ptr[:-1]]


def row_blocks(A: CSR, B: CSR, parts: int) -> np.ndarray:
    """cuts[0..parts]: block r holds rows cuts[r] .. cuts[r+1]-1.  Each cut is
    the first row at which the running product count reaches r/parts of the
    total, so blocks carry about equal work; blocks may be empty."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    cum = np.zeros(A.M + 1, dtype=np.int64)
    np.cumsum(row_products(A, B), out=cum[1:])
    total = int(cum[-1])
    targets = [(total * r + parts - 1) // parts for r in range(parts + 1)]
    cuts = np.searchsorted(cum, targets, side="left").astype(np.int64)
    cuts[0], cuts[-1] = 0, A.M
    return np.maximum.accumulate(np.minimum(cuts, A.M))


def host_block(A: CSR, r0: int, r1: int) -> CSR:
    """rows r0..r1-1 of A as a CSR of its own (row pointers rebased to 0)"""
    e0, e1 = int(A.row_ptr[r0]), int(A.row_ptr[r1])
    return CSR(r1 - r0, A.N, (A.row_ptr[r0:r1 + 1] - e0).astype(np.int32), A.col[e0:e1], A.val[e0:e1])


def device_block(dA, r0: int, r1: int):
    """rows r0..r1-1 of a device CSR as a view (its row pointers are not
    rebased: the engine reads entries from row_ptr[0] on, as given)"""
    from . import DeviceCSR, c_csr

    d = dA.desc
    return DeviceCSR(c_csr(r1 - r0, d.N, d.nnz, 0, d.row_ptr + 4 * r0, d.col, d.val), keep=dA)


def global_offsets(shard_nnz) -> np.ndarray:
    """exclusive scan of the per-shard entry counts (the result of the
    all-gather): shard r's entries start at offsets[r] of the global C"""
    n = np.asarray(shard_nnz, dtype=np.int64)
    out = np.zeros(n.size + 1, dtype=np.int64)
    np.cumsum(n, out=out[1:])
    return out


def stitch(shards, N: int):
    """one CSR (int64 row pointers) from the shards' (row_ptr, col, val), in
    rank order; each shard's row_ptr starts at 0"""
    offs = global_offsets([int(s[0][-1]) for s in shards])
    rp = [np.zeros(1, dtype=np.int64)]
    for (srp, _, _), o in zip(shards, offs[:-1]):
        rp.append(np.asarray(srp[1:], dtype=np.int64) + o)
    col = np.concatenate([np.asarray(s[1], dtype=np.int32) for s in shards]) if shards else np.zeros(0, np.int32)
    val = np.concatenate([np.asarray(s[2], dtype=np.float64) for s in shards]) if shards else np.zeros(0)
    return np.concatenate(rp), col, val
