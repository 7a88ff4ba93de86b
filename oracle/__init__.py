"""CPU oracle for the HSMU SpGEMM path -- TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check in __graft_entry__.py and the cpu_baseline /
``--impl reference`` legs of bench.py may import this package.  The engine
(include/hsmu_gb.h, libhsmu_gb.so) never calls it, and it is never the thing
measured as the GPU result.

``gustavson.c`` is the host FP64 Gustavson restatement of the reference's
C = A*B semantics (see its header for the reference file:line anchors); this
module compiles it into ``liboracle.so`` and wraps it with ctypes.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "gustavson.c")

_lib = None


def build(force: bool = False) -> str:
    """Compile gustavson.c with OpenMP and without FMA contraction."""
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(SRC):
        tmp = SO + ".tmp%d" % os.getpid()
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
               "-shared", "-o", tmp, SRC, "-lm"]
        subprocess.check_call(cmd)
        os.replace(tmp, SO)
    return SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(SO)
        P = ctypes.c_void_p
        I = ctypes.c_int
        L.oracle_products.restype = ctypes.c_uint64
        L.oracle_products.argtypes = [I, P, P, P]
        L.oracle_symbolic.restype = I
        L.oracle_symbolic.argtypes = [I, P, I, P, P, P, P, P, I]
        L.oracle_numeric.restype = I
        L.oracle_numeric.argtypes = [I, P, I, P, P, P, P, P, P, P, P, P, I]
        L.oracle_numeric_fma.restype = I
        L.oracle_numeric_fma.argtypes = [I, P, I, P, P, P, P, P, P, P, P, P, I]
        L.oracle_abs_numeric.restype = I
        L.oracle_abs_numeric.argtypes = [I, P, I, P, P, P, P, P, P, P, P, P, I]
        L.oracle_transpose.restype = I
        L.oracle_transpose.argtypes = [I, I, P, P, P, P, P, P]
        L.oracle_max_threads.restype = I
        _lib = L
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def max_threads() -> int:
    return lib().oracle_max_threads()


def products(A, B) -> int:
    return int(lib().oracle_products(A.M, _p(A.row_ptr), _p(A.col), _p(B.row_ptr)))


def spgemm(A, B, rows: np.ndarray | None = None, nthreads: int = 0, with_abs: bool = False,
           fma: bool = False):
    """C = A*B on the host (rows=None: all rows; else only the listed rows).
    fma=True accumulates with one rounding per product (c = fma(a, b, c)).

    Returns (row_ptr int64[nrows+1], col int32[nnz], val float64[nnz]) and,
    with with_abs, also sum |a||b| per entry."""
    if A.N != B.M:
        raise ValueError("inner dimensions differ")
    L = lib()
    if rows is not None:
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        nrows = rows.shape[0]
    else:
        nrows = A.M
    cnt = np.zeros(nrows, dtype=np.int64)
    rc = L.oracle_symbolic(nrows, _p(rows), B.N, _p(A.row_ptr), _p(A.col), _p(B.row_ptr),
                           _p(B.col), _p(cnt), nthreads)
    if rc:
        raise MemoryError("oracle_symbolic failed: %d" % rc)
    rp = np.zeros(nrows + 1, dtype=np.int64)
    np.cumsum(cnt, out=rp[1:])
    col = np.empty(int(rp[-1]), dtype=np.int32)
    val = np.empty(int(rp[-1]), dtype=np.float64)
    num = L.oracle_numeric_fma if fma else L.oracle_numeric
    rc = num(nrows, _p(rows), B.N, _p(A.row_ptr), _p(A.col), _p(A.val),
             _p(B.row_ptr), _p(B.col), _p(B.val), _p(rp), _p(col), _p(val), nthreads)
    if rc:
        raise MemoryError("oracle_numeric failed: %d" % rc)
    if not with_abs:
        return rp, col, val
    absv = np.empty_like(val)
    rc = L.oracle_abs_numeric(nrows, _p(rows), B.N, _p(A.row_ptr), _p(A.col), _p(A.val),
                              _p(B.row_ptr), _p(B.col), _p(B.val), _p(rp), _p(col), _p(absv),
                              nthreads)
    if rc:
        raise MemoryError("oracle_abs_numeric failed: %d" % rc)
    return rp, col, val, absv


def symbolic(A, B, rows: np.ndarray | None = None, nthreads: int = 0) -> np.ndarray:
    """nnz per output row (int64)."""
    L = lib()
    if rows is not None:
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        nrows = rows.shape[0]
    else:
        nrows = A.M
    cnt = np.zeros(nrows, dtype=np.int64)
    rc = L.oracle_symbolic(nrows, _p(rows), B.N, _p(A.row_ptr), _p(A.col), _p(B.row_ptr),
                           _p(B.col), _p(cnt), nthreads)
    if rc:
        raise MemoryError("oracle_symbolic failed: %d" % rc)
    return cnt


def transpose(A):
    """(row_ptr, col, val) of A^T with sorted columns."""
    trp = np.empty(A.N + 1, dtype=np.int32)
    tcol = np.empty(A.nnz, dtype=np.int32)
    tval = np.empty(A.nnz, dtype=np.float64)
    rc = lib().oracle_transpose(A.M, A.N, _p(A.row_ptr), _p(A.col), _p(A.val), _p(trp),
                                _p(tcol), _p(tval))
    if rc:
        raise MemoryError("oracle_transpose failed")
    return trp, tcol, tval
