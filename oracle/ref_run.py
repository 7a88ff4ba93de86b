"""Run the reference HSMU-SpGEMM GPU path through oracle/_ref/ref_harness.

TEST INFRASTRUCTURE ONLY (parity pinning against the reference's own output,
and timing of the reference on the same GPU).  Needs a GPU and the harness
built by oracle/ref_build.py.
"""
from __future__ import annotations

import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_ref", "ref_harness")


def available() -> bool:
    return os.path.exists(BIN)


def _write(path, A):
    with open(path, "wb") as f:
        np.array([A.M, A.N, A.nnz], dtype=np.int32).tofile(f)
        np.ascontiguousarray(A.row_ptr, dtype=np.int32).tofile(f)
        np.ascontiguousarray(A.col, dtype=np.int32).tofile(f)
        np.ascontiguousarray(A.val, dtype=np.float64).tofile(f)


def _read(path):
    from hsmu_gb.gen import CSR

    with open(path, "rb") as f:
        M, N, nnz = (int(x) for x in np.fromfile(f, dtype=np.int32, count=3))
        rp = np.fromfile(f, dtype=np.int32, count=M + 1)
        col = np.fromfile(f, dtype=np.int32, count=nnz)
        val = np.fromfile(f, dtype=np.float64, count=nnz)
    return CSR(M, N, rp, col, val)


def run(A, B=None, reps: int = 2, timeout: float = 1800.0, output: bool = True):
    """C = A*B with the reference (B=None: a second copy of A, as its driver
    does for C = A*A).  Returns (C, info) with info = {call_ms: [...],
    time2_ms: [...], conversion_ms: [...]} -- time2 is the reference's own
    timed region (symbolic + allocation + columns + values, no setup or B
    conversion, src/compressed/compressed_NHC_spgemm.cu:35-202).  output=False
    only times the calls (C is None): nothing is copied back or written."""
    if not available():
        raise FileNotFoundError(BIN)
    with tempfile.TemporaryDirectory() as td:
        a, b, c = (os.path.join(td, x) for x in ("A.bin", "B.bin", "C.bin"))
        _write(a, A)
        if B is not None:
            _write(b, B)
        # the reference appends CSV lines to ../../data/*.csv relative to its cwd
        cwd = os.path.join(td, "w", "x")
        os.makedirs(cwd)
        os.makedirs(os.path.join(td, "data"))
        r = subprocess.run([BIN, a, b if B is not None else "same", c if output else "none", str(reps)], cwd=cwd,
                           capture_output=True, text=True, timeout=timeout)
        out = r.stdout
        if r.returncode != 0:
            raise RuntimeError("reference harness failed (%d): %s\n%s" % (r.returncode, out[-2000:],
                                                                          r.stderr[-2000:]))
        info = {
            "call_ms": [float(x) for x in re.findall(r"HARNESS_CALL_MS ([0-9.]+)", out)],
            "time2_ms": [float(x) for x in re.findall(r"the total run time of NHC_spgemm is ([0-9.]+) ms", out)],
            "conversion_ms": [float(x) for x in
                              re.findall(r"the run time for Initialize_compressed_mask64_matrix is ([0-9.]+)", out)],
        }
        return (_read(c) if output else None), info
