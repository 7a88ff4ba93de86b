"""The oracle pinned against the reference's own output (CPU test).

tests/golden/reference_outputs.json was produced on a GB300 by running the
reference's GPU path itself (tests/golden/make_golden.py).  The oracle must
reproduce its structure exactly (row pointers and columns, by SHA-256) and its
values within 1e-12 (the reference's atomics make its own summation order
vary)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_outputs.json")


def load():
    if not os.path.exists(GOLDEN):
        pytest.skip("golden fixtures not generated yet")
    with open(GOLDEN) as f:
        return json.load(f)


def cases():
    if not os.path.exists(GOLDEN):
        return []
    with open(GOLDEN) as f:
        return sorted(json.load(f)["cases"])


@pytest.mark.parametrize("name", cases())
def test_oracle_matches_reference_output(name):
    import sys

    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import make_case

    g = load()["cases"][name]
    A, B = make_case(name)
    rp, col, val, absv = oracle.spgemm(A, B, with_abs=True)
    assert int(rp[-1]) == g["nnz"]
    assert oracle.products(A, B) == g["products"]
    assert hashlib.sha256(rp.astype(np.int32).tobytes()).hexdigest() == g["row_ptr_sha256"]
    assert hashlib.sha256(np.ascontiguousarray(col).tobytes()).hexdigest() == g["col_sha256"]
    for r, c, v in g["sample"]:
        lo, hi = rp[r], rp[r + 1]
        k = lo + int(np.searchsorted(col[lo:hi], c))
        assert col[k] == c
        assert abs(val[k] - v) <= 1e-12 * max(abs(val[k]), absv[k])
