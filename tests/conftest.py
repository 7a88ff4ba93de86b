"""Shared test setup: import paths, the `gpu` marker, and small helpers.

CPU tests (-m "not gpu") cover the oracle against its pins, the workload
generators, the host layer and the C ABI's exported symbols.  GPU tests
(-m gpu) are the parity tests proper: they run the engine through the C ABI
and compare with the oracle.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "hsmu-spgemm_gb300")
for p in (ROOT, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) device and the built engine")


# Value tolerance of the parity tests: the engine accumulates in the oracle's
# order and should match bit for bit; the bar is 1e-12 relative, scaled by
# sum |a||b| for entries whose terms cancel.
RTOL = 1e-12


def assert_csr_equal(C, ref, absv=None, rtol=RTOL, exact=True):
    """C: gen.CSR from the engine; ref: (row_ptr, col, val) from the oracle."""
    rp, col, val = ref
    np.testing.assert_array_equal(C.row_ptr.astype(np.int64), rp.astype(np.int64))
    np.testing.assert_array_equal(C.col, col)
    if exact:
        bad = np.flatnonzero(C.val.view(np.int64) != val.view(np.int64))
        if bad.size and absv is None:
            raise AssertionError("values differ bitwise at %d entries (first %s: %r vs %r)"
                                 % (bad.size, bad[:3], C.val[bad[:3]], val[bad[:3]]))
    scale = np.maximum(np.abs(val), absv if absv is not None else np.abs(val))
    err = np.abs(C.val - val)
    ok = err <= rtol * scale
    if not np.all(ok):
        i = np.flatnonzero(~ok)[:5]
        raise AssertionError("value error above %g at %d entries, e.g. %s: %r vs %r"
                             % (rtol, int((~ok).sum()), i, C.val[i], val[i]))


@pytest.fixture(scope="session")
def engine():
    import hsmu_gb

    return hsmu_gb.Engine()
