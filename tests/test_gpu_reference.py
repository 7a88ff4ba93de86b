"""The engine against the reference's own GPU output (oracle/_ref harness,
compiled from the reference sources on this machine): identical structure,
values within 1e-12 (the reference adds with shared-memory atomics, so its
own summation order varies run to run)."""
import numpy as np
import pytest

import oracle
from hsmu_gb import gen
from oracle import ref_run

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_run.available(), reason="reference harness not built here")]


def engine_run(engine, A, B):
    import hsmu_gb

    dA = hsmu_gb.DeviceCSR.from_host(A)
    dB = dA if B is A else hsmu_gb.DeviceCSR.from_host(B)
    C = engine.spgemm(dA, dB)
    out = C.to_host()
    C.free()
    return out


@pytest.mark.parametrize("name", ["lap64", "st12", "rmat12", "rmat12T", "rect"])
def test_engine_matches_reference(engine, name):
    if name == "lap64":
        A = B = gen.laplacian2d(64, seed=0)
    elif name == "st12":
        A = B = gen.stencil27(12, 3, seed=1)
    elif name == "rmat12":
        A = B = gen.rmat(12, 16, seed=2)
    elif name == "rmat12T":
        A = gen.rmat(12, 16, seed=2)
        B = gen.transpose(A)
    else:
        A = gen.poisson_random(3000, 10, seed=21, ncols=6000)
        B = gen.poisson_random(6000, 8, seed=22, ncols=9000)
    R, info = ref_run.run(A, None if B is A else B, reps=1)
    C = engine_run(engine, A, B)
    np.testing.assert_array_equal(C.row_ptr, R.row_ptr)
    np.testing.assert_array_equal(C.col, R.col)
    _, _, val, absv = oracle.spgemm(A, B, with_abs=True)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))
    err = np.abs(R.val - C.val) / np.maximum(np.abs(C.val), absv)
    assert err.max() <= 1e-12
