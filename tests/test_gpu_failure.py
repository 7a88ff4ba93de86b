"""Failure paths, made to happen on the host side or through bounded waits
that are told to give up -- no GPU fault, trap or endless wait is involved.

* The value pass's wait for a window's column copy, and the batched
  engine's grid barriers, are bounded.  The `wait_polls` test hook of
  hsmu_opts makes them give up after one poll: the call must report
  HSMU_ERR_TIMEOUT, and the same handle must then compute the exact product.
* hsmu_debug_fail_alloc makes the nth device allocation fail: every call
  must return HSMU_ERR_ALLOC (or succeed, when it needs fewer allocations)
  and leave the device memory pool's in-use bytes where they were.
"""
import ctypes

import numpy as np
import pytest

import oracle
from hsmu_gb import gen

pytestmark = pytest.mark.gpu

HSMU_ERR_ALLOC = 2
HSMU_ERR_TIMEOUT = 7


def pool_used_bytes():
    """bytes in use from the device's default stream-ordered memory pool
    (what the library allocates from), after the device has finished and
    unreferenced outputs of earlier tests have been released"""
    import gc

    import hsmu_gb

    gc.collect()
    hsmu_gb.load_library()
    rt = ctypes.CDLL("libcudart.so.13")
    assert rt.cudaDeviceSynchronize() == 0
    dev = ctypes.c_int()
    assert rt.cudaGetDevice(ctypes.byref(dev)) == 0
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0
    used = ctypes.c_uint64()
    CUDA_MEMPOOL_ATTR_USED_MEM_CURRENT = 7
    assert rt.cudaMemPoolGetAttribute(pool, CUDA_MEMPOOL_ATTR_USED_MEM_CURRENT, ctypes.byref(used)) == 0
    return used.value


def exact(C, A, B):
    rp, col, val = oracle.spgemm(A, B)
    np.testing.assert_array_equal(C.row_ptr.astype(np.int64), rp)
    np.testing.assert_array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def test_value_pass_copy_wait_gives_up_then_engine_recovers(engine):
    import hsmu_gb

    A = gen.rmat(15, 16, seed=2)
    dA = hsmu_gb.DeviceCSR.from_host(A)
    C = engine.spgemm(dA, dA, stats=True)
    assert engine.last_stats["windows"] > 0  # the product goes through the value pass
    C.free()
    with pytest.raises(hsmu_gb.HsmuError) as ei:
        engine.spgemm(dA, dA, wait_polls=1)
    assert ei.value.status == HSMU_ERR_TIMEOUT
    exact(engine.spgemm(dA, dA).to_host(), A, A)


def test_learned_copy_wait_gives_up_then_engine_recovers(engine):
    import torch

    import hsmu_gb
    from hsmu_gb import learned

    A = gen.rmat(15, 16, seed=2)
    dA = hsmu_gb.DeviceCSR.from_host(A)
    params, margin, _ = learned.load()
    pt = torch.from_numpy(params).cuda()
    with pytest.raises(hsmu_gb.HsmuError) as ei:
        engine.spgemm_learned(dA, dA, pt, margin, wait_polls=1)
    assert ei.value.status == HSMU_ERR_TIMEOUT
    exact(engine.spgemm_learned(dA, dA, pt, margin).to_host(), A, A)


def galerkin_inputs(sides):
    import hsmu_gb

    As, Ps, Pts = [], [], []
    for s in sides:
        As.append(hsmu_gb.gen_poisson7(s))
        P, Pt = hsmu_gb.gen_aggregation(s)
        Ps.append(P)
        Pts.append(Pt)
    return As, Ps, Pts


def test_batch_grid_barrier_gives_up_then_engine_recovers(engine):
    import hsmu_gb

    sides = [40, 7, 33, 12, 25, 3, 38, 19]
    As, Ps, Pts = galerkin_inputs(sides)
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_GALERKIN, As, Ps, Pts, wait_polls=1)
    b.execute()
    with pytest.raises(hsmu_gb.HsmuError) as ei:
        b.status()
    assert ei.value.status == HSMU_ERR_TIMEOUT
    b.close()
    good = hsmu_gb.Batch(engine, hsmu_gb.BATCH_GALERKIN, As, Ps, Pts)
    good.execute()
    good.status()
    for p in (0, 2, 6):
        A, P, Pt = As[p].to_host(), Ps[p].to_host(), Pts[p].to_host()
        rp, col, val = oracle.spgemm(A, P)
        AP = gen.CSR(A.M, P.N, rp.astype(np.int32), col, val)
        exact(good.result(p).to_host(), Pt, AP)
    good.close()


def test_every_allocation_failure_is_reported_without_leaks(engine):
    import torch

    import hsmu_gb
    from hsmu_gb import learned

    A = gen.rmat(12, 16, seed=3)
    B = gen.rmat(12, 8, seed=4)
    dA, dB = hsmu_gb.DeviceCSR.from_host(A), hsmu_gb.DeviceCSR.from_host(B)
    params, margin, _ = learned.load()
    pt = torch.from_numpy(params).cuda()
    calls = {
        "plain": lambda: engine.spgemm(dA, dB, validate=True),
        "learned": lambda: engine.spgemm_learned(dA, dB, pt, margin),
        "int64": lambda: engine.spgemm64(dA, dB, max_panel_nnz=40000),
        "transpose": lambda: engine.transpose(dA),
    }
    want = oracle.spgemm(A, B)
    base = pool_used_bytes()
    n_calls = 0
    for name, call in calls.items():
        failed = 0
        for nth in range(1, 60):
            hsmu_gb.debug_fail_alloc(nth)
            try:
                out = call()
            except hsmu_gb.HsmuError as e:
                assert e.status == HSMU_ERR_ALLOC, (name, nth, e)
                failed += 1
                out = None
            finally:
                hsmu_gb.debug_fail_alloc(0)
            n_calls += 1
            if out is not None:
                if name in ("plain", "learned"):
                    C = out.to_host()
                    np.testing.assert_array_equal(C.col, want[1])
                    assert np.array_equal(C.val.view(np.int64), want[2].view(np.int64))
                out.free()
                assert pool_used_bytes() == base, (name, nth)
                break  # the call needs fewer than nth allocations: every failure point was covered
            assert pool_used_bytes() == base, "%s leaked after failing allocation %d" % (name, nth)
        assert failed >= 3, name
    assert n_calls >= 20
