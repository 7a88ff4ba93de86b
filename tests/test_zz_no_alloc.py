"""hsmu_btiles_build_noalloc: the B tile conversion for callers that cannot
allocate device memory (their memory belongs to their own pool or a fixed
budget).  It must give exactly what the allocating hsmu_btiles_build gives,
call after call, although every call reuses the same static scratch.

This file is named to be collected last, and it needs no state from other
tests: it passes alone in a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

from hsmu_gb import gen

pytestmark = pytest.mark.gpu


HSMU_ERR_UNSORTED = 5


def noalloc_call(B, slack=0):
    """Status of the no-alloc entry point (C ABI) on host matrix B and its output
    arrays.  slack: extra entries after every device array (the malformed cases
    below keep every access in bounds even if the checks did not run)."""
    import torch

    import hsmu_gb

    L = hsmu_gb.load_library()
    rp = torch.from_numpy(np.ascontiguousarray(B.row_ptr, dtype=np.int32)).cuda()
    col = torch.zeros(B.col.size + slack, dtype=torch.int32, device="cuda")
    col[:B.col.size] = torch.from_numpy(np.ascontiguousarray(B.col, dtype=np.int32)).cuda()
    val = torch.zeros(B.col.size + slack, dtype=torch.float64, device="cuda")
    desc = hsmu_gb.c_csr(B.M, B.N, int(B.col.size), 0, rp.data_ptr(), col.data_ptr(), val.data_ptr())
    cap = max(B.col.size, 1) + slack
    tile_ptr = torch.full((B.M + 1 + slack,), -7, dtype=torch.int32, device="cuda")
    tile_col = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
    mask = torch.zeros(cap, dtype=torch.int64, device="cuda")
    tile_off = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
    rc = L.hsmu_btiles_build_noalloc(ctypes.byref(desc), tile_ptr.data_ptr(), tile_col.data_ptr(),
                                     mask.data_ptr(), tile_off.data_ptr(),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc, (tile_ptr, tile_col, mask, tile_off)


def noalloc_tiles(B):
    """Tiles of host matrix B through the no-alloc entry point (C ABI)."""
    import hsmu_gb

    rc, (tile_ptr, tile_col, mask, tile_off) = noalloc_call(B)
    assert rc == 0, hsmu_gb.load_library().hsmu_strerror(rc)
    tp = tile_ptr.cpu().numpy()
    T = int(tp[-1])
    return (tp, tile_col[:T].cpu().numpy(), mask[:T].cpu().numpy().view(np.uint64),
            tile_off[:T].cpu().numpy())


def allocating_tiles(engine, B):
    import hsmu_gb

    bt = hsmu_gb.BTiles(engine, hsmu_gb.DeviceCSR.from_host(B))
    out = bt.arrays()
    bt.free()
    return out


def test_noalloc_matches_allocating_entry_point_twice(engine):
    # two calls in a row on different matrices share (and must reset) the scratch
    for B in (gen.rmat(13, 16, seed=2), gen.stencil27(10, 3, seed=1)):
        got = noalloc_tiles(B)
        want = allocating_tiles(engine, B)
        assert got[0][-1] == want[1].size
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)


def test_noalloc_rejects_too_many_rows():
    import torch

    import hsmu_gb

    L = hsmu_gb.load_library()
    M = (1 << 24) + 1
    rp = torch.zeros(M + 1, dtype=torch.int32, device="cuda")
    desc = hsmu_gb.c_csr(M, 8, 0, 0, rp.data_ptr(), 0, 0)
    rc = L.hsmu_btiles_build_noalloc(ctypes.byref(desc), rp.data_ptr(), 0, 0, 0, None)
    assert rc == 4  # HSMU_ERR_OVERFLOW: beyond the static scratch's row limit


def test_noalloc_rejects_bad_input_then_recovers(engine):
    # a failed call leaves its error bits in the shared control word; the next
    # valid call must clear them and give the allocating entry point's tiles
    good = gen.rmat(11, 8, seed=4)
    unsorted = gen.CSR(good.M, good.N, good.row_ptr.copy(), good.col.copy(), good.val.copy())
    r = int(np.argmax(np.diff(good.row_ptr)))  # a row with several entries
    lo = int(good.row_ptr[r])
    unsorted.col[lo], unsorted.col[lo + 1] = unsorted.col[lo + 1], unsorted.col[lo]
    rc, _ = noalloc_call(unsorted)
    assert rc == HSMU_ERR_UNSORTED
    out_of_range = gen.CSR(good.M, good.N, good.row_ptr.copy(), good.col.copy(), good.val.copy())
    out_of_range.col[lo] = good.N + 3
    rc, _ = noalloc_call(out_of_range, slack=64)
    assert rc == HSMU_ERR_UNSORTED
    # row_ptr[M] past nnz: rejected before any tile kernel indexes through it
    bad_rp = gen.CSR(good.M, good.N, good.row_ptr.copy(), good.col.copy(), good.val.copy())
    bad_rp.row_ptr[-1] = good.nnz + 5
    rc, _ = noalloc_call(bad_rp, slack=64)
    assert rc == HSMU_ERR_UNSORTED
    got = noalloc_tiles(good)
    want = allocating_tiles(engine, good)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
