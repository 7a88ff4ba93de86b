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


def noalloc_tiles(B):
    """Tiles of host matrix B through the no-alloc entry point (C ABI)."""
    import torch

    import hsmu_gb

    L = hsmu_gb.load_library()
    dB = hsmu_gb.DeviceCSR.from_host(B)
    cap = max(B.nnz, 1)
    tile_ptr = torch.full((B.M + 1,), -7, dtype=torch.int32, device="cuda")
    tile_col = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
    mask = torch.zeros(cap, dtype=torch.int64, device="cuda")
    tile_off = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
    rc = L.hsmu_btiles_build_noalloc(ctypes.byref(dB.desc), tile_ptr.data_ptr(), tile_col.data_ptr(),
                                     mask.data_ptr(), tile_off.data_ptr(),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
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
