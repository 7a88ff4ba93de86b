"""Row panels of the host-buffer call (hsmu_spgemm_host), planned on the host:
the cuts follow the output bytes (shares that double to the middle and halve
again when the copy back is the longer part, shrinking by 0.7 otherwise), and
the panels run in the two-stage flow-shop order of Johnson's rule -- panels
whose copy is the longer part first, by increasing compute, then the others by
decreasing copy.  Host-only: no GPU needed."""
import ctypes

import numpy as np
import pytest

LINK_BOUND = 1.5  # output bytes per intermediate product at which copy and compute take as long
CHUNK = 64


@pytest.fixture(scope="module")
def lib():
    from hsmu_gb import build

    build.build()
    import hsmu_gb

    return hsmu_gb.load_library()


def plan(lib, rp, products, chunk, panels=0):
    rp = np.ascontiguousarray(rp, dtype=np.int32)
    M = len(rp) - 1
    n = ctypes.c_int32()
    cut = (ctypes.c_int32 * 9)()
    order = (ctypes.c_int32 * 8)()
    ch = None if chunk is None else np.ascontiguousarray(chunk, dtype=np.int64)
    rc = lib.hsmu_debug_plan_panels(M, rp.ctypes.data, int(products), None if ch is None else ch.ctypes.data,
                                    panels, ctypes.byref(n), cut, order)
    assert rc == 0
    return list(cut[:n.value + 1]), list(order[:n.value])


def chunks_of(row_products):
    M = len(row_products)
    pad = np.zeros((M + CHUNK - 1) // CHUNK * CHUNK, dtype=np.int64)
    pad[:M] = row_products
    return pad.reshape(-1, CHUNK).sum(axis=1)


def johnson(cut, rp, row_products, order):
    """the order's panels: copy-longer ones first by increasing compute, then the rest by decreasing copy"""
    comp = [float(np.sum(row_products[cut[q]:cut[q + 1]])) for q in range(len(cut) - 1)]
    copy = [12.0 * (rp[cut[q + 1]] - rp[cut[q]]) / LINK_BOUND for q in range(len(cut) - 1)]
    link = [q for q in order if comp[q] < copy[q]]
    rest = [q for q in order if comp[q] >= copy[q]]
    assert order[:len(link)] == link, "copy-longer panels come first"
    assert all(comp[a] <= comp[b] for a, b in zip(link, link[1:]))
    assert all(copy[a] >= copy[b] for a, b in zip(rest, rest[1:]))


def valid_cuts(cut, M, np_expected):
    assert cut[0] == 0 and cut[-1] == M and len(cut) == np_expected + 1
    assert all(a <= b for a, b in zip(cut, cut[1:]))


def test_compute_longer_product_keeps_row_order_and_shrinking_panels(lib):
    # 200k rows of 100 entries (240 MB of output, 8 panels) and 20 products per entry
    M = 200_000
    rp = np.arange(M + 1, dtype=np.int64) * 100
    rowp = np.full(M, 2000, dtype=np.int64)
    cut, order = plan(lib, rp, rowp.sum(), chunks_of(rowp))
    valid_cuts(cut, M, 8)
    assert order == list(range(8))
    sizes = np.diff(cut)
    assert all(sizes[q] > sizes[q + 1] for q in range(6))  # shares 0.7^q
    johnson(cut, rp, rowp, order)


def test_copy_longer_uniform_product_starts_with_a_smallest_panel(lib):
    # one product per output entry: the copy is the longer part; shares 1,2,4,8,8,4,2,1
    M = 200_000
    rp = np.arange(M + 1, dtype=np.int64) * 100
    rowp = np.full(M, 100, dtype=np.int64)
    cut, order = plan(lib, rp, rowp.sum(), chunks_of(rowp))
    valid_cuts(cut, M, 8)
    sizes = np.diff(cut)
    assert sizes[order[0]] == sizes.min() and sizes[order[-1]] == sizes.max()
    johnson(cut, rp, rowp, order)


def test_hub_rows_go_last(lib):
    # power-law-like: the first rows hold most of the products for few output bytes
    M = 200_000
    rp = np.arange(M + 1, dtype=np.int64) * 100
    rowp = np.full(M, 50, dtype=np.int64)
    rowp[:500] = 200_000
    cut, order = plan(lib, rp, rowp.sum(), chunks_of(rowp))
    valid_cuts(cut, M, 8)
    assert 12.0 * rp[-1] > LINK_BOUND * rowp.sum()  # the copy is the longer part overall
    assert order[0] != 0 and order[-1] == 0  # the hub panel runs last
    johnson(cut, rp, rowp, order)


def test_without_products_the_panels_run_in_row_order(lib):
    M = 100_000
    rp = np.arange(M + 1, dtype=np.int64) * 100
    cut, order = plan(lib, rp, 10**7, None, panels=5)
    valid_cuts(cut, M, 5)
    assert order == list(range(5))


@pytest.mark.parametrize("panels", [1, 3, 8, 32])
def test_explicit_panel_counts_and_small_inputs(lib, panels):
    rng = np.random.default_rng(panels)
    for M in (1, 2, 7, 65, 1000):
        rp = np.concatenate([[0], np.cumsum(rng.integers(0, 40, M))])
        rowp = rng.integers(0, 500, M)
        cut, order = plan(lib, rp, int(rowp.sum()), chunks_of(rowp), panels=panels)
        valid_cuts(cut, M, min(panels, 8, M))
        assert sorted(order) == list(range(len(order)))
