"""Learned row scheduler: FP32 kernels against the FP64 restatement, training,
and the speculative SpGEMM path against the plain engine (bit for bit)."""
import os

import numpy as np
import pytest

import oracle
from hsmu_gb import gen
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def rand_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(mlp_ref.NTOTAL, np.float32)
    p[:mlp_ref.NPARAM] = rng.normal(0, 0.3, mlp_ref.NPARAM)
    p[mlp_ref.O_MU:mlp_ref.O_SD] = [3.0, 8.0, 5.0, 12.0]
    p[mlp_ref.O_SD:mlp_ref.O_YMU] = [1.5, 3.0, 2.0, 4.0]
    p[mlp_ref.O_YMU] = 7.0
    p[mlp_ref.O_YSD] = 2.5
    return p


def rand_data(n, seed=1):
    rng = np.random.default_rng(seed)
    X = np.abs(rng.normal([3, 8, 5, 12], [1.5, 3, 2, 4], size=(n, 4))).astype(np.float32)
    y = (0.6 * X[:, 1] + 0.2 * X[:, 3] + rng.normal(0, 0.3, n)).astype(np.float32)
    return X, y


def test_mlp_forward_matches_fp64():
    from hsmu_gb import learned

    p = rand_params()
    X, _ = rand_data(5000)
    got = learned.predict(p, X)
    want = mlp_ref.forward(p.astype(np.float64), X)
    assert np.max(np.abs(got - want)) <= 1e-4 * (1 + np.max(np.abs(want)))


def test_mlp_gradient_matches_fp64():
    import torch

    import hsmu_gb

    L = hsmu_gb.load_library()
    p = rand_params(2)
    X, y = rand_data(3000, 3)
    g = torch.zeros(mlp_ref.NPARAM, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    pd, Xd, yd = (torch.from_numpy(a).cuda() for a in (p, X, y))
    assert L.hsmu_mlp_grad(pd.data_ptr(), Xd.data_ptr(), yd.data_ptr(), X.shape[0], g.data_ptr(),
                           loss.data_ptr(), None) == 0
    torch.cuda.synchronize()
    want_loss, want = mlp_ref.loss_and_grad(p.astype(np.float64), X, y)
    got = g.cpu().numpy().astype(np.float64)
    assert abs(loss.item() - want_loss) <= 1e-4 * want_loss
    err = np.abs(got - want) / (np.abs(want) + 1e-3 * np.max(np.abs(want)))
    assert err.max() <= 1e-3, (err.argmax(), got[err.argmax()], want[err.argmax()])


def test_training_reduces_loss(engine):
    from hsmu_gb import learned

    X, y = learned.collect(engine, nmat=18, rows_per_matrix=96, seed=5, workers=1)
    assert X.shape[0] > 200 and np.all(np.isfinite(X))
    params, hist = learned.train(X, y, epochs=12, batch=512, lr=3e-3, seed=1)
    assert hist[-1] < 0.5 * hist[0]
    pred = learned.predict(params, X)
    assert np.mean(np.abs(pred - y)) < 1.0  # within a factor of 2 of nnz on average


def model_for_tests(engine):
    from hsmu_gb import learned

    if os.path.exists(learned.DEFAULT_MODEL):
        p, margin, _ = learned.load()
        return p, margin
    X, y = learned.collect(engine, nmat=24, rows_per_matrix=128, seed=7, workers=1)
    p, _ = learned.train(X, y, epochs=15, batch=512, lr=3e-3)
    return p, learned.choose_margin(p, X, y, 0.99)


def run_both(engine, A, B, params, margin, always=False):
    import torch

    import hsmu_gb

    dA = hsmu_gb.DeviceCSR.from_host(A)
    dB = dA if B is A else hsmu_gb.DeviceCSR.from_host(B)
    P = engine.spgemm(dA, dB).to_host()
    pt = torch.from_numpy(np.ascontiguousarray(params, np.float32)).cuda()
    Cd = engine.spgemm_learned(dA, dB, pt, margin, stats=True, always=always)
    st = engine.last_stats
    return P, Cd.to_host(), st


@pytest.mark.parametrize("always", [False, True])
@pytest.mark.parametrize("name", ["lap", "st27", "rmat12", "rmat13T", "rect", "wide"])
def test_learned_identical_to_plain(engine, name, always):
    # always: the prediction is used whatever the rows (the routing to the plain path is off),
    # so the speculative passes run on every input
    p, margin = model_for_tests(engine)
    if name == "lap":
        A = B = gen.laplacian2d(64, seed=0)
    elif name == "st27":
        A = B = gen.stencil27(10, 3, seed=1)
    elif name == "rmat12":
        A = B = gen.rmat(12, 16, seed=2, lo=-1.0, hi=1.0)
    elif name == "rmat13T":
        A = gen.rmat(13, 16, seed=2)
        B = gen.transpose(A)
    elif name == "rect":
        A = gen.poisson_random(3000, 12, seed=5, ncols=50000)
        B = gen.poisson_random(50000, 6, seed=6, ncols=70000)
    else:
        A = gen.poisson_random(400, 40, seed=7, ncols=2000)
        B = gen.poisson_random(2000, 60, seed=8, ncols=1_200_000)
    P, C, st = run_both(engine, A, B, p, margin, always)
    np.testing.assert_array_equal(C.row_ptr, P.row_ptr)
    np.testing.assert_array_equal(C.col, P.col)
    assert np.array_equal(C.val.view(np.int64), P.val.view(np.int64))
    assert st["nnz_c"] == P.nnz
    if always:
        assert st["routed"] == 0


def test_learned_fma_mode(engine):
    import torch

    import hsmu_gb

    p, margin = model_for_tests(engine)
    A = gen.rmat(12, 16, seed=6, lo=-1.0, hi=1.0)
    dA = hsmu_gb.DeviceCSR.from_host(A)
    pt = torch.from_numpy(np.ascontiguousarray(p, np.float32)).cuda()
    C = engine.spgemm_learned(dA, dA, pt, margin, arith=hsmu_gb.ARITH_FMA).to_host()
    rp, col, val = oracle.spgemm(A, A, fma=True)
    np.testing.assert_array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def test_learned_all_rows_fall_back(engine):
    # a model that predicts nothing fits: every non-tiny row is redone, result unchanged
    p, _ = model_for_tests(engine)
    # R-MAT 15: every row in the warp class (at most 512 tiles of span), many above the fused
    # limit: not handed to the plain path, and every row's slot is too small
    A = gen.rmat(15, 16, seed=4, lo=-1.0, hi=1.0)
    P, C, st = run_both(engine, A, A, p, -40.0)
    assert not st["routed"]
    assert st["fallback_rows"] > 0
    np.testing.assert_array_equal(C.col, P.col)
    assert np.array_equal(C.val.view(np.int64), P.val.view(np.int64))
    rp, col, val = oracle.spgemm(A, A)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def test_trained_model_sizes_slots_tighter_than_the_bound(engine):
    # what the network gains: slot memory close to nnz(C), instead of the product-count bound
    p, margin = model_for_tests(engine)
    A = gen.stencil27(14, 3, seed=1)
    P, C, st = run_both(engine, A, A, p, margin, always=True)
    prods = gen.products(A, A)
    assert st["spec_capacity"] < 0.25 * prods           # the bound would allocate `prods` entries
    assert st["fallback_rows"] <= 0.15 * A.M            # boundary rows of a small grid are the hardest


@pytest.mark.parametrize("name", ["lap", "st27", "rmat16"])
def test_inputs_the_prediction_cannot_help_go_to_the_plain_path(engine, name):
    # every row tiny (Laplacian); warp rows none of which is predicted above the fused warp
    # path (stencil); wide rows all of the large class, whose exact count builds the tile
    # lists the structure pass streams (R-MAT scale 16, 1,024 tiles of columns): the plain
    # path finishes the product on the same tiles and bounds
    p, margin = model_for_tests(engine)
    A = {"lap": lambda: gen.laplacian2d(96, seed=0), "st27": lambda: gen.stencil27(12, 3, seed=1),
         "rmat16": lambda: gen.rmat(16, 16, seed=2)}[name]()
    P, C, st = run_both(engine, A, A, p, margin)
    assert st["routed"] == 1
    np.testing.assert_array_equal(C.row_ptr, P.row_ptr)
    np.testing.assert_array_equal(C.col, P.col)
    assert np.array_equal(C.val.view(np.int64), P.val.view(np.int64))


def test_learned_is_faster_where_it_skips_the_count_pass(engine):
    # What the prediction saves is the exact count of the rows that end up in numeric
    # windows.  For warp-class rows (tile span <= 512) that count is a second OR walk
    # over B's tiles, which the learned path skips: R-MAT scale 15, whose C rows reach
    # thousands of entries within 32768 columns.  (Large-class rows keep their tile
    # list from the count pass, which the structure pass then streams, so there the
    # prediction has nothing to skip and both paths do the same work.)  Median of 5
    # CUDA-event timings each, outputs bit for bit equal.
    import statistics

    import torch

    import hsmu_gb
    from hsmu_gb import learned

    A = gen.rmat(15, 16, seed=2)
    dA = hsmu_gb.DeviceCSR.from_host(A)
    params, margin, _ = learned.load()
    pt = torch.from_numpy(params).cuda()
    st = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(2):
            fn().free()
        ts = []
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            C = fn()
            e1.record(st)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
            C.free()
        return statistics.median(ts)

    t_plain = timed(lambda: engine.spgemm(dA, dA))
    t_learned = timed(lambda: engine.spgemm_learned(dA, dA, pt, margin))
    assert t_learned < t_plain, (t_learned, t_plain)
    P = engine.spgemm(dA, dA).to_host()
    L = engine.spgemm_learned(dA, dA, pt, margin, stats=True)
    assert engine.last_stats["routed"] == 0
    L = L.to_host()
    np.testing.assert_array_equal(L.col, P.col)
    assert np.array_equal(L.val.view(np.int64), P.val.view(np.int64))
