"""Learned row scheduler: training data, GPU training loop, model files.

The model is the 4 -> 32 -> 32 -> 1 FP32 MLP of hsmu_spgemm_learned (see
csrc/learned.cu).  Everything numeric runs in the engine's own CUDA kernels
(hsmu_row_features, hsmu_row_nnz, hsmu_mlp_grad, hsmu_mlp_adam,
hsmu_mlp_forward); this module only prepares inputs and drives the loop.

Training data.  2,000 seeded matrices with n between 1e4 and 1e6, from three
families: grid stencils (2-D 5/9-point, 3-D 7/27-point, 1-3 dofs), uniform
random rows (nnz/row ~ Poisson(lambda), lambda in [2, 64]) and R-MAT graphs
(scale 14-20, edge factor 8 or 16).  Every family is defined row by row, so a
matrix never has to be built in full: for each matrix 256 rows of A are
sampled, the B rows they reference are generated, and the engine computes the
exact nnz of those C rows with its symbolic pass (the labels) and their
features with the feature kernel.  R-MAT rows are drawn from the R-MAT model
itself (row degree ~ Poisson(edges * prod of the row bits' quadrant
probabilities), column bits drawn level by level given the row bits), which
is how an R-MAT edge list distributes over one row; A's sampled rows and the
B rows they reference are drawn independently from that distribution.

Model files: JSON with the parameter vector (HSMU_MLP_FLOATS floats) and the
prediction margin, and the same floats as a raw little-endian binary.
"""
from __future__ import annotations

import json
import os

import numpy as np

MLP_FLOATS = 1259
NPARAM = 1249
H, NF = 32, 4
TINY_MAX = 32
HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(HERE, "scheduler_mlp.json")


def _csr_from_keys(nrows: int, row_idx: np.ndarray, cols: np.ndarray, ncols: int):
    """Sorted, de-duplicated rows from (row index, column) pairs -> (row_ptr int64, cols int64)."""
    key = np.unique(row_idx.astype(np.int64) * ncols + cols.astype(np.int64))
    r = key // ncols
    rp = np.zeros(nrows + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=nrows), out=rp[1:])
    return rp, key % ncols


# ------------------------------------------------------------------ row families
# rows(r) -> (row_ptr, cols) of the listed rows (in the order given), sorted and unique per row
class StencilFamily:
    """dim-D grid (side^dim nodes, natural order) with a 'points' stencil and dof x dof blocks."""

    def __init__(self, dim: int, side: int, points: int, dof: int):
        self.dim, self.side, self.points, self.dof = dim, side, points, dof
        self.n = side ** dim * dof
        if dim == 2:
            offs = [(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1)] if points == 5 else \
                [(dx, dy) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
        else:
            offs = [(0, 0, 0), (-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)] \
                if points == 7 else [(dx, dy, dz) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
        self.offs = np.array(offs, np.int64)

    def rows(self, r: np.ndarray, rng=None):
        s, dof, dim = self.side, self.dof, self.dim
        node = r // dof
        coords = np.stack([(node // s ** d) % s for d in range(dim)], axis=1)      # (R, dim)
        nb = coords[:, None, :] + self.offs[None, :, :]                            # (R, P, dim)
        ok = np.all((nb >= 0) & (nb < s), axis=2)
        nid = sum(nb[:, :, d] * s ** d for d in range(dim))                        # (R, P)
        ri = np.repeat(np.arange(r.size), ok.sum(axis=1))
        nodes = nid[ok]
        cols = (nodes[:, None] * dof + np.arange(dof)[None, :]).reshape(-1)
        return _csr_from_keys(r.size, np.repeat(ri, dof), cols, self.n)


class PoissonFamily:
    def __init__(self, n: int, lam: float, seed: int):
        self.n, self.lam, self.seed = n, lam, seed

    def rows(self, r: np.ndarray, rng):
        k = rng.poisson(self.lam, size=r.size)
        ri = np.repeat(np.arange(r.size), k)
        c = rng.integers(0, self.n, size=ri.size)
        return _csr_from_keys(r.size, ri, c, self.n)


class RmatFamily:
    def __init__(self, scale: int, ef: int, seed: int, probs=(0.57, 0.19, 0.19, 0.05)):
        self.scale, self.n, self.seed = scale, 1 << scale, seed
        self.ne = ef * (1 << scale)
        self.a, self.b, self.c, self.d = probs

    def rows(self, r: np.ndarray, rng):
        s = self.scale
        bits = (r[:, None] >> np.arange(s - 1, -1, -1)[None, :]) & 1  # most significant first
        p_row = np.where(bits == 0, self.a + self.b, self.c + self.d).prod(axis=1)
        k = rng.poisson(self.ne * p_row)
        q1 = np.where(bits == 0, self.b / (self.a + self.b), self.d / (self.c + self.d)).astype(np.float32)
        ri = np.repeat(np.arange(r.size), k)
        col = np.zeros(ri.size, np.int64)
        for lev in range(s):  # column bit `lev` given the row's bit at that level
            col |= (rng.random(ri.size, dtype=np.float32) < q1[ri, lev]).astype(np.int64) << (s - 1 - lev)
        return _csr_from_keys(r.size, ri, col, self.n)


def family_for(idx: int, seed: int = 0):
    """Matrix idx of the training set: (family, description)."""
    rng = np.random.default_rng([seed, idx])
    kind = idx % 3
    if kind == 0:
        dim = int(rng.integers(2, 4))
        points = int(rng.choice([5, 9])) if dim == 2 else int(rng.choice([7, 27]))
        dof = int(rng.integers(1, 4))
        n_target = float(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
        side = max(4, int(round((n_target / dof) ** (1.0 / dim))))
        return StencilFamily(dim, side, points, dof), "stencil%dd-%dpt-dof%d-side%d" % (dim, points, dof, side)
    if kind == 1:
        n = int(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
        lam = float(rng.uniform(2, 64))
        return PoissonFamily(n, lam, int(rng.integers(1 << 30))), "poisson-n%d-lam%.1f" % (n, lam)
    scale = int(rng.integers(14, 21))
    ef = int(rng.choice([8, 16]))
    return RmatFamily(scale, ef, int(rng.integers(1 << 30))), "rmat-s%d-ef%d" % (scale, ef)


def sample_problem(fam, nrows: int, seed: int):
    """A_s (sampled rows of A, columns renumbered) and B_s (the rows they reference), host CSR."""
    from .gen import CSR

    rng = np.random.default_rng(seed)
    r = np.sort(rng.choice(fam.n, size=min(nrows, fam.n), replace=False)).astype(np.int64)
    arp, acol = fam.rows(r, rng)
    ks = np.unique(acol)
    brp, bcol = fam.rows(ks, rng) if ks.size else (np.zeros(1, np.int64), np.zeros(0, np.int64))
    acol_s = np.searchsorted(ks, acol)  # renumber A's columns to rows of B_s
    A = CSR(r.size, ks.size, arp.astype(np.int32), acol_s.astype(np.int32), np.ones(acol_s.size))
    B = CSR(ks.size, fam.n, brp.astype(np.int32), bcol.astype(np.int32), np.ones(bcol.size))
    return A, B


def _problem(args):
    idx, rows_per_matrix, seed = args
    fam, desc = family_for(idx, seed)
    A, B = sample_problem(fam, rows_per_matrix, seed * 1000003 + idx)
    return idx, desc, A, B


def collect(engine, nmat: int = 2000, rows_per_matrix: int = 256, seed: int = 0, workers: int = 0, log=None):
    """(X [n,4] float32, y [n] float32 log2 nnz) over nmat training matrices (rows with > TINY_MAX products).

    Host-side sampling runs in `workers` spawned processes (0: all cores but one); the features and the
    labels come from the engine on the GPU."""
    import concurrent.futures as cf
    import multiprocessing as mp

    import torch

    from . import DeviceCSR

    Xs, ys = [], []
    workers = workers or max(1, (os.cpu_count() or 2) - 1)
    jobs = [(i, rows_per_matrix, seed) for i in range(nmat)]

    def consume(idx, desc, A, B):
        if A.nnz == 0 or B.nnz == 0:
            return
        dA, dB = DeviceCSR.from_host(A), DeviceCSR.from_host(B)
        feat, prod = engine.row_features(dA, dB)
        nnz = engine.row_nnz(dA, dB)
        keep = (prod > TINY_MAX) & (nnz > 0)
        Xs.append(feat[keep].cpu().numpy())
        ys.append(np.log2(nnz[keep].cpu().numpy().astype(np.float64)).astype(np.float32))
        if log and idx % 100 == 0:
            log("matrix %d/%d %s: %d rows kept" % (idx, nmat, desc, int(keep.sum().item())))

    if workers <= 1:
        for j in jobs:
            consume(*_problem(j))
    else:
        with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            for res in ex.map(_problem, jobs, chunksize=4):
                consume(*res)
    torch.cuda.synchronize()
    return np.concatenate(Xs), np.concatenate(ys)


# ------------------------------------------------------------------ model
def init_params(X: np.ndarray, y: np.ndarray, seed: int = 0) -> np.ndarray:
    """He-initialised weights and normalisation constants from the data."""
    rng = np.random.default_rng(seed)
    p = np.zeros(MLP_FLOATS, np.float32)
    p[0:128] = rng.normal(0, np.sqrt(2.0 / NF), 128)
    p[160:160 + 1024] = rng.normal(0, np.sqrt(2.0 / H), 1024)
    p[1216:1248] = rng.normal(0, np.sqrt(1.0 / H), 32)
    p[1249:1253] = X.mean(axis=0)
    p[1253:1257] = X.std(axis=0) + 1e-3
    p[1257] = y.mean()
    p[1258] = y.std() + 1e-3
    return p


def train(X: np.ndarray, y: np.ndarray, epochs: int = 20, batch: int = 4096, lr: float = 2e-3, seed: int = 0,
          params: np.ndarray | None = None, log=None):
    """Adam on the GPU with the engine's gradient and update kernels; returns (params, loss history)."""
    import ctypes

    import torch

    from . import _check, _stream_ptr, load_library

    L = load_library()
    p = torch.from_numpy(params if params is not None else init_params(X, y, seed)).cuda()
    m = torch.zeros(NPARAM, dtype=torch.float32, device="cuda")
    v = torch.zeros_like(m)
    g = torch.zeros_like(m)
    lossd = torch.zeros(1, dtype=torch.float32, device="cuda")
    Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
    yd = torch.from_numpy(np.ascontiguousarray(y, np.float32)).cuda()
    n = X.shape[0]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    step, hist = 0, []
    sp = _stream_ptr(None)
    for ep in range(epochs):
        perm = torch.randperm(n, device="cuda", generator=gen)
        lossd.zero_()
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            xb = Xd.index_select(0, idx).contiguous()
            yb = yd.index_select(0, idx).contiguous()
            g.zero_()
            _check(L.hsmu_mlp_grad(p.data_ptr(), xb.data_ptr(), yb.data_ptr(), int(idx.numel()), g.data_ptr(),
                                   lossd.data_ptr(), sp), "hsmu_mlp_grad")
            step += 1
            lr_t = lr * 0.5 * (1 + np.cos(np.pi * min(1.0, step / max(1, epochs * ((n + batch - 1) // batch)))))
            _check(L.hsmu_mlp_adam(p.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), ctypes.c_float(lr_t),
                                   ctypes.c_float(1.0 / idx.numel()), step, sp), "hsmu_mlp_adam")
        hist.append(float(lossd.item()) / n)
        if log:
            log("epoch %d loss %.5f" % (ep, hist[-1]))
    return p.cpu().numpy(), hist


def predict(params: np.ndarray, X: np.ndarray) -> np.ndarray:
    """log2(nnz) predictions through the engine's forward kernel."""
    import torch

    from . import _check, _stream_ptr, load_library

    p = torch.from_numpy(np.ascontiguousarray(params, np.float32)).cuda()
    Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
    out = torch.empty(X.shape[0], dtype=torch.float32, device="cuda")
    _check(load_library().hsmu_mlp_forward(p.data_ptr(), Xd.data_ptr(), X.shape[0], out.data_ptr(),
                                           _stream_ptr(None)), "hsmu_mlp_forward")
    return out.cpu().numpy()


def choose_margin(params, X, y, quantile: float = 0.99) -> float:
    """log2 margin so that `quantile` of the rows fit their predicted slot."""
    res = y - predict(params, X)
    return float(np.quantile(res, quantile))


def save(path: str, params: np.ndarray, margin: float, meta: dict | None = None) -> None:
    params = np.asarray(params, np.float32)
    with open(path, "w") as f:
        json.dump({"format": "hsmu-scheduler-mlp-1", "floats": MLP_FLOATS, "margin": margin,
                   "meta": meta or {}, "params": [float(x) for x in params]}, f)
    params.astype("<f4").tofile(os.path.splitext(path)[0] + ".bin")


def load(path: str = DEFAULT_MODEL):
    with open(path) as f:
        d = json.load(f)
    p = np.array(d["params"], np.float32)
    if p.size != MLP_FLOATS:
        raise ValueError("model file has %d floats, expected %d" % (p.size, MLP_FLOATS))
    return p, float(d["margin"]), d.get("meta", {})


def main():
    """Train the shipped model: python -m hsmu_gb.learned [nmat] [rows_per_matrix] [epochs]."""
    import sys
    import time

    from . import Engine

    nmat = int(sys.argv[1]) if len(sys.argv) > 1 else 2000
    rows = int(sys.argv[2]) if len(sys.argv) > 2 else 256
    epochs = int(sys.argv[3]) if len(sys.argv) > 3 else 20
    eng = Engine()
    t0 = time.time()
    X, y = collect(eng, nmat, rows, seed=0, log=print)
    print("samples", X.shape[0], "collected in %.1fs" % (time.time() - t0), flush=True)
    rng = np.random.default_rng(1)
    perm = rng.permutation(X.shape[0])
    nval = max(1, X.shape[0] // 10)
    va, tr = perm[:nval], perm[nval:]
    params, hist = train(X[tr], y[tr], epochs=epochs, log=print)
    margin = choose_margin(params, X[va], y[va], 0.99)
    pred = predict(params, X[va])
    mae = float(np.mean(np.abs(pred - y[va])))
    meta = {"matrices": nmat, "rows_per_matrix": rows, "samples": int(X.shape[0]), "epochs": epochs,
            "val_mae_log2": mae, "val_fit_fraction": float(np.mean(y[va] <= pred + margin)),
            "train_loss": hist}
    save(DEFAULT_MODEL, params, margin, meta)
    print(json.dumps({k: v for k, v in meta.items() if k != "train_loss"}), "margin", margin)


if __name__ == "__main__":
    main()
