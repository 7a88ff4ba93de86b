"""Generate tests/golden/reference_outputs.json from the reference itself.

Runs the reference HSMU-SpGEMM GPU path (oracle/_ref/ref_harness, compiled
from the reference sources by oracle/ref_build.py) on seeded workloads and
records, per case: the generator call, nnz(C), the intermediate product
count, SHA-256 digests of C's row pointers and column indices, and a seeded
sample of (row, column, value) entries.  The reference adds products with
shared-memory atomics, so its values are only reproducible to rounding; the
CPU tests compare the oracle's values with these within 1e-12.

Needs a GPU and the built harness:  python tests/golden/make_golden.py [out.json]
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "hsmu-spgemm_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

CASES = {
    "laplacian2d_64_AA": "laplacian2d(64, seed=0) * itself",
    "laplacian2d_256_AA": "laplacian2d(256, seed=0) * itself (the 2-D Laplacian workload)",
    "stencil27_12_dof3_AA": "stencil27(12, 3, seed=1) * itself",
    "rmat12_AA": "rmat(12, 16, seed=2) * itself",
    "rmat12_AAt": "rmat(12, 16, seed=2) * its transpose",
    "rmat14_AA": "rmat(14, 16, seed=2) * itself",
    "random_rect": "poisson_random(3000, 10, seed=21, ncols=6000) * poisson_random(6000, 8, seed=22, ncols=9000)",
}


def make_case(name):
    from hsmu_gb import gen

    if name == "laplacian2d_64_AA":
        A = gen.laplacian2d(64, seed=0)
        return A, A
    if name == "laplacian2d_256_AA":
        A = gen.laplacian2d(256, seed=0)
        return A, A
    if name == "stencil27_12_dof3_AA":
        A = gen.stencil27(12, 3, seed=1)
        return A, A
    if name == "rmat12_AA":
        A = gen.rmat(12, 16, seed=2)
        return A, A
    if name == "rmat12_AAt":
        A = gen.rmat(12, 16, seed=2)
        return A, gen.transpose(A)
    if name == "rmat14_AA":
        A = gen.rmat(14, 16, seed=2)
        return A, A
    if name == "random_rect":
        return (gen.poisson_random(3000, 10, seed=21, ncols=6000),
                gen.poisson_random(6000, 8, seed=22, ncols=9000))
    raise KeyError(name)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def sample_entries(C, k=400, seed=0):
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(C.nnz, size=min(k, C.nnz), replace=False))
    rows = np.searchsorted(C.row_ptr, idx, side="right") - 1
    return [[int(r), int(C.col[i]), float(C.val[i])] for r, i in zip(rows, idx)]


def main():
    from hsmu_gb import gen
    from oracle import ref_run

    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "reference_outputs.json")
    res = {"source": "reference HSMU-SpGEMM GPU path (NHC_spgemm), compiled for sm_103a and run on a GB300",
           "cases": {}}
    for name, desc in CASES.items():
        A, B = make_case(name)
        C, info = ref_run.run(A, None if B is A else B, reps=1)
        res["cases"][name] = {"inputs": desc, "M": C.M, "N": C.N, "nnz": C.nnz,
                              "products": gen.products(A, B), "row_ptr_sha256": digest(C.row_ptr),
                              "col_sha256": digest(C.col), "sample": sample_entries(C)}
        print(name, C.nnz, flush=True)
    with open(out, "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
