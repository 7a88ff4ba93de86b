"""Command-line product of a Matrix Market matrix, the counterpart of the
reference's driver (`./test matrix.mtx`, src/test.cu:10-94): C = A*A, or
C = A*A^T with --aat (the reference's AAT build), on one GPU.

    python -m hsmu_gb.cli matrix.mtx [--aat] [--repeat N] [--arith rn|fma] [--out C.mtx]

Prints the matrix sizes, load time, products, nnz(C), the product's time and
GFLOPS (2 x intermediate products / time, the reference's definition); --out
writes C as a Matrix Market file (values with 17 significant digits, exact).
"""
from __future__ import annotations

import argparse
import sys
import time


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m hsmu_gb.cli", description=__doc__.split("\n\n")[0])
    ap.add_argument("matrix", help="Matrix Market file (coordinate)")
    ap.add_argument("--aat", action="store_true", help="C = A * A^T instead of A * A")
    ap.add_argument("--repeat", type=int, default=10, help="timed products (after one warm-up)")
    ap.add_argument("--arith", default="rn", choices=("rn", "fma"))
    ap.add_argument("--out", help="write C to this Matrix Market file")
    args = ap.parse_args(argv)

    import torch

    import hsmu_gb
    from hsmu_gb import gen, mtx

    print("the matrix is: -------------- %s --------------" % args.matrix)
    t0 = time.perf_counter()
    A = mtx.read_mtx(args.matrix)
    print("input matrix A: ( %d, %d ) nnz = %d\nloadfile time    = %.5f sec" % (A.M, A.N, A.nnz,
                                                                             time.perf_counter() - t0))
    if not args.aat and A.M != A.N:
        print("A * A needs a square matrix; use --aat", file=sys.stderr)
        return 2
    eng = hsmu_gb.Engine()
    dA = hsmu_gb.DeviceCSR.from_host(A)
    dB = eng.transpose(dA) if args.aat else dA
    arith = hsmu_gb.ARITH_FMA if args.arith == "fma" else hsmu_gb.ARITH_RN
    products = gen.products(A, dB.to_host() if args.aat else A)
    eng.spgemm(dA, dB, arith=arith).free()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(max(1, args.repeat)):
        C = eng.spgemm(dA, dB, arith=arith, stats=True)
        nnz = C.nnz
        C.free()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(1, args.repeat)
    st = eng.last_stats
    print("products = %d, nnz(C) = %d" % (products, nnz))
    print("spgemm time      = %.4f ms (B tiles %.4f, symbolic %.4f, structure %.4f, values %.4f)"
          % (ms, st["ms_convert"], st["ms_symbolic"], st["ms_structure"], st["ms_numeric"]))
    print("GFLOPS           = %.3f" % (2.0 * products / (ms * 1e-3) / 1e9))
    if args.out:
        mtx.write_mtx(args.out, eng.spgemm(dA, dB, arith=arith).to_host())
        print("C written to %s" % args.out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
