#!/usr/bin/env python
"""Benchmark of the GB300 HSMU SpGEMM engine, C = A*B (int32 CSR, FP64).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
                    [--workload NAME]

One step = one C = A*B through the engine's C ABI (hsmu_spgemm: B tile
conversion, bounds, exact symbolic count, scan, output allocation, sorted
structure, values) with A and B already resident in HBM; the step's output
is freed after it.  `value` is 2 * intermediate products / step time
(GFLOPS, the reference's own definition, src/compressed/compressed_NHC_spgemm.cu:191-202),
summed over ranks.  `e2e` is the same metric through the same public call
with host buffers: pinned host -> device copy of A and B, the product, and
device -> pinned host copy of C inside the timed region.

Default workload: the FEM-like 27-point stencil on a 40^3 grid with 3 dofs
per node (n = 192,000, nnz = 14.8M), C = A*A, values uniform(-1,1), seed 1.
Inputs (A, B = 177 MB each) and the output (789 MB) are larger than L2.

`--impl reference` times the CPU arm on the host cores: the host FP64
Gustavson restatement of the reference's path (the reference itself has no
CPU implementation of C = A*B), with every host thread, on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "hsmu-spgemm_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "SpGEMM GFLOPS + HBM GB/s, 1 GB300, plain vs learned/batched, ≤1e-12 rel FP64"
FALLBACK_HBM_GBS = 6800.0
# FP64 pipe: DADD/DMUL/DFMA lane-ops per second on GB300 (152 SMs), measured
# with a dependent-chain throughput probe: 1.61 lane-ops/clk/SM at 2070 MHz.
FP64_LANE_OPS_PER_S = 5.06e11
# DRAM bytes (read + write) per launch of the dominant kernel, from ncu captures
# summarised under profiles/ (null until captured for a workload).
class HostCSR:
    """host CSR operand of hsmu_spgemm_host (page-locked torch tensors)"""

    def __init__(self, M, N, row_ptr, col, val):
        self.M, self.N, self.row_ptr, self.col, self.val = M, N, row_ptr, col, val

    def nbytes(self):
        return sum(x.numel() * x.element_size() for x in (self.row_ptr, self.col, self.val))


# hsmu_opts.arith of the --arith choices
ARITH = {"rn": 0, "fma": 1, "imul": 2}

TRAFFIC = {
    # profiles/k_struct_ds_stencil27_32_dof3.md: 445.5 MB on the 32^3 case, scaled by the
    # algorithmic bytes (x1.993) to the 40^3 workload
    "stencil27_40_dof3_AA": 887.9e6,
    # profiles/k_numeric_rmat16_AA.md: 2.070 GB on R-MAT scale 16, scaled by the algorithmic
    # bytes (x7.73) to scale 18
    "rmat18_AA": 16.00e9,
    # profiles/k_batch_amg32_galerkin.md: 5.37 GB per launch of the 32-product batch (tuned
    # launch); the 512-product batch scaled by its algorithmic bytes (x11.82)
    "amg32_galerkin": 5.37e9,
    "amg512_galerkin": 63.5e9,
}

WORKLOADS = {
    "stencil27_40_dof3_AA": "27-point stencil, 40^3 grid x 3 dofs (n=192,000), C=A*A, uniform(-1,1), seed 1",
    "stencil27_32_dof3_AA": "27-point stencil, 32^3 grid x 3 dofs (n=98,304), C=A*A, uniform(-1,1), seed 1 (profiling size)",
    "rmat16_AA": "R-MAT scale 16, edge factor 16, merged, uniform(0,1), seed 2, C=A*A (profiling size)",
    "laplacian2d_256_AA": "5-point Laplacian, 256^2 grid (n=65,536), C=A*A, uniform(-1,1), seed 0",
    "rmat18_AA": "R-MAT scale 18, edge factor 16, (0.57,0.19,0.19,0.05), merged, uniform(0,1), seed 2, C=A*A",
    "rmat18_AAt": "R-MAT scale 18, edge factor 16, merged, uniform(0,1), seed 2, C=A*A^T",
    "rmat20_panels": "R-MAT scale 20, edge factor 16, merged, uniform(0,1), seed 3, C=A*A in row panels of at most "
                     "1.9e9 products each (nnz(C) ~ 1e10 does not fit one int32 CSR); learned scheduler vs plain",
    "amg32_galerkin": "the first 32 of the amg512_galerkin products (profiling size)",
    "amg512_galerkin": "512 AMG Galerkin products P^T(A P): A 7-point Poisson on side^3 grids, side uniform "
                       "in [16,96] (seed 4), P 2x2x2 aggregation; batched persistent engine under a CUDA graph "
                       "vs 1,024 plain calls",
}


def make_workload(name):
    from hsmu_gb import gen

    if name == "stencil27_40_dof3_AA":
        A = gen.stencil27(40, 3, seed=1)
        return A, A
    if name == "stencil27_32_dof3_AA":
        A = gen.stencil27(32, 3, seed=1)
        return A, A
    if name == "rmat16_AA":
        A = gen.rmat(16, 16, seed=2)
        return A, A
    if name == "laplacian2d_256_AA":
        A = gen.laplacian2d(256, seed=0)
        return A, A
    if name == "rmat18_AA":
        A = gen.rmat(18, 16, seed=2)
        return A, A
    if name == "rmat18_AAt":
        A = gen.rmat(18, 16, seed=2)
        return A, gen.transpose(A)
    raise SystemExit("unknown workload %s" % name)


def csr_bytes(M, nnz):
    return 4 * (M + 1) + 12 * nnz


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.proc = None
        self.dev = device_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup(n_gpus):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def cpu_model():
    """host CPU description for the baseline record (machine + model name when the kernel lists one)"""
    import platform

    name = ""
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu model")):
                    name = ln.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    return (platform.machine() + " " + name).strip()


def cpu_oracle_run(A, B, max_products=1.2e9, reps=3):
    """Time the host Gustavson oracle (all host threads) on A*B or a row sample."""
    import numpy as np

    import oracle
    from hsmu_gb import gen

    total = gen.products(A, B)
    rows = None
    sample = "all %d rows" % A.M
    prods = total
    if total > max_products:
        step = int(np.ceil(total / max_products))
        rows = np.arange(0, A.M, step, dtype=np.int32)
        blen = np.diff(B.row_ptr).astype(np.int64)
        prods = int(sum(int(blen[A.col[A.row_ptr[r]:A.row_ptr[r + 1]]].sum()) for r in rows))
        sample = "every %d-th row (%d rows, %d products)" % (step, rows.size, prods)
    nthreads = oracle.max_threads()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.spgemm(A, B, rows=rows, nthreads=nthreads)
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    return {"value": 2.0 * prods / t / 1e9, "unit": "GFLOPS", "cores": nthreads, "cpu": cpu_model(), "kind": "port",
            "sample": sample + ", median of %d" % reps, "seconds": t}


def run_reference(args):
    """CPU arm: the oracle port on the host cores, same workload and metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    A, B = make_workload(args.workload)
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_oracle_run(A, B, reps=1)
    vals, secs = [], []
    info = None
    for _ in range(args.steps):
        info = cpu_oracle_run(A, B, reps=1)
        vals.append(info["value"])
        secs.append(info["seconds"])
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "GFLOPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * statistics.median(secs), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "desc": WORKLOADS[args.workload]},
            "cpu_baseline": {"value": round(v, 3), "unit": "GFLOPS", "cores": info["cores"],
                             "kind": "port", "sample": info["sample"]},
            "e2e": {"value": round(v, 3), "unit": "GFLOPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_engine(args):
    import numpy as np
    import torch

    import hsmu_gb
    from hsmu_gb import gen

    rank, world, local = dist_setup(args.gpus)
    A, B = make_workload(args.workload)
    same = B is A
    eng = hsmu_gb.Engine()
    dA = hsmu_gb.DeviceCSR.from_host(A)
    dB = dA if same else hsmu_gb.DeviceCSR.from_host(B)
    products = gen.products(A, B)
    stream = torch.cuda.current_stream()

    # warm-up (also gives nnz(C) for the e2e host buffers)
    nnz_c = 0
    for _ in range(args.warmup):
        C = eng.spgemm(dA, dB, stats=True, arith=ARITH[args.arith])
        nnz_c = C.nnz
        C.free()
    torch.cuda.synchronize()

    # ---- device-resident timed region
    clocks = ClockSampler(local)
    clocks.start()
    dist_barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    stage = {k: 0.0 for k in ("ms_convert", "ms_symbolic", "ms_alloc", "ms_structure", "ms_numeric")}
    launches = 0
    for _ in range(args.steps):
        C = eng.spgemm(dA, dB, stats=True, arith=ARITH[args.arith])
        st = eng.last_stats
        for k in stage:
            stage[k] += st[k]
        launches += st["launches"]
        C.free()
    ev1.record(stream)
    torch.cuda.synchronize()
    dist_barrier(world)
    ms = ev0.elapsed_time(ev1) / args.steps
    clk = clocks.stop()
    ms = dist_max(ms, world)
    value = world * 2.0 * products / (ms * 1e-3) / 1e9

    # ---- end to end through the public host-buffer call (hsmu_spgemm_host): page-locked
    # host operands in, host CSR out; the copies run inside the call, behind the compute
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    hA = HostCSR(A.M, A.N, pin(A.row_ptr), pin(A.col), pin(A.val))
    hB = hA if same else HostCSR(B.M, B.N, pin(B.row_ptr), pin(B.col), pin(B.val))
    oC = (torch.empty(A.M + 1, dtype=torch.int32).pin_memory(),
          torch.empty(nnz_c, dtype=torch.int32).pin_memory(),
          torch.empty(nnz_c, dtype=torch.float64).pin_memory())
    h2d = hA.nbytes() + (0 if same else hB.nbytes())
    d2h = sum(x.numel() * x.element_size() for x in oC)

    def e2e_step():
        eng.spgemm_host(hA, hB, out=oC, arith=ARITH[args.arith], stream=stream)

    e2e_step()
    torch.cuda.synchronize()
    dist_barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ke = max(1, min(args.steps, 5))
    for _ in range(ke):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = dist_max(e0.elapsed_time(e1) / ke, world)
    e2e_value = world * 2.0 * products / (e2e_ms * 1e-3) / 1e9

    # ---- roofline of the dominant kernel.  Values are accumulated either in the
    # warp/CTA structure kernels (rows that fit one warp: columns + values in one
    # pass) or in the window kernel k_numeric (wider rows); whichever stage takes
    # longer is the dominant one.  Algorithmic bytes of that pass: read A and B,
    # write C (4(M+1) + 12 nnz per matrix), each once.
    peak, peak_kind = load_peaks()
    alg_bytes = csr_bytes(A.M, A.nnz) + csr_bytes(B.M, B.nnz) + csr_bytes(A.M, nnz_c)
    st_ms = stage["ms_structure"] / args.steps
    nu_ms = stage["ms_numeric"] / args.steps
    if st_ms >= nu_ms:
        kname, kms = "k_struct_ds/k_struct_l (sorted columns + values of warp-sized rows)", st_ms
    else:
        kname, kms = "k_numeric (values, per window)", nu_ms
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    # FP64 lane-ops/s: one DMUL + one DADD per product (rn), one DFMA (fma), one DADD (imul)
    fp64_per_product = {"rn": 2.0, "fma": 1.0, "imul": 1.0}[args.arith]
    fp64_ach = fp64_per_product * products / (kms * 1e-3)
    traffic = TRAFFIC.get(args.workload)

    if rank != 0:
        return
    cpu = cpu_oracle_run(A, B)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GFLOPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator; the reference's SuiteSparse inputs are not available)",
        "config": {"workload": args.workload, "desc": WORKLOADS[args.workload], "n": A.M,
                   "nnz_A": A.nnz, "nnz_B": B.nnz, "nnz_C": nnz_c, "products": products,
                   "l2": "inputs and output larger than L2 (A %.0f MB, C %.0f MB > 129 MB)" % (
                       csr_bytes(A.M, A.nnz) / 1e6, csr_bytes(A.M, nnz_c) / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU", "arith": args.arith},
        "hbm_gbs_step": round(alg_bytes / (ms * 1e-3) / 1e9, 2),
        "stages_ms": {k: round(v / args.steps, 4) for k, v in stage.items()},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 2),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_kind": peak_kind, "traffic": traffic,
                     "alg_bytes": alg_bytes, "ms": round(kms, 4)},
        "fp64_pipe": {"achieved_lane_ops_per_s": fp64_ach, "peak_lane_ops_per_s": FP64_LANE_OPS_PER_S,
                      "frac": round(fp64_ach / FP64_LANE_OPS_PER_S, 4),
                      "note": "FP64 pipe lane-ops of the value pass (rn: DMUL + DADD per product; fma: one DFMA; imul: one DADD)"},
        "cpu_baseline": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in cpu.items()
                         if k != "seconds"},
        "e2e": {"value": round(e2e_value, 3), "unit": "GFLOPS", "ms_per_step": round(e2e_ms, 4),
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "clocks": clk,
        "gpu_launches": launches,
    }
    # the reference's own timed section excludes the conversion of B and the setup
    conv = stage["ms_convert"] / args.steps
    line["reference_equivalent"] = {"ms_per_step": round(ms - conv, 4),
                                    "value": round(2.0 * products / ((ms - conv) * 1e-3) / 1e9, 3),
                                    "note": "step time without the B tile conversion"}
    if args.workload.endswith("_AAt"):
        # B = A^T formed on the device (hsmu_csr_transpose); the reference transposes on the host
        for _ in range(2):
            eng.transpose(dA).free()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(3):
            eng.transpose(dA, stream=stream).free()
        t1.record(stream)
        torch.cuda.synchronize()
        line["device_transpose_ms"] = round(t0.elapsed_time(t1) / 3, 4)
    print(json.dumps(line), flush=True)


def run_batched(args):
    """Config: 512 Galerkin triple products in one persistent launch (graph replay)."""
    import numpy as np
    import torch

    import hsmu_gb

    eng = hsmu_gb.Engine()
    sides = np.random.default_rng(4).integers(16, 97, size=512)
    if args.workload == "amg32_galerkin":
        sides = sides[:32]
    As, Ps, Pts = [], [], []
    for sd in sides:
        As.append(hsmu_gb.gen_poisson7(int(sd)))
        P, Pt = hsmu_gb.gen_aggregation(int(sd))
        Ps.append(P)
        Pts.append(Pt)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()

    # plain baseline: 1,024 hsmu_spgemm calls (A*P, then P^T*(AP)), also gives the product counts
    csr_b = lambda X: csr_bytes(X.M, X.nnz)
    alg = [0]

    def plain_all():
        prods = 0
        alg[0] = 0
        for A, P, Pt in zip(As, Ps, Pts):
            AP = eng.spgemm(A, P)
            prods += A.nnz + AP.nnz  # P has one entry per row; each AP row belongs to one P^T row
            C = eng.spgemm(Pt, AP)
            # compulsory bytes of the triple product: read A, P, P^T; write AP and read it back; write C
            alg[0] += csr_b(A) + csr_b(P) + csr_b(Pt) + 2 * csr_b(AP) + csr_b(C)
            C.free()
            AP.free()
        return prods

    products = plain_all()  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_all()
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1e3

    b = hsmu_gb.Batch(eng, hsmu_gb.BATCH_GALERKIN, As, Ps, Pts)
    tiny, grid, tune_ms = b.autotune()
    b.graph_launch()
    b.status()
    for _ in range(args.warmup):
        b.graph_launch()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        b.graph_launch()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    b.status()
    ms = ev0.elapsed_time(ev1) / args.steps
    value = 2.0 * products / (ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GFLOPS", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (operators generated on the device)",
        "config": {"workload": args.workload, "desc": WORKLOADS[args.workload], "products_total": products,
                   "fine_rows": int((sides.astype(np.int64) ** 3).sum()), "spgemms": 2 * len(sides)},
        "roofline": {"bound": "hbm", "kernel": "k_batch (persistent: both products, count + scan + fill)",
                     "achieved": round(alg[0] / (ms * 1e-3) / 1e9, 2), "peak": load_peaks()[0], "unit": "GB/s",
                     "frac": round(alg[0] / (ms * 1e-3) / 1e9 / load_peaks()[0], 4), "peak_kind": load_peaks()[1],
                     "traffic": TRAFFIC.get(args.workload), "alg_bytes": alg[0]},
        "batched": {"ms": round(ms, 4), "plain_calls_ms": round(plain_ms, 3), "plain_calls": 2 * len(sides),
                    "speedup_vs_plain": round(plain_ms / ms, 2), "autotuned": {"tiny": tiny, "grid": grid},
                    "launches_per_step": 1, "graph": True},
        "clocks": clk, "gpu_launches": args.steps,
    }
    print(json.dumps(line), flush=True)


def run_learned_panels(args):
    """Learned scheduler vs plain engine on R-MAT scale 20, processed in row panels."""
    import numpy as np
    import torch

    import hsmu_gb
    from hsmu_gb import gen, learned

    A = gen.rmat(20, 16, seed=3)
    blen = np.diff(A.row_ptr).astype(np.int64)
    cs = np.concatenate(([0], np.cumsum(blen[A.col])))
    rowprod = cs[A.row_ptr[1:]] - cs[A.row_ptr[:-1]]
    cum = np.concatenate(([0], np.cumsum(rowprod)))
    cuts = [0]
    while cuts[-1] < A.M:  # panels of at most 1.9e9 products (so nnz(C) < 2^31)
        nxt = int(np.searchsorted(cum, cum[cuts[-1]] + 1.9e9, side="right")) - 1
        cuts.append(max(nxt, cuts[-1] + 1) if nxt < A.M else A.M)
    eng = hsmu_gb.Engine()
    dA = hsmu_gb.DeviceCSR.from_host(A)
    params, margin, meta = learned.load()
    pt = torch.from_numpy(params).cuda()

    def panel(r0, r1):
        c = hsmu_gb.c_csr(r1 - r0, A.N, A.nnz, 0, dA.desc.row_ptr + 4 * r0, dA.desc.col, dA.desc.val)
        return hsmu_gb.DeviceCSR(c, keep=dA)

    panels = [panel(cuts[k], cuts[k + 1]) for k in range(len(cuts) - 1)]
    # warm-up on the first panel
    eng.spgemm(panels[0], dA).free()
    eng.spgemm_learned(panels[0], dA, pt, margin).free()
    res = {"plain": [], "learned": []}
    fallback = capacity = nnz_total = 0
    for P in panels:
        for mode in ("plain", "learned"):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if mode == "plain":
                C = eng.spgemm(P, dA, stats=True)
            else:
                C = eng.spgemm_learned(P, dA, pt, margin, stats=True)
            torch.cuda.synchronize()
            res[mode].append(time.perf_counter() - t0)
            st = eng.last_stats
            if mode == "learned":
                fallback += st["fallback_rows"]
                capacity += st["spec_capacity"]
                nnz_total += st["nnz_c"]
            C.free()
    products = int(cum[-1])
    tp, tl = sum(res["plain"]), sum(res["learned"])
    line = {
        "metric": METRIC, "value": round(2.0 * products / tl / 1e9, 3), "unit": "GFLOPS", "n_gpus": 1,
        "steps": 1, "warmup": 1, "ms_per_step": round(tl * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded R-MAT scale 20)",
        "config": {"workload": "rmat20_panels", "desc": WORKLOADS["rmat20_panels"], "n": A.M, "nnz_A": A.nnz,
                   "products": products, "nnz_C": nnz_total, "panels": len(panels)},
        "learned": {"ms": round(tl * 1e3, 3), "plain_ms": round(tp * 1e3, 3), "speedup_vs_plain": round(tp / tl, 3),
                    "fallback_rows": fallback, "slot_entries": capacity,
                    "slot_entries_over_nnz": round(capacity / max(1, nnz_total), 3),
                    "product_bound_over_nnz": round(products / max(1, nnz_total), 3),
                    "model": {k: v for k, v in meta.items() if k != "train_loss"}, "margin": margin},
        "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", default="stencil27_40_dof3_AA", choices=sorted(WORKLOADS))
    ap.add_argument("--arith", default="rn", choices=sorted(ARITH),
                    help="accumulation: rn = product rounded then added (the reference's arithmetic), "
                         "fma = one fused multiply-add per product, imul = rn with integer-pipe multiply")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in ("amg512_galerkin", "amg32_galerkin"):
        run_batched(args)
    elif args.workload == "rmat20_panels":
        run_learned_panels(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
