#!/usr/bin/env python
"""Benchmark of the GB300 HSMU SpGEMM engine, C = A*B (int32 CSR, FP64).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
                    [--workload NAME] [--configs all|none] [--arith rn|fma|imul]

One step = one C = A*B through the engine's C ABI (hsmu_spgemm: B tile
conversion, bounds, exact symbolic count, scan, output allocation, sorted
structure, values) with A and B already resident in HBM; the step's output
is freed after it.  `value` is 2 * intermediate products / step time
(GFLOPS, the reference's own definition, src/compressed/compressed_NHC_spgemm.cu:191-202),
over all ranks.  `e2e` is the same metric through the public host-buffer call
(hsmu_spgemm_host): pinned host -> device copy of A and B, the product, and
device -> pinned host copy of C inside the timed region.

Default (headline) workload: the largest plain configuration, C = A*A on an
R-MAT graph of scale 18 (262,144 rows, edge factor 16, probabilities
0.57/0.19/0.19/0.05, duplicates merged, values uniform(0,1), seed 2):
2.93e9 products, 1.28e9 entries of C (15.4 GB).  Inputs and output exceed L2.

Before it prints, the run checks its own output: every row pointer against
the oracle's exact count and sampled rows (random blocks and the rows with
the most products) against the host Gustavson oracle, bit for bit
(`parity`).  With `--configs all` (the default at N=1) the same line also
carries, measured in the same process: the 27-point stencil (40^3 x 3
dofs), the 5-point Laplacian (256^2) and R-MAT 18 A*A^T, each with
value / e2e / roofline; the learned scheduler vs the plain engine on R-MAT
scale 20 in row panels; the batched engine on 512 Galerkin products vs
1,024 plain calls.  Every plain configuration also carries `reference_gpu`:
the reference's own GPU path built from its sources for sm_103a and timed on
the same GPU (its `time2`, which excludes setup and the B conversion),
outside the engine's timed region.

`--gpus N` (N > 1) runs one process per GPU (it re-launches itself under
torch.distributed.run when WORLD_SIZE is unset): A's rows are split into N
blocks of about equal products, B is replicated on every GPU, and each rank
computes its block of C (hsmu_gb.shard); `value` = all products / the
slowest rank's time.

`--impl reference` times the CPU arm on the host cores: the host FP64
Gustavson restatement of the reference's path (the reference itself has no
CPU implementation of C = A*B), with every host thread, on the same workload
(a bounded row sample per step).
"""
from __future__ import annotations

import argparse
import json
import os
import socket
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
HEADLINE = "rmat18_AA"
SUB_CONFIGS = ("stencil27_40_dof3_AA", "laplacian2d_256_AA", "rmat18_AAt")


class HostCSR:
    """host CSR operand of hsmu_spgemm_host (page-locked torch tensors)"""

    def __init__(self, M, N, row_ptr, col, val):
        self.M, self.N, self.row_ptr, self.col, self.val = M, N, row_ptr, col, val

    def nbytes(self):
        return sum(x.numel() * x.element_size() for x in (self.row_ptr, self.col, self.val))


# hsmu_opts.arith of the --arith choices
ARITH = {"rn": 0, "fma": 1, "imul": 2}

TRAFFIC = {
    # DRAM bytes (read + write) per launch of the dominant kernel, from the ncu captures
    # summarised under profiles/.
    # profiles/k_struct_ds_stencil27_32_dof3.md: 445.5 MB on the 32^3 case, scaled by the
    # algorithmic bytes (x1.993) to the 40^3 workload
    "stencil27_40_dof3_AA": 887.9e6,
    # profiles/k_numeric_rmat16_AA.md: 1.828 GB on R-MAT scale 16, scaled by the algorithmic
    # bytes (x7.765) to scale 18
    "rmat18_AA": 14.19e9,
    # profiles/k_batch_amg32_galerkin.md: 3.12 GB per launch of the 32-product batch (tuned
    # launch); the 512-product batch scaled by its algorithmic bytes (x11.82)
    "amg32_galerkin": 3.12e9,
    "amg512_galerkin": 36.9e9,
}

WORKLOADS = {
    "stencil27_40_dof3_AA": "27-point stencil, 40^3 grid x 3 dofs (n=192,000), C=A*A, uniform(-1,1), seed 1",
    "stencil27_32_dof3_AA": "27-point stencil, 32^3 grid x 3 dofs (n=98,304), C=A*A, uniform(-1,1), seed 1 (profiling size)",
    "rmat16_AA": "R-MAT scale 16, edge factor 16, merged, uniform(0,1), seed 2, C=A*A (profiling size)",
    "laplacian2d_256_AA": "5-point Laplacian, 256^2 grid (n=65,536), C=A*A, uniform(-1,1), seed 0",
    "rmat18_AA": "R-MAT scale 18, edge factor 16, (0.57,0.19,0.19,0.05), merged, uniform(0,1), seed 2, C=A*A",
    "rmat18_AAt": "R-MAT scale 18, edge factor 16, merged, uniform(0,1), seed 2, C=A*A^T",
    "rmat20_panels": "R-MAT scale 20, edge factor 16, merged, uniform(0,1), seed 3, C=A*A in row panels of at most "
                     "1.9e9 products each (nnz(C) ~ 9.7e9 does not fit one int32 CSR); learned scheduler vs plain",
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


def workload_config(name, A, B, nnz_c, world=1, arith="rn"):
    """the `config` object of a plain workload (the same dict on both arms)"""
    from hsmu_gb import gen

    return {"workload": name, "desc": WORKLOADS[name], "n": A.M, "nnz_A": A.nnz, "nnz_B": B.nnz,
            "nnz_C": int(nnz_c), "products": gen.products(A, B),
            "l2": l2_note(A, B, nnz_c),
            "parallelism": ("row blocks x%d" % world) if world > 1 else "single GPU", "arith": arith}


def l2_note(A, B, nnz_c):
    """how the timed steps stand to the 129 MB L2 (no flush between steps)"""
    mb = lambda x: x / 1e6
    a, b, c = csr_bytes(A.M, A.nnz), csr_bytes(B.M, B.nnz), csr_bytes(A.M, nnz_c)
    if a + c > 129e6:
        return "no L2 flush: inputs and output larger than L2 (A %.0f MB, B %.0f MB, C %.0f MB; L2 129 MB)" % (
            mb(a), mb(b), mb(c))
    return "no L2 flush: working set fits L2 (A %.1f MB, B %.1f MB, C %.1f MB; L2 129 MB)" % (mb(a), mb(b), mb(c))


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
        return self

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


# ------------------------------------------------------------------ ranks
def dist_setup(n_gpus):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def dist_max(x, world):
    return _dist_reduce(x, world, "max")


def dist_sum(x, world):
    return _dist_reduce(x, world, "sum")


def _dist_reduce(x, world, op):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def relaunch_under_torchrun(args) -> int:
    """--gpus N without WORLD_SIZE: start N processes (one per GPU) and wait"""
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(args.gpus),
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


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


# ------------------------------------------------------------------ CPU arm
def cpu_oracle_run(A, B, max_products=1.0e9, reps=3):
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
        cs = np.concatenate(([0], np.cumsum(blen[A.col])))
        prods = int((cs[A.row_ptr[rows + 1]] - cs[A.row_ptr[rows]]).sum())
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
    """CPU arm: the oracle port on the host cores, same workload, metric and config."""
    import oracle

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload not in WORKLOADS or args.workload in ("rmat20_panels", "amg32_galerkin", "amg512_galerkin"):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU arm times the plain workloads only"}))
        return
    A, B = make_workload(args.workload)
    for _ in range(args.warmup):
        cpu_oracle_run(A, B, reps=1)
    vals, secs = [], []
    info = None
    for _ in range(args.steps):
        info = cpu_oracle_run(A, B, reps=1)
        vals.append(info["value"])
        secs.append(info["seconds"])
    v = statistics.median(vals)
    nnz_c = int(oracle.symbolic(A, B).sum())
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "GFLOPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * statistics.median(secs), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.workload, A, B, nnz_c, arith=args.arith),
            "cpu_baseline": {"value": round(v, 3), "unit": "GFLOPS", "cores": info["cores"], "cpu": info["cpu"],
                             "kind": "port", "sample": info["sample"].replace(", median of 1", "") +
                             "; median over %d steps" % args.steps},
            "e2e": {"value": round(v, 3), "unit": "GFLOPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ reference GPU path
def reference_gpu(A, B, products, reps=3):
    """The reference's own GPU path (oracle/_ref harness) on the same inputs: its time2
    (symbolic + allocation + columns + values, no setup or B conversion) and the whole
    NHC_spgemm call; warm medians over reps - 1 calls after the first."""
    from oracle import ref_run

    if not ref_run.available():
        return {"unavailable": "reference harness not built on this machine"}
    if B.N < 4096:
        return {"unavailable": "B has fewer than 4096 columns (the reference's small path)"}
    try:
        _, info = ref_run.run(A, None if B is A else B, reps=reps, output=False)
    except Exception as e:  # noqa: BLE001
        return {"unavailable": str(e).splitlines()[0][:200]}
    t2 = info["time2_ms"][1:] or info["time2_ms"]
    call = info["call_ms"][1:] or info["call_ms"]
    if not t2:
        return {"unavailable": "the harness printed no time"}
    ms = statistics.median(t2)
    return {"ms": round(ms, 3), "value": round(2.0 * products / (ms * 1e-3) / 1e9, 3),
            "call_ms": round(statistics.median(call), 3), "reps": len(t2),
            "timer": "reference's time2 (src/compressed/compressed_NHC_spgemm.cu:191-202): stages after setup "
                     "and B conversion; call_ms: the whole NHC_spgemm call"}


# ------------------------------------------------------------------ plain engine
def measure_plain(eng, A, B, name, steps, warmup, arith, world=1, rank=0, local=0, clocks=True):
    """device-resident step time, end-to-end host-buffer time and the dominant
    kernel's roofline for C = A*B (this rank's row block when world > 1)."""
    import numpy as np
    import torch

    import hsmu_gb
    from hsmu_gb import gen, shard

    same = B is A
    products_total = gen.products(A, B)
    dA_full = hsmu_gb.DeviceCSR.from_host(A)
    dB = dA_full if same else hsmu_gb.DeviceCSR.from_host(B)
    r0, r1 = 0, A.M
    if world > 1:
        cuts = shard.row_blocks(A, B, world)
        r0, r1 = int(cuts[rank]), int(cuts[rank + 1])
    dA = dA_full if world == 1 else shard.device_block(dA_full, r0, r1)
    Ah = A if world == 1 else shard.host_block(A, r0, r1)
    stream = torch.cuda.current_stream()
    ar = ARITH[arith]

    nnz_c = 0
    for _ in range(warmup):
        C = eng.spgemm(dA, dB, stats=True, arith=ar)
        nnz_c = C.nnz
        C.free()
    torch.cuda.synchronize()

    # ---- device-resident timed region
    clk = ClockSampler(local).start() if clocks else None
    dist_barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    stage = {k: 0.0 for k in ("ms_convert", "ms_symbolic", "ms_alloc", "ms_structure", "ms_numeric")}
    launches = 0
    for _ in range(steps):
        C = eng.spgemm(dA, dB, stats=True, arith=ar)
        st = eng.last_stats
        for k in stage:
            stage[k] += st[k]
        launches += st["launches"]
        C.free()
    ev1.record(stream)
    torch.cuda.synchronize()
    dist_barrier(world)
    ms = ev0.elapsed_time(ev1) / steps
    clk = clk.stop() if clk else None
    ms = dist_max(ms, world)
    value = 2.0 * products_total / (ms * 1e-3) / 1e9

    # ---- end to end through the public host-buffer call (hsmu_spgemm_host): page-locked
    # host operands in, host CSR out; the copies run inside the call, behind the compute
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    hA = HostCSR(Ah.M, Ah.N, pin(Ah.row_ptr), pin(Ah.col), pin(Ah.val))
    hB = hA if (same and world == 1) else HostCSR(B.M, B.N, pin(B.row_ptr), pin(B.col), pin(B.val))
    oC = (torch.empty(Ah.M + 1, dtype=torch.int32).pin_memory(),
          torch.empty(nnz_c, dtype=torch.int32).pin_memory(),
          torch.empty(nnz_c, dtype=torch.float64).pin_memory())
    h2d = hA.nbytes() + (0 if hB is hA else hB.nbytes())
    d2h = sum(x.numel() * x.element_size() for x in oC)

    def e2e_step():
        eng.spgemm_host(hA, hB, out=oC, arith=ar, stream=stream)

    # the host link is shared with the machine's other jobs: a plain copy of the same
    # output bytes into the same page-locked arrays, just before and just after the
    # timed calls, records what it gave during them
    def link_copy_ms():
        d_col = torch.empty(oC[1].shape, dtype=oC[1].dtype, device=stream.device)
        d_val = torch.empty(oC[2].shape, dtype=oC[2].dtype, device=stream.device)
        c0 = torch.cuda.Event(enable_timing=True)
        c1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        c0.record(stream)
        with torch.cuda.stream(stream):
            oC[1].copy_(d_col, non_blocking=True)
            oC[2].copy_(d_val, non_blocking=True)
        c1.record(stream)
        torch.cuda.synchronize()
        del d_col, d_val
        torch.cuda.empty_cache()  # the engine's own pool serves the configs that follow
        return c0.elapsed_time(c1)

    e2e_step()
    link_before = link_copy_ms()
    torch.cuda.synchronize()
    dist_barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ke = max(1, min(steps, 5))
    for _ in range(ke):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    link_after = link_copy_ms()
    e2e_ms = dist_max(e0.elapsed_time(e1) / ke, world)
    e2e_value = 2.0 * products_total / (e2e_ms * 1e-3) / 1e9
    link_bytes = oC[1].numel() * oC[1].element_size() + oC[2].numel() * oC[2].element_size()
    del hA, hB, oC

    # ---- roofline of the dominant kernel.  Values are accumulated either in the
    # warp/CTA structure kernels (rows that fit one warp: columns + values in one
    # pass) or in the window kernel k_numeric (wider rows); whichever stage takes
    # longer is the dominant one.  Algorithmic bytes of that pass: read A and B,
    # write C (4(M+1) + 12 nnz per matrix), each once.
    peak, peak_kind = load_peaks()
    alg_bytes = csr_bytes(Ah.M, Ah.nnz) + csr_bytes(B.M, B.nnz) + csr_bytes(Ah.M, nnz_c)
    st_ms = stage["ms_structure"] / steps
    nu_ms = stage["ms_numeric"] / steps
    if st_ms >= nu_ms:
        kname, kms = "k_struct_ds/k_struct_l (sorted columns + values of warp-sized rows)", st_ms
    else:
        kname, kms = "k_numeric (values, per window)", nu_ms
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    products_mine = gen.products(Ah, B)
    # diagnostic, not the graded figure: every product gathers its B entry (12 bytes), plus the
    # A and C terms
    gather_bytes = 12 * products_mine + csr_bytes(Ah.M, Ah.nnz) + csr_bytes(Ah.M, nnz_c)
    fp64_per_product = {"rn": 2.0, "fma": 1.0, "imul": 1.0}[arith]
    return {
        "ms": ms, "value": value, "nnz_c": nnz_c, "products": products_total, "products_rank": products_mine,
        "block": (r0, r1), "dA": dA, "dB": dB, "Ah": Ah,
        "stages": {k: round(v / steps, 4) for k, v in stage.items()}, "launches": launches,
        "alg_bytes": alg_bytes,
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": TRAFFIC.get(name),
                     "alg_bytes": alg_bytes, "ms": round(kms, 4), "gather_bytes": gather_bytes,
                     "gather_gbs": round(gather_bytes / (kms * 1e-3) / 1e9, 2)},
        "fp64_ops": fp64_per_product * products_mine, "kernel_ms": kms,
        "e2e": {"value": round(e2e_value, 3), "unit": "GFLOPS", "ms_per_step": round(e2e_ms, 4),
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "link": {"note": "plain copy of C's columns and values over the host link, just before / "
                                 "after the timed calls",
                         "ms": [round(link_before, 2), round(link_after, 2)],
                         "gbs": [round(link_bytes / (t * 1e-3) / 1e9, 1) for t in (link_before, link_after)]}},
        "clocks": clk,
    }


def self_check(eng, m, B, arith, full_rowptr=True):
    """one more product of the measured workload, checked against the oracle:
    every row pointer (exact symbolic count) and sampled rows bit for bit"""
    import numpy as np

    import oracle
    from oracle import sampled

    if arith != "rn":
        return {"skipped": "the oracle check runs for the rn arithmetic"}
    Ah = m["Ah"]
    C = eng.spgemm(m["dA"], m["dB"], arith=ARITH[arith])
    rp = C.row_ptr_host()
    out = {}
    if full_rowptr:
        want = np.zeros(Ah.M + 1, dtype=np.int64)
        np.cumsum(oracle.symbolic(Ah, B), out=want[1:])
        out["row_ptr_all_rows"] = bool(np.array_equal(rp.astype(np.int64), want))
    rows = sampled.sample_rows(Ah, B)
    try:
        res = sampled.check_rows(C.rows_to_host(rows, row_ptr=rp), Ah, B, rows)
        out.update(res)
    except AssertionError as e:
        out.update({"rows": int(rows.size), "bitwise": False, "error": str(e)[:300]})
    C.free()
    out["ok"] = bool(out.get("bitwise")) and out.get("row_ptr_all_rows", True)
    return out


def plain_summary(m, name, ref=None, parity=None):
    """compact record of one plain workload for the `configs` object"""
    return {"desc": WORKLOADS[name], "value": round(m["value"], 3), "unit": "GFLOPS",
            "ms_per_step": round(m["ms"], 4), "nnz_C": m["nnz_c"], "products": m["products"],
            "stages_ms": m["stages"], "e2e": m["e2e"],
            "roofline": {k: m["roofline"][k] for k in ("kernel", "achieved", "peak", "frac", "traffic", "ms")},
            "reference_gpu": ref, "vs_reference_gpu": (round(m["value"] / ref["value"], 2)
                                                       if ref and ref.get("value") else None),
            "parity": parity, "clocks": m["clocks"]}


def run_engine(args):
    import torch

    import hsmu_gb

    rank, world, local = dist_setup(args.gpus)
    A, B = make_workload(args.workload)
    eng = hsmu_gb.Engine()
    m = measure_plain(eng, A, B, args.workload, args.steps, args.warmup, args.arith, world, rank, local)
    parity = self_check(eng, m, B, args.arith) if args.parity == "on" else None
    ok = dist_max(0.0 if (parity is None or parity.get("ok")) else 1.0, world) == 0.0
    fp64_peak = hsmu_gb.probe_fp64_rate()
    fp64_ach = dist_sum(m["fp64_ops"], world) / (m["kernel_ms"] * 1e-3)
    if rank != 0:
        return
    cpu = cpu_oracle_run(A, B)
    line = {
        "metric": METRIC, "value": round(m["value"], 3), "unit": "GFLOPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(m["ms"], 4),
        "higher_is_better": True, "scaling": "weak" if world == 1 else "strong", "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded generator; the reference's SuiteSparse inputs are not available)",
        "config": workload_config(args.workload, A, B, m["nnz_c"] if world == 1 else
                                  int(dist_sum(m["nnz_c"], world)), world, args.arith),
        "hbm_gbs_step": round((csr_bytes(A.M, A.nnz) + csr_bytes(B.M, B.nnz) + csr_bytes(A.M, m["nnz_c"]))
                              / (m["ms"] * 1e-3) / 1e9, 2),
        "stages_ms": m["stages"],
        "roofline": m["roofline"],
        "fp64_pipe": {"achieved_lane_ops_per_s": fp64_ach, "peak_lane_ops_per_s": fp64_peak,
                      "frac": round(fp64_ach / fp64_peak, 4), "peak_kind": "measured in this run (hsmu_probe_fp64_rate)",
                      "note": "FP64 pipe lane-ops of the dominant pass (rn: DMUL + DADD per product; fma: one DFMA; "
                              "imul: one DADD)"},
        "cpu_baseline": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in cpu.items() if k != "seconds"},
        "e2e": m["e2e"],
        "clocks": m["clocks"],
        "gpu_launches": m["launches"],
        "parity": dict(parity or {}, all_ranks_ok=ok),
    }
    conv = m["stages"]["ms_convert"]
    line["reference_equivalent"] = {"ms_per_step": round(m["ms"] - conv, 4),
                                    "value": round(2.0 * m["products"] / ((m["ms"] - conv) * 1e-3) / 1e9, 3),
                                    "note": "step time without the B tile conversion"}
    if world == 1:
        if args.workload.endswith("_AAt"):
            line["device_transpose_ms"] = device_transpose_ms(eng, m["dA"])
        line["reference_gpu"] = reference_gpu(A, B, m["products"])
        if line["reference_gpu"].get("value"):
            line["vs_reference_gpu"] = round(m["value"] / line["reference_gpu"]["value"], 2)
    del m
    torch.cuda.synchronize()
    if world == 1 and args.configs == "all":
        line["configs"] = run_sub_configs(eng, args)
    print(json.dumps(line), flush=True)


def device_transpose_ms(eng, dA):
    """A^T on the device (hsmu_csr_transpose); the reference transposes on the host"""
    import torch

    stream = torch.cuda.current_stream()
    for _ in range(2):
        eng.transpose(dA).free()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(3):
        eng.transpose(dA, stream=stream).free()
    t1.record(stream)
    torch.cuda.synchronize()
    return round(t0.elapsed_time(t1) / 3, 4)


def run_sub_configs(eng, args):
    """every other stated configuration, measured in the same process"""
    import torch

    out = {}
    steps = max(3, min(args.steps, 10))
    for name in SUB_CONFIGS:
        if name == args.workload:
            continue
        A, B = make_workload(name)
        m = measure_plain(eng, A, B, name, steps, 3, args.arith)
        par = self_check(eng, m, B, args.arith)
        rec = plain_summary(m, name, reference_gpu(A, B, m["products"]), par)
        if name.endswith("_AAt"):
            rec["device_transpose_ms"] = device_transpose_ms(eng, m["dA"])
        out[name] = rec
        del m
        torch.cuda.synchronize()
    out["rmat20_panels_learned"] = measure_learned(eng, reps=3)
    out["amg512_galerkin_batched"] = measure_batched(eng, "amg512_galerkin", steps, 3)
    return out


# ------------------------------------------------------------------ learned scheduler
def measure_learned(eng, reps=3):
    """Learned scheduler vs plain engine on R-MAT scale 20 in row panels of at most
    1.9e9 products (each panel's C fits int32 CSR); CUDA events around all panels,
    median of `reps` repeats of each form, clocks sampled over the timed repeats."""
    import numpy as np
    import torch

    import hsmu_gb
    from hsmu_gb import gen, learned, shard
    from oracle import sampled

    A = gen.rmat(20, 16, seed=3)
    rowprod = shard.row_products(A, A)
    cum = np.concatenate(([0], np.cumsum(rowprod)))
    cuts = [0]
    while cuts[-1] < A.M:  # panels of at most 1.9e9 products (so nnz(C) < 2^31)
        nxt = int(np.searchsorted(cum, cum[cuts[-1]] + 1.9e9, side="right")) - 1
        cuts.append(max(nxt, cuts[-1] + 1) if nxt < A.M else A.M)
    dA = hsmu_gb.DeviceCSR.from_host(A)
    params, margin, meta = learned.load()
    pt = torch.from_numpy(params).cuda()

    def panel(r0, r1):
        c = hsmu_gb.c_csr(r1 - r0, A.N, A.nnz, 0, dA.desc.row_ptr + 4 * r0, dA.desc.col, dA.desc.val)
        return hsmu_gb.DeviceCSR(c, keep=dA)

    panels = [panel(cuts[k], cuts[k + 1]) for k in range(len(cuts) - 1)]
    stream = torch.cuda.current_stream()

    def run_all(mode):
        fb = cap = nnz = 0
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for P in panels:
            if mode == "plain":
                C = eng.spgemm(P, dA, stats=True)
            else:
                C = eng.spgemm_learned(P, dA, pt, margin, stats=True)
                st = eng.last_stats
                fb += st["fallback_rows"]
                cap += st["spec_capacity"]
                nnz += st["nnz_c"]
            C.free()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), fb, cap, nnz

    run_all("plain")  # warm-up (also sizes the pool)
    run_all("learned")
    clk = ClockSampler(0).start()
    tp, tl = [], []
    fallback = capacity = nnz_total = 0
    for _ in range(reps):
        tp.append(run_all("plain")[0])
        t, fallback, capacity, nnz_total = run_all("learned")
        tl.append(t)
    clocks = clk.stop()
    # output check: the first panel, learned vs plain on sampled rows, and the plain rows vs the oracle
    r0, r1 = cuts[0], cuts[1]
    hp = gen.CSR(r1 - r0, A.N, (A.row_ptr[r0:r1 + 1] - A.row_ptr[r0]).astype(np.int32),
                 A.col[A.row_ptr[r0]:A.row_ptr[r1]], A.val[A.row_ptr[r0]:A.row_ptr[r1]])
    Cl = eng.spgemm_learned(panels[0], dA, pt, margin)
    Cp = eng.spgemm(panels[0], dA)
    rows = sampled.sample_rows(hp, A, blocks=16, heavy=16)
    gl, gp = Cl.rows_to_host(rows), Cp.rows_to_host(rows)
    same = all(np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8)) for x, y in zip(gl, gp))
    try:
        par = sampled.check_rows(gp, hp, A, rows)
    except AssertionError as e:
        par = {"bitwise": False, "error": str(e)[:300]}
    par["learned_equals_plain"] = same
    Cl.free()
    Cp.free()
    products = int(cum[-1])
    ml, mp = statistics.median(tl), statistics.median(tp)
    return {"desc": WORKLOADS["rmat20_panels"], "value": round(2.0 * products / (ml * 1e-3) / 1e9, 3),
            "unit": "GFLOPS", "ms": round(ml, 3), "plain_ms": round(mp, 3), "plain_value":
            round(2.0 * products / (mp * 1e-3) / 1e9, 3), "speedup_vs_plain": round(mp / ml, 3),
            "reps": reps, "times_ms": {"learned": [round(x, 3) for x in tl], "plain": [round(x, 3) for x in tp]},
            "n": A.M, "nnz_A": A.nnz, "products": products, "nnz_C": nnz_total, "panels": len(panels),
            "fallback_rows": fallback, "slot_entries_over_nnz": round(capacity / max(1, nnz_total), 3),
            "product_bound_over_nnz": round(products / max(1, nnz_total), 3), "margin": margin,
            "timer": "CUDA events around all panels (host reads inside the calls included)",
            "parity": par, "clocks": clocks,
            "reference_gpu": {"unavailable": "nnz(C) ~ 9.7e9 exceeds the reference's int32 CSR (index_t = int, "
                                             "inc/NHC_spgemm.h:13)"}}


# ------------------------------------------------------------------ batched engine
def measure_batched(eng, name, steps, warmup):
    """512 (or 32) Galerkin triple products in one persistent launch (graph replay) vs
    1,024 (64) plain hsmu_spgemm calls, both timed with CUDA events"""
    import numpy as np
    import torch

    import hsmu_gb
    import oracle
    from hsmu_gb import gen

    sides = np.random.default_rng(4).integers(16, 97, size=512)
    if name == "amg32_galerkin":
        sides = sides[:32]
    As, Ps, Pts = [], [], []
    for sd in sides:
        As.append(hsmu_gb.gen_poisson7(int(sd)))
        P, Pt = hsmu_gb.gen_aggregation(int(sd))
        Ps.append(P)
        Pts.append(Pt)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()

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
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    plain_all()
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1)

    b = hsmu_gb.Batch(eng, hsmu_gb.BATCH_GALERKIN, As, Ps, Pts)
    tiny, grid, tune_ms = b.autotune()
    b.graph_launch()
    b.status()
    for _ in range(warmup):
        b.graph_launch()
    torch.cuda.synchronize()
    clocks = ClockSampler(0).start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        b.graph_launch()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    b.status()
    ms = ev0.elapsed_time(ev1) / steps
    # output check: 4 products (the largest grid among them) against the two-stage oracle
    pick = sorted({int(np.argmax(sides)), 0, len(sides) // 2, len(sides) - 1})
    bitwise = True
    for p in pick:
        A, P, Pt = As[p].to_host(), Ps[p].to_host(), Pts[p].to_host()
        rp, col, val = oracle.spgemm(A, P)
        rp, col, val = oracle.spgemm(Pt, gen.CSR(A.M, P.N, rp.astype(np.int32), col, val))
        C = b.result(p).to_host()
        bitwise &= bool(np.array_equal(C.row_ptr.astype(np.int64), rp) and np.array_equal(C.col, col)
                        and np.array_equal(C.val.view(np.int64), val.view(np.int64)))
    peak, peak_kind = load_peaks()
    gbs = alg[0] / (ms * 1e-3) / 1e9
    res = {"desc": WORKLOADS[name], "value": round(2.0 * products / (ms * 1e-3) / 1e9, 3), "unit": "GFLOPS",
           "ms": round(ms, 4), "steps": steps, "products_total": int(products),
           "fine_rows": int((sides.astype(np.int64) ** 3).sum()), "spgemms": 2 * len(sides),
           "plain_calls_ms": round(plain_ms, 3), "plain_calls": 2 * len(sides),
           "plain_value": round(2.0 * products / (plain_ms * 1e-3) / 1e9, 3),
           "speedup_vs_plain": round(plain_ms / ms, 2), "autotuned": {"tiny": tiny, "grid": grid},
           "launches_per_step": 1, "graph": True,
           "roofline": {"bound": "hbm", "kernel": "k_batch (persistent: both products, one pass each, block allocation per tile)",
                        "achieved": round(gbs, 2), "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
                        "peak_kind": peak_kind, "traffic": TRAFFIC.get(name), "alg_bytes": alg[0]},
           "parity": {"products_checked": pick, "bitwise": bitwise},
           "clocks": clk,
           "reference_gpu": {"unavailable": "the reference takes one product per call (the plain engine's "
                                            "1,024 calls stand in)"}}
    b.close()
    return res


def run_batched(args):
    res = measure_batched(__import__("hsmu_gb").Engine(), args.workload, args.steps, args.warmup)
    line = {"metric": METRIC, "value": res["value"], "unit": "GFLOPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (operators generated on the device)",
            "config": {"workload": args.workload, "desc": res["desc"], "products_total": res["products_total"],
                       "fine_rows": res["fine_rows"], "spgemms": res["spgemms"]},
            "roofline": res["roofline"], "batched": res, "clocks": res["clocks"], "gpu_launches": args.steps,
            "parity": res["parity"]}
    print(json.dumps(line), flush=True)


def run_learned_panels(args):
    import hsmu_gb

    res = measure_learned(hsmu_gb.Engine(), reps=max(3, min(args.steps, 5)))
    line = {"metric": METRIC, "value": res["value"], "unit": "GFLOPS", "n_gpus": 1, "steps": res["reps"],
            "warmup": 1, "ms_per_step": res["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded R-MAT scale 20)",
            "config": {"workload": "rmat20_panels", "desc": res["desc"], "n": res["n"], "nnz_A": res["nnz_A"],
                       "products": res["products"], "nnz_C": res["nnz_C"], "panels": res["panels"]},
            "learned": res, "clocks": res["clocks"], "gpu_launches": None, "parity": res["parity"]}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", default=HEADLINE, choices=sorted(WORKLOADS))
    ap.add_argument("--configs", default="all", choices=["all", "none"],
                    help="all: also measure every other stated configuration in the same run (N=1)")
    ap.add_argument("--parity", default="on", choices=["on", "off"],
                    help="check the measured workload's output against the oracle before printing")
    ap.add_argument("--arith", default="rn", choices=sorted(ARITH),
                    help="accumulation: rn = product rounded then added (the reference's arithmetic), "
                         "fma = one fused multiply-add per product, imul = rn with integer-pipe multiply")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_under_torchrun(args))
    elif args.workload in ("amg512_galerkin", "amg32_galerkin"):
        run_batched(args)
    elif args.workload == "rmat20_panels":
        run_learned_panels(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
