"""Benchmark: FP64 Ax=b solves/s (dgetrf + dgetrs) on GB300, plus sub-benchmarks.

Workload (one "step"): the plain-FP64 LU + solve configuration -- n=8192,
column-major A with entries uniform[-1,1] and the diagonal shifted by +n/4,
one right-hand side b = A x_true -- factorised with flens_gb300_dgetrf and
solved with flens_gb300_dgetrs on the device, A restored from a pristine copy
at the start of every step (inside the timed region).  A is 512 MiB, larger
than L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line on rank 0.  value = solves/s (whole job), e2e = the same
metric through the Fortran-ABI dgesv_ with pinned host buffers (host<->device
copies inside the timed region), roofline = the dominant kernel against a
measured FP64 peak, cpu_baseline = the oracle CPU path on a bounded sample.
With --impl reference the reference's CPU implementation (oracle/_ref when it
was built here, else the bitwise-identical C restatement) is timed on all host
cores instead.
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
sys.path.insert(0, ROOT)

METRIC = "Ax=b solves/s at FP64 accuracy (dgetrf+dgetrs, n=8192, 1 rhs)"
UNIT = "solves/s"
NB = 64


def lu_block_flops(n: int, nblocks: int | None = None) -> float:
    """Flops of the blocked right-looking LU (block 64), per block step, summed
    over the first nblocks steps: panel r*w^2 + trsm w^2(r-w) + update 2(r-w)^2 w."""
    fl, b, j = 0.0, 0, 0
    while j < n and (nblocks is None or b < nblocks):
        r = n - j
        w = min(NB, r)
        fl += r * w * w + w * w * (r - w) + 2.0 * (r - w) * (r - w) * w
        j += NB
        b += 1
    return fl


def l2_note(n: int, what: str = "input") -> str:
    """The L2 line of a config: the size of an n x n FP64 matrix against the
    129 MB L2 (below it, every step would re-read it from L2)."""
    mib = 8.0 * n * n / 2 ** 20
    rel = ">" if 8.0 * n * n > 129e6 else "<"
    return f"{what} {mib:.0f} MiB {rel} L2"


def lu_step_flops(n: int, b: int) -> float:
    """Flops of block step b (nb = 64) of the n x n blocked LU."""
    r = n - NB * b
    w = min(NB, r)
    return r * w * w + w * w * (r - w) + 2.0 * (r - w) * (r - w) * w


def lu_sample_blocks(n: int) -> list[int]:
    """Block steps spread over the factorisation (n = 8192: 0, 32, 64, 96, 120):
    the first carries the largest trailing update, the late ones are small
    and cache-resident, so their per-flop rates differ."""
    nsteps = -(-n // NB)
    return sorted({min(nsteps - 1, int(round(f * nsteps))) for f in (0.0, 0.25, 0.5, 0.75, 0.9375)})


def lu_seconds_from_samples(n: int, rates: dict) -> float:
    """Time of the whole LU plus the two triangular solves from per-flop rates
    measured at a few block steps: the rate is interpolated linearly in the
    step index between the samples (flat beyond the last), each step's flops
    divided by its rate, and the 2 n^2 flops of trs taken at the mean rate."""
    nsteps = -(-n // NB)
    bs = sorted(rates)
    total = 0.0
    for b in range(nsteps):
        if b <= bs[0]:
            rt = rates[bs[0]]
        elif b >= bs[-1]:
            rt = rates[bs[-1]]
        else:
            hi = next(x for x in bs if x >= b)
            lo = max(x for x in bs if x <= b)
            rt = rates[lo] if hi == lo else rates[lo] + (rates[hi] - rates[lo]) * (b - lo) / (hi - lo)
        total += lu_step_flops(n, b) / rt
    return total + 2.0 * n * n / (sum(rates.values()) / len(rates))


# ------------------------------------------------------------- clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        if self.gpu is None:
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------ reference arm --
def reference_arm(args, rank: int) -> None:
    if rank != 0:
        return
    import oracle
    n = args.n
    threads = os.cpu_count() or 1
    kind = "port"
    # the C restatement is bitwise identical to the reference's own trf
    # (pinned by tests/test_oracle_pin.py); oracle/_ref is only on machines
    # that hold the FLENS sources, and has no partial-factorisation entry.
    port = oracle.Port()
    # each timed step runs one block step of the factorisation on every host
    # thread (each on its own n x n copy), cycling through block steps spread
    # over the factorisation; the per-flop rate of each sampled step is the
    # mean over its repetitions, and the whole dgetrf+dgetrs time follows from
    # those rates (lu_seconds_from_samples)
    blocks = lu_sample_blocks(n)
    for w in range(args.warmup):
        port.time_dgetrf_step_at(n, blocks[-1], threads, seed=7 + w)
    times, per_block = [], {b: [] for b in blocks}
    for s in range(args.steps):
        b = blocks[s % len(blocks)]
        t, fl = port.time_dgetrf_step_at(n, b, threads, seed=11 + s)
        times.append(t)
        per_block[b].append(fl / t)
    if any(not v for v in per_block.values()):       # fewer steps than sample points
        for b, v in per_block.items():
            if not v:
                t, fl = port.time_dgetrf_step_at(n, b, threads, seed=99 + b)
                v.append(fl / t)
    rates = {b: statistics.mean(v) for b, v in per_block.items()}
    per_solve_s = lu_seconds_from_samples(n, rates)
    # each thread factorised its own copy: `threads` solves per that wall time
    value = threads / per_solve_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (splitmix64 uniform[-1,1] + n/4 diagonal, seeded)",
        "config": {"workload": f"dgetrf+dgetrs n={n} 1 rhs FP64 column-major", "n": n,
                   "nrhs": 1, "l2": l2_note(n)},
        "cpu_baseline": {
            "value": value, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": (f"step s: {threads} threads each run block step {blocks}[s mod {len(blocks)}] "
                       f"(panel+laswp+trsm+trailing gemm, nb=64) of the n={n} LU on its own copy; "
                       f"whole dgetrf+dgetrs from the per-flop rates of those steps interpolated "
                       f"over all {-(-n // NB)} block steps ({per_solve_s:.1f} s per thread)"),
            "rates_gflops_per_thread": {str(b): round(r / 1e9, 4) for b, r in rates.items()}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ our arm --
def make_inputs(torch, n, seed, dev, shift=True):
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    A0 = torch.rand((n, n), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
    if shift:
        A0.diagonal().add_(n / 4.0)
    A0 = A0.t()  # column-major view: stride(0) == 1
    x_true = torch.rand((n, 1), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
    b0 = A0 @ x_true
    return A0, x_true, b0


def fp64_peak(torch, dev):
    """cuBLAS FP64 GEMM throughput (TFLOP/s), best of 3 at 8192^3, as the
    measured FP64 roofline for this GPU."""
    n = 8192
    a = torch.rand((n, n), dtype=torch.float64, device=dev)
    b = torch.rand((n, n), dtype=torch.float64, device=dev)
    c = a @ b
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b, c
    return best


def gemm_subbench(torch, fg, dev, reps=10):
    """Config 1: C = 1.5*A*B + 0.5*C, M=N=K=1024 FP64, through flens_gb300_dgemm.
    L2 is flushed (a 256 MiB write) between timed repetitions."""
    n = 1024
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    A = torch.rand((n, n), generator=g, dtype=torch.float64, device=dev).t()
    B = torch.rand((n, n), generator=g, dtype=torch.float64, device=dev).t()
    C0 = torch.rand((n, n), generator=g, dtype=torch.float64, device=dev).t()
    C = fg.to_colmajor(C0.clone())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(3):
        fg.dgemm_dev("N", "N", 1.5, A, B, 0.5, C)
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(reps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fg.dgemm_dev("N", "N", 1.5, A, B, 0.5, C)
        e1.record()
        e1.synchronize()
        tot += e0.elapsed_time(e1)
    ms = tot / reps
    return {"workload": "dgemm 1024^3 alpha=1.5 beta=0.5 FP64", "ms": ms,
            "tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12, "l2": "flushed between reps"}


def our_arm(args, rank: int, world: int) -> None:
    import numpy as np
    import torch
    import flens_gb300 as fg

    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    n = args.n
    stream = torch.cuda.current_stream()
    A0, x_true, b0 = make_inputs(torch, n, 20261203 + rank, dev, shift=not args.unshifted)
    A = fg.to_colmajor(A0.clone())
    b = b0.clone()
    ipiv = torch.zeros(n, dtype=torch.int32, device=dev)
    info = torch.zeros(1, dtype=torch.int32, device=dev)

    def step():
        A.copy_(A0)
        b.copy_(b0)
        fg.dgetrf_dev(A, ipiv, info, stream)
        fg.dgetrs_dev("N", A, ipiv, b, stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    fg.sync(stream)

    # -- timed region
    fg.timing_enable(True)
    launches0 = fg.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = fg.launch_count() - launches0
    ms_total = e0.elapsed_time(e1)
    fam = fg.timing_read()
    fg.timing_enable(False)
    fg.sync(stream)
    if dist:
        t = torch.tensor([ms_total], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())

    # -- accuracy of the last solve
    inf = int(info.item())
    piv = ipiv.cpu().numpy()
    pivots_identity = bool(np.array_equal(piv, np.arange(1, n + 1)))
    x = b
    r = b0 - A0 @ x
    eps = float(np.finfo(np.float64).eps)
    anorm = A0.abs().sum(0).max().item()
    berr_solve = (r.abs().max() / (anorm * x.abs().max() + b0.abs().max())).item()
    fwd = ((x - x_true).abs().max() / x_true.abs().max()).item()

    value = world * args.steps / (ms_total * 1e-3)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": ("synthetic (torch seeded uniform[-1,1], NO diagonal shift: profiling input; b = A x_true)"
                 if args.unshifted else "synthetic (torch seeded uniform[-1,1] + n/4 diagonal; b = A x_true)"),
        "config": {"workload": f"dgetrf+dgetrs n={n} 1 rhs FP64 column-major",
                   "n": n, "nrhs": 1, "nb": NB, "parallelism": f"replicas x{world}",
                   "l2": l2_note(n) + " (no flush)",
                   "step": "A,b restored from pristine copies + dgetrf + dgetrs"},
        "gpu_launches": launches,
        "accuracy": {"info": inf, "pivots_identity": pivots_identity,
                     "backward_error_normwise": berr_solve,
                     "backward_error_over_n_eps": berr_solve / (n * eps),
                     "forward_error_vs_x_true": fwd},
        "clocks": clk.summary(),
        "kernels": {k: {"ms_per_step": v["ms"] / args.steps, "launches_per_step": v["launches"] / args.steps,
                        "tflops": (v["flops"] / (v["ms"] * 1e-3) / 1e12) if v["ms"] > 0 else None}
                    for k, v in fam.items()},
    }

    if rank == 0:
        # -- e2e through the Fortran ABI with pinned host buffers, right after
        # the device-resident leg and before anything else runs (the cuBLAS
        # peak and the sub-benchmarks below leave seconds of heavy load and
        # several GB of workspace behind them)
        if not args.no_e2e:
            result["e2e"] = e2e_dgesv(torch, fg, A0, b0, args)
        # -- dominant kernel vs the measured FP64 peak
        cublas_peak = None if args.quick else fp64_peak(torch, dev)
        # FP64 pipe issue rate (ncu: 2 DFMA per cycle per SM) at the sampled clock
        sm_mhz = result["clocks"].get("sm_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        pipe_peak = 2 * 2 * sms * sm_mhz * 1e6 / 1e12
        peak = max(p for p in (cublas_peak, pipe_peak) if p)
        dom = max(fam.items(), key=lambda kv: kv[1]["ms"])[0] if fam else None
        if dom:
            d = fam[dom]
            achieved = d["flops"] / (d["ms"] * 1e-3) / 1e12
            # DRAM bytes per launch: the ncu-measured DRAM/algorithmic ratio of
            # this kernel (profiles/traffic.json) times its per-launch
            # algorithmic bytes in this run
            traffic = None
            tpath = os.path.join(ROOT, "profiles", "traffic.json")
            if os.path.exists(tpath):
                ratio = json.load(open(tpath)).get(dom, {}).get("dram_over_algorithmic")
                if ratio and d["launches"]:
                    traffic = ratio * d["bytes"] / d["launches"]
            result["roofline"] = {
                "kernel": dom, "bound": "fp64_pipe", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": (achieved / peak) if peak else None,
                "traffic": traffic,
                "peak_source": ("max of cuBLAS FP64 dgemm 8192^3 measured in this run "
                                f"({cublas_peak}) and the FP64 pipe issue rate 2 DFMA/clk/SM x "
                                f"{sms} SMs x {sm_mhz} MHz ({pipe_peak:.3f}); MEASURED_PEAKS.json "
                                "has no FP64 entry and tcgen05 has no f64 kind"),
                "share_of_step": d["ms"] / ms_total,
                "algorithmic": "2*m*n*k flops per trailing-update/trsm GEMM launch"}
        if not args.quick:
            result["gemm_fp64_config1"] = gemm_subbench(torch, fg, dev)
        if not args.quick and not args.no_mixed:
            result["mixed_config3"] = mixed_subbench(torch, fg, dev, n=args.mixed_n)
        if not args.quick and not args.no_split:
            result["split_gemm_config4"] = split_subbench(torch, fg, dev, cublas_tflops=cublas_peak)
        if not args.quick and not args.no_cholesky:
            result["cholesky_fp64"] = cholesky_subbench(torch, fg, dev)
            result["inverse_fp64"] = inverse_subbench(torch, fg, dev)
            result["blas3_fp64"] = blas3_subbench(torch, fg, dev)
            result["tcgen05_kinds"] = tc_kinds_subbench(torch, fg, dev)
        if not args.quick and not args.no_batched:
            result["batched_config5"] = batched_subbench(torch, fg, dev, count=args.batch_count)
        # -- CPU baseline (oracle C restatement, 1 thread, bounded sample)
        if not args.no_cpu:
            result["cpu_baseline"] = cpu_baseline(n)
        print(json.dumps(result), flush=True)
    if dist:
        dist.destroy_process_group()


# (kappa, nrhs, label, precision, solver, max_iter): precision 0 TF32, 1 BF16,
# 2 FP8 e4m3, 3 FP32-accurate 3xTF32, 5 / 6 FP8 e4m3 with two / three terms
# per entry (all FP32 storage), 4 split (FP64 storage, FP64-accurate
# split-GEMM trailing updates); solver 0 classical, 1 GMRES-IR, 2 classical
# switching to GMRES-IR.  The one- and two-term FP8 and the FP32 kappa=1e10
# cases are capped: their factors are too inexact a preconditioner at this n,
# and the lines report where the refinement stands after the cap.
MIXED_CASES = (
    (1e2, 1, "fp32(3xTF32)", 3, 2, 30),
    (1e2, 1, "tf32", 0, 2, 30),
    (1e2, 1, "bf16", 1, 2, 30),
    (1e2, 1, "fp8", 2, 2, 4),
    (1e2, 1, "fp8x2", 5, 2, 4),
    (1e2, 1, "fp8x3", 6, 2, 30),
    (1e2, 1, "split", 4, 2, 30),
    (1e2, 64, "fp32(3xTF32)", 3, 2, 30),
    (1e2, 64, "split", 4, 2, 30),
    (1e6, 1, "fp32(3xTF32)", 3, 2, 30),
    (1e6, 1, "split", 4, 2, 30),
    (1e10, 1, "split", 4, 2, 30),
    (1e10, 1, "fp32(3xTF32)", 3, 1, 4),
    (1e10, 64, "split", 4, 2, 30),
)


def mixed_subbench(torch, fg, dev, n=16384, reps=3, cases=None, gen="svd"):
    """Mixed-solve configuration: A = U diag(s) V^T (U, V from Householder QR of
    seeded Gaussian matrices, s geometric 1 -> 1/kappa), b = A x_true with 1 or
    64 right-hand sides.  Times flens_gb300_dgesv_mixed in every factor
    precision (MIXED_CASES) against the plain FP64 dgetrf+dgetrs on the same
    n and nrhs, and reports refinement steps, backward and forward error.  A
    case whose first run takes over 2 s is reported from that single run."""
    import ctypes
    import numpy as np
    eps = float(np.finfo(np.float64).eps)
    g = torch.Generator(device=dev)
    g.manual_seed(2026)
    t0 = time.time()
    if gen == "svd":
        U, _ = torch.linalg.qr(torch.randn((n, n), generator=g, dtype=torch.float64, device=dev))
        V, _ = torch.linalg.qr(torch.randn((n, n), generator=g, dtype=torch.float64, device=dev))
    else:
        # profiling input without torch.linalg (which a profiler may fail to
        # load): unshifted uniform[-1,1), kappa in the 1e4-1e5 range
        U = V = None
    gen_s = time.time() - t0
    f = fg.lib().flens_gb300_dgesv_mixed
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int),
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    f.restype = ctypes.c_int
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    out = {"workload": f"dgesv_mixed n={n}, 1 and 64 rhs, A=U diag(s) V^T, s geometric 1..1/kappa",
           "n": n, "generation_s": round(gen_s, 1), "plain_fp64": {}, "cases": []}
    solver_names = {0: "classical", 1: "gmres-ir", 2: "classical->gmres-ir"}
    plain = {}
    mats, rhs = {}, {}

    def system(kappa, nrhs):
        if kappa not in mats:
            mats.clear()
            rhs.clear()
            torch.cuda.empty_cache()
            if U is None:
                A = fg.to_colmajor(torch.rand((n, n), generator=g, dtype=torch.float64,
                                              device=dev).mul_(2).sub_(1))
            else:
                s = kappa ** (-torch.arange(n, dtype=torch.float64, device=dev) / (n - 1))
                A = fg.to_colmajor((U * s) @ V.t())
            mats[kappa] = (A, A.abs().sum(1).max())
        A, anorm = mats[kappa]
        if nrhs not in rhs:
            x = torch.rand((n, nrhs), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
            rhs[nrhs] = (fg.to_colmajor(A @ x), x)
        b, x = rhs[nrhs]
        return A, b, x, anorm

    def berr_of(A, X, b, anorm):
        r = b - A @ X
        return (r.abs().amax(0) / (anorm * X.abs().amax(0) + b.abs().amax(0))).max().item()

    for kappa, nrhs, label, prec, solver, max_iter in MIXED_CASES:
        if cases and label not in cases:
            continue
        A, b, x, anorm = system(kappa, nrhs)
        if nrhs not in plain:
            # plain FP64 GPU solve on the same n and nrhs (timed after one warm-up)
            W = fg.to_colmajor(A.clone())
            bb = fg.to_colmajor(b.clone())
            ipiv = torch.zeros(n, dtype=torch.int32, device=dev)
            inf = torch.zeros(1, dtype=torch.int32, device=dev)
            for rep in range(2):
                W.copy_(A)
                bb.copy_(b)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fg.dgetrf_dev(W, ipiv, inf, stream)
                fg.dgetrs_dev("N", W, ipiv, bb, stream)
                e1.record(stream)
                e1.synchronize()
                plain_ms = e0.elapsed_time(e1)
            pb = berr_of(A, bb, b, anorm)
            plain[nrhs] = plain_ms
            out["plain_fp64"][f"nrhs{nrhs}"] = {"ms": plain_ms, "kappa": kappa, "backward_error": pb,
                                                "backward_error_over_n_eps": pb / (n * eps)}
            del W, bb
        X = fg.colmajor_empty(n, nrhs, device=dev)
        it, be, inf_ = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
        times = []
        st = 0
        rep = 0
        while rep < 1 + reps:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = f(n, nrhs, A.data_ptr(), n, b.data_ptr(), n, X.data_ptr(), n, prec, solver, max_iter,
                   0.0, ctypes.byref(it), ctypes.byref(be), ctypes.byref(inf_), sp)
            torch.cuda.synchronize()
            dt = 1000.0 * (time.perf_counter() - t0)
            if rep == 0 and dt > 2000.0:
                times = [dt]
                break
            if rep > 0:
                times.append(dt)
            rep += 1
        ms = sum(times) / len(times)
        # one more run with per-launch event timing: where the time goes
        fg.timing_enable(True)
        torch.cuda.synchronize()
        f(n, nrhs, A.data_ptr(), n, b.data_ptr(), n, X.data_ptr(), n, prec, solver, max_iter,
          0.0, ctypes.byref(it), ctypes.byref(be), ctypes.byref(inf_), sp)
        torch.cuda.synchronize()
        fam = fg.timing_read()
        fg.timing_enable(False)
        kernels = {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                       "gbs": (round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["ms"] > 0 else None)}
                   for k, v in sorted(fam.items(), key=lambda kv: -kv[1]["ms"])}
        berr = berr_of(A, X, b, anorm)
        fwd = ((X - x).abs().amax(0) / x.abs().amax(0)).max().item()
        out["cases"].append({"kappa": kappa, "nrhs": nrhs, "factor_precision": label,
                             "solver": solver_names[solver], "max_iter": max_iter, "status": st,
                             "ms": ms, "timed_runs": len(times), "iterations": it.value,
                             "backward_error": berr, "backward_error_over_n_eps": berr / (n * eps),
                             "forward_error": fwd,
                             "time_ratio_vs_plain_fp64": ms / plain[nrhs],
                             "meets_10_n_eps": berr <= 10 * n * eps,
                             "kernels": kernels})
        del X
    mats.clear()
    rhs.clear()
    U = V = None
    torch.cuda.empty_cache()
    return out


def measured_peak(key):
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        v = json.load(open(path)).get(key)
        if v:
            return float(v), "measured"
    return {"bf16_tflops": 1900.0, "hbm_gbs": 6800.0}[key], "fallback"


def wide_range_pair(torch, n, E, seed, dev):
    """A, B (n x n, column-major FP64): u * 2^e, u uniform[-1,1], e uniform
    integer in [-E, E] (seeded torch generator)."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    out = []
    for _ in range(2):
        u = torch.rand((n, n), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
        e = torch.randint(-E, E + 1, (n, n), generator=g, device=dev).to(torch.float64)
        out.append(torch.ldexp(u, e).t())       # column-major view
        del u, e
    return out


def split_subbench(torch, fg, dev, n=8192, Es=(0, 16, 48), reps=5, ref_slices=14,
                   cublas_tflops=None):
    """Split-precision FP64 GEMM configuration: C = A*B, M = N = K = n, entries
    u*2^e with e uniform in [-E, E].  Times flens_gb300_dgemm_split (stats,
    slicing, exact BF16 tcgen05 products, FP64 recombination; inputs 512 MiB
    each > L2) and, beside it, the plain FP64 dgemm kernel.  Accuracy: max
    elementwise relative error of both against the same kernel run with
    `ref_slices` slices (7*ref_slices bits per operand; the kernel matches its
    NumPy model bit for bit and the reference's gemm to 1e-13 in the tests)."""
    import numpy as np
    peak, peak_src = measured_peak("bf16_tflops")
    out = {"workload": f"dgemm {n}^3 FP64 in/out, entries u*2^e, e in [-E,E]",
           "fp64_equivalent_flops": 2.0 * n ** 3, "l2": l2_note(n, "inputs, each") + " (no flush)",
           "accuracy_reference": f"same kernel with {ref_slices} slices ({7 * ref_slices} bits)",
           "per_E": {}}
    stream = torch.cuda.current_stream()
    plain_ms = None
    for E in Es:
        A, B = wide_range_pair(torch, n, E, 4000 + E, dev)
        C = torch.zeros((n, n), dtype=torch.float64, device=dev).t()
        S = fg.dgemm_split_dev("N", "N", 1.0, A, B, 0.0, C)      # warm-up, picks S
        torch.cuda.synchronize()
        fg.timing_enable(True)
        times = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fg.dgemm_split_dev("N", "N", 1.0, A, B, 0.0, C)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        fam = fg.timing_read()
        fg.timing_enable(False)
        ms = sum(times) / len(times)
        sp = fam.get("split_gemm", {"ms": 0.0, "flops": 0.0, "launches": 0})
        k_ms = sp["ms"] / max(1, sp["launches"])
        tc_tflops = sp["flops"] / max(1e-9, sp["ms"] * 1e-3) / 1e12
        # accuracy against the many-slice result
        Cref = torch.zeros((n, n), dtype=torch.float64, device=dev).t()
        fg.dgemm_split_dev("N", "N", 1.0, A, B, 0.0, Cref, slices=ref_slices)
        C64 = torch.zeros((n, n), dtype=torch.float64, device=dev).t()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fg.dgemm_dev("N", "N", 1.0, A, B, 0.0, C64)
        e1.record(stream)
        e1.synchronize()
        plain_ms = e0.elapsed_time(e1)
        den = Cref.abs()
        nz = den > 0
        rel_split = ((C - Cref).abs()[nz] / den[nz]).max().item()
        rel_plain = ((C64 - Cref).abs()[nz] / den[nz]).max().item()
        norm_split = ((C - Cref).abs().max() / den.max()).item()
        out["per_E"][str(E)] = {
            "slices": S, "ms": ms, "fp64_equiv_tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12,
            "products_kernel_ms": k_ms, "tensor_tflops": tc_tflops,
            "tensor_frac_of_bf16_peak": tc_tflops / peak,
            "max_rel_err_split": rel_split, "max_rel_err_plain_fp64": rel_plain,
            "normwise_rel_err_split": norm_split,
            "speedup_vs_plain_fp64": plain_ms / ms,
            "kernels_ms_per_call": {k: v["ms"] / reps for k, v in fam.items() if v["ms"] > 0}}
        del A, B, C, Cref, C64
        torch.cuda.empty_cache()
    out["plain_fp64_dgemm"] = {"ms": plain_ms, "tflops": 2.0 * n ** 3 / (plain_ms * 1e-3) / 1e12,
                               "cublas_fp64_tflops": cublas_tflops}
    out["bf16_peak_tflops"] = {"value": peak, "source": f"{peak_src} (MEASURED_PEAKS.json bf16_tflops)"}
    return out


def tc_kinds_subbench(torch, fg, dev, n=8192, reps=3):
    """The tcgen05 GEMM kernel per operand kind at a compute-bound shape
    (flens_gb300_sgemm_tc, M = N = K = 8192, FP32 in/out): kernel-only
    TFLOP/s from the library's per-launch CUDA events (the call also converts
    the FP32 operands to the kind's K-major copies, timed separately as aux),
    against the measured dense BF16 peak scaled by the kind's nominal rate
    (TF32 1/2, FP8 2x; 3xTF32 and two-term FP8 run one product over 3K)."""
    import ctypes
    bf16, src = measured_peak("bf16_tflops")
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    A = torch.rand((n, n), generator=g, dtype=torch.float32, device=dev).t()
    B = torch.rand((n, n), generator=g, dtype=torch.float32, device=dev).t()
    C = torch.zeros((n, n), dtype=torch.float32, device=dev).t()
    f = fg.lib().flens_gb300_sgemm_tc
    f.argtypes = [ctypes.c_int, ctypes.c_char, ctypes.c_char] + [ctypes.c_int] * 3 + [
        ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
        ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {"workload": f"sgemm_tc {n}^3, FP32 in/out, tcgen05 kernel only", "kinds": {},
           "bf16_peak_tflops": {"value": bf16, "source": f"{src} (MEASURED_PEAKS.json bf16_tflops)"}}
    for prec, name, rate in ((0, "tf32", 0.5), (1, "bf16", 1.0), (2, "fp8_e4m3", 2.0),
                             (3, "3xtf32", 0.5), (5, "fp8x2_e4m3", 2.0), (6, "fp8x3_e4m3", 2.0)):
        st = f(prec, b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.0,
               C.data_ptr(), n, sp)
        if st != 0:
            out["kinds"][name] = {"error": fg.last_error()}
            continue
        torch.cuda.synchronize()
        fg.timing_enable(True)
        for _ in range(reps):
            f(prec, b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.0,
              C.data_ptr(), n, sp)
        fam = fg.timing_read()
        fg.timing_enable(False)
        tc = fam.get("tc_gemm", {"ms": 0.0, "flops": 0.0})
        tfl = tc["flops"] / max(1e-9, tc["ms"] * 1e-3) / 1e12
        kind_peak = bf16 * rate
        out["kinds"][name] = {"kernel_ms": tc["ms"] / reps, "tensor_tflops": tfl,
                              "kind_peak_tflops": kind_peak, "frac_of_kind_peak": tfl / kind_peak,
                              "conversion_ms": fam.get("aux", {"ms": 0.0})["ms"] / reps}
    del A, B, C
    torch.cuda.empty_cache()
    return out


def blas3_subbench(torch, fg, dev, n=4096, reps=3):
    """Level-3 BLAS at n = 4096 (FP64, column-major, device memory, L2
    flushed by the 128 MiB operands): gemm in its four transpose variants,
    syrk, syr2k, trmm, symm through the flens_gb300_* entry points, each as
    TFLOP/s of its algorithmic count (gemm, symm 2n^3; syrk n^3, syr2k 2n^3,
    trmm n^3)."""
    import ctypes
    L = fg.lib()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    g = torch.Generator(device=dev)
    g.manual_seed(33)
    mk = lambda: fg.to_colmajor(torch.rand((n, n), generator=g, dtype=torch.float64, device=dev) - 0.5)
    A, B, C = mk(), mk(), mk()
    calls = {
        "gemm NN": (2.0, lambda: L.flens_gb300_dgemm(b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.5, C.data_ptr(), n, sp)),
        "gemm NT": (2.0, lambda: L.flens_gb300_dgemm(b"N", b"T", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.5, C.data_ptr(), n, sp)),
        "gemm TN": (2.0, lambda: L.flens_gb300_dgemm(b"T", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.5, C.data_ptr(), n, sp)),
        "gemm TT": (2.0, lambda: L.flens_gb300_dgemm(b"T", b"T", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.5, C.data_ptr(), n, sp)),
        "syrk LN": (1.0, lambda: L.flens_gb300_dsyrk(b"L", b"N", n, n, 1.0, A.data_ptr(), n, 0.5, C.data_ptr(), n, sp)),
        "syr2k UT": (2.0, lambda: L.flens_gb300_dsyr2k(b"U", b"T", n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.5, C.data_ptr(), n, sp)),
        "trmm LUNN": (1.0, lambda: L.flens_gb300_dtrmm(b"L", b"U", b"N", b"N", n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, sp)),
        "symm LL": (2.0, lambda: L.flens_gb300_dsymm(b"L", b"L", n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.5, C.data_ptr(), n, sp)),
    }
    out = {"workload": f"level-3 BLAS n={n} FP64", "n": n, "tflops": {}, "ms": {}}
    for name, (fmul, f) in calls.items():
        times = []
        for rep in range(1 + reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = f()
            e1.record(stream)
            e1.synchronize()
            assert st == 0, (name, fg.last_error())
            if rep:
                times.append(e0.elapsed_time(e1))
        ms = sum(times) / len(times)
        out["ms"][name] = ms
        out["tflops"][name] = fmul * n ** 3 / (ms * 1e-3) / 1e12
    del A, B, C
    torch.cuda.empty_cache()
    return out


def cholesky_subbench(torch, fg, dev, n=8192, reps=3):
    """Cholesky solve configuration: A = G G^T / n + I (G seeded uniform[-1,1]),
    b = A x_true, one rhs, through flens_gb300_dposv (dpotrf + dpotrs) with A
    and b restored from pristine copies inside every timed repetition (A is
    512 MiB > L2).  FLOP count n^3/3 + 2 n^2."""
    g = torch.Generator(device=dev)
    g.manual_seed(81)
    Gm = torch.rand((n, n), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
    A0 = torch.addmm(torch.eye(n, dtype=torch.float64, device=dev), Gm, Gm.T, alpha=1.0 / n)
    del Gm
    A0 = A0.t()                                   # column-major view (A0 is symmetric)
    x = torch.rand((n, 1), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
    b0 = A0 @ x
    A = fg.to_colmajor(A0.clone())
    b = b0.clone()
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    A.copy_(A0)
    b.copy_(b0)
    fg.dposv_dev("L", A, b, info)
    torch.cuda.synchronize()
    fg.timing_enable(True)
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        A.copy_(A0)
        b.copy_(b0)
        fg.dposv_dev("L", A, b, info)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    fam = fg.timing_read()
    fg.timing_enable(False)
    ms = sum(times) / len(times)
    flop = n ** 3 / 3.0 + 2.0 * n * n
    L = torch.tril(A)
    R = torch.tril(A0 - L @ L.T)
    eps = float(torch.finfo(torch.float64).eps)
    be = (R.abs().sum(0).max() / (n * A0.abs().sum(0).max() * eps)).item()
    out = {"workload": f"dposv n={n} 1 rhs FP64, A = G G^T/n + I", "n": n, "ms": ms,
           "tflops": flop / (ms * 1e-3) / 1e12, "info": int(info.item()),
           "backward_error_over_n_eps": be,
           "forward_error": ((b - x).abs().max() / x.abs().max()).item(),
           "kernels_ms_per_call": {k: v["ms"] / reps for k, v in fam.items()},
           "launches_per_call": {k: v["launches"] / reps for k, v in fam.items()},
           "l2": "A restored from a pristine copy each rep (512 MiB > L2)"}
    del A, A0, b, b0
    torch.cuda.empty_cache()
    return out


def inverse_subbench(torch, fg, dev, n=8192, reps=2):
    """Matrix inverse configuration: A uniform[-1,1] + n/4 I (n = 8192), dgetrf
    then dgetri through the device entry points, A restored from a pristine
    copy each repetition.  FLOP count 2 n^3 ((2/3) n^3 LU + (4/3) n^3 inverse)."""
    g = torch.Generator(device=dev)
    g.manual_seed(91)
    A0 = torch.rand((n, n), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
    A0.diagonal().add_(n / 4.0)
    A0 = A0.t()
    A = fg.to_colmajor(A0.clone())
    ipiv = torch.zeros(n, dtype=torch.int32, device=dev)
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()

    def run():
        A.copy_(A0)
        fg.dgetrf_dev(A, ipiv, info, stream)
        st = fg.lib().flens_gb300_dgetri(n, A.data_ptr(), n, ipiv.data_ptr(), info.data_ptr(),
                                         ctypes_stream(stream))
        assert st == 0, fg.last_error()

    run()
    torch.cuda.synchronize()
    fg.timing_enable(True)
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    fam = fg.timing_read()
    fg.timing_enable(False)
    ms = sum(times) / len(times)
    R = A0 @ A - torch.eye(n, dtype=torch.float64, device=dev)
    nrm = lambda M: M.abs().sum(0).max().item()
    eps = float(torch.finfo(torch.float64).eps)
    out = {"workload": f"dgetrf+dgetri n={n} FP64", "n": n, "ms": ms,
           "tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12, "info": int(info.item()),
           "residual_over_n_eps": nrm(R) / (n * nrm(A0) * nrm(A) * eps),
           "kernels_ms_per_call": {k: v["ms"] / reps for k, v in fam.items()},
           "l2": "A restored from a pristine copy each rep (512 MiB > L2)"}
    del A, A0, R
    torch.cuda.empty_cache()
    return out


def ctypes_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


def batched_cpu_baseline(sample=4000, seed=55):
    """The batched configuration on the host cores: the oracle's dgesv (the C
    restatement of the reference's trf + trs, bitwise the reference) over a
    sample of matrices drawn like the batch (n log-uniform in [8, 512],
    uniform[-1,1] + n/4 on the diagonal, k in {1, 4, 16}), one worker thread
    per host core, each solving its share of the sample (the C calls release
    the interpreter lock).  Returns solves/s for the whole host."""
    import concurrent.futures as cf
    import numpy as np
    import oracle
    rng = np.random.default_rng(seed)
    n = np.floor(np.exp(rng.uniform(np.log(8), np.log(512.999), size=sample))).astype(np.int32)
    k = rng.choice(np.array([1, 4, 16], dtype=np.int32), size=sample)
    mats = []
    for i in range(sample):
        A = oracle.uniform(rng, int(n[i]), int(n[i]))
        A[np.arange(n[i]), np.arange(n[i])] += n[i] / 4.0
        mats.append((A, oracle.uniform(rng, int(n[i]), int(k[i]))))
    port = oracle.Port()
    threads = os.cpu_count() or 1

    def work(lo):
        for i in range(lo, sample, threads):
            port.dgesv(mats[i][0], mats[i][1])

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(work, range(threads)))
    t = time.perf_counter() - t0
    flops = float(np.sum(2.0 / 3.0 * n.astype(np.float64) ** 3 + 2.0 * n.astype(np.float64) ** 2 * k))
    return {"value": sample / t, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": (f"{sample} matrices drawn like the batch, oracle dgesv (bitwise the "
                       f"reference's trf+trs), {threads} threads, {t:.2f} s"),
            "gflops": flops / t / 1e9}


def batched_subbench(torch, fg, dev, count=20000, reps=3, loop_sample=2000, uniform=None):
    """Batched configuration: `count` independent FP64 systems, n log-uniform
    in [8, 512], entries uniform[-1,1] + (n/4) I, k uniform in {1, 4, 16}.
    Times one plan execution (one persistent launch, graph replay) in FP64 and
    in FP32 LU + FP64 refinement, against a per-matrix flens_gb300_dgesv loop
    (timed on the first `loop_sample` matrices and scaled), and reports
    p50/p99 normwise backward errors.  uniform=(N, K): every matrix N x N
    with K right-hand sides instead (for profiling one size)."""
    import ctypes
    import numpy as np
    rng = np.random.default_rng(55)
    n = np.floor(np.exp(rng.uniform(np.log(8), np.log(512.999), size=count))).astype(np.int32)
    k = rng.choice(np.array([1, 4, 16], dtype=np.int32), size=count)
    if uniform:
        n = np.full(count, uniform[0], dtype=np.int32)
        k = np.full(count, uniform[1], dtype=np.int32)
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)])
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) * k)])
    g = torch.Generator(device=dev)
    g.manual_seed(77)
    F0 = torch.rand(int(a_off[-1]), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
    diag = np.concatenate([a_off[i] + np.arange(n[i]) * (n[i] + 1) for i in range(count)])
    shift = np.concatenate([np.full(n[i], n[i] / 4.0) for i in range(count)])
    F0[torch.from_numpy(diag).to(dev)] += torch.from_numpy(shift).to(dev)
    G0 = torch.rand(int(b_off[-1]), generator=g, dtype=torch.float64, device=dev).mul_(2).sub_(1)
    F, G = F0.clone(), G0.clone()
    P = torch.zeros(int(n.sum()), dtype=torch.int32, device=dev)
    p_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))])
    pa = (F.data_ptr() + 8 * a_off[:-1]).astype(np.uint64)
    pb = (G.data_ptr() + 8 * b_off[:-1]).astype(np.uint64)
    pp = (P.data_ptr() + 4 * p_off[:-1]).astype(np.uint64)
    lda = n.copy()
    info = torch.zeros(count, dtype=torch.int32, device=dev)
    iters = torch.zeros(count, dtype=torch.int32, device=dev)
    berr = torch.zeros(count, dtype=torch.float64, device=dev)
    L = fg.lib()
    vp = ctypes.c_void_p
    f = L.flens_gb300_dgesv_batched_plan
    f.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int, vp, vp, ctypes.c_int,
                  vp, ctypes.POINTER(ctypes.c_void_p)]
    f.restype = ctypes.c_int
    L.flens_gb300_batched_execute.argtypes = [vp, vp]
    L.flens_gb300_batched_destroy.argtypes = [vp]
    L.flens_gb300_batched_team.argtypes = [vp, ctypes.c_int]
    L.flens_gb300_batched_team.restype = ctypes.c_int
    L.flens_gb300_batched_panel.argtypes = [vp, ctypes.c_int]
    L.flens_gb300_batched_panel.restype = ctypes.c_int
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    flops = float(np.sum(2.0 / 3.0 * n.astype(np.float64) ** 3 + 2.0 * n.astype(np.float64) ** 2 * k))
    eps = float(np.finfo(np.float64).eps)
    what = (f"n={uniform[0]}, k={uniform[1]}" if uniform else "n log-uniform [8,512], k in {1,4,16}")
    out = {"workload": f"{count} dgesv, {what}", "count": count,
           "flop": flops, "variants": {}}

    def berr_sample(sample):
        errs = []
        for i in sample:
            ni, ki = int(n[i]), int(k[i])
            A = F0[a_off[i]:a_off[i + 1]].view(ni, ni).t()
            B = G0[b_off[i]:b_off[i + 1]].view(ki, ni).t()
            X = G[b_off[i]:b_off[i + 1]].view(ki, ni).t()
            R = B - A @ X
            den = A.abs().sum(1).max() * X.abs().amax(0) + B.abs().amax(0)
            errs.append((R.abs().amax(0) / den).max().item())
        return np.array(errs)

    sample = rng.choice(count, size=min(1000, count), replace=False)
    for prec, name in ((0, "fp64"), (1, "fp32_lu+fp64_ir"), (2, "auto_per_matrix")):
        plan = ctypes.c_void_p()
        t0 = time.time()
        st = f(count, n.ctypes.data, k.ctypes.data, pa.ctypes.data, lda.ctypes.data, pp.ctypes.data,
               pb.ctypes.data, lda.ctypes.data, info.data_ptr(), prec, iters.data_ptr(),
               berr.data_ptr(), 10, sp, ctypes.byref(plan))
        plan_s = time.time() - t0
        if st != 0:
            out["variants"][name] = {"error": fg.last_error()}
            continue
        times = []
        for rep in range(1 + reps):
            F.copy_(F0)
            G.copy_(G0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            L.flens_gb300_batched_execute(plan, sp)
            e1.record(stream)
            e1.synchronize()
            if rep > 0:
                times.append(e0.elapsed_time(e1))
        teams = [L.flens_gb300_batched_team(plan, b) for b in range(16)]
        teams = teams[:teams.index(-1)] if -1 in teams else teams
        panels = [L.flens_gb300_batched_panel(plan, b) for b in range(len(teams))]
        L.flens_gb300_batched_destroy(plan)
        ms = sum(times) / len(times)
        inf = info.cpu().numpy()
        be = berr_sample(sample) / (n[sample] * eps)
        v = {"ms": ms, "solves_per_s": count / (ms * 1e-3), "gflops": flops / (ms * 1e-3) / 1e9,
             "plan_s": round(plan_s, 2), "teams_per_bucket": teams, "panel_per_bucket": panels,
             "info_nonzero": int((inf != 0).sum()),
             "backward_error_over_n_eps_p50": float(np.percentile(be, 50)),
             "backward_error_over_n_eps_p99": float(np.percentile(be, 99)),
             "backward_error_sample": f"{len(sample)} matrices"}
        if prec >= 1:
            it = iters.cpu().numpy()
            v["refinement_steps_mean"] = float(it[it >= 0].mean()) if (it >= 0).any() else None
            v["fp64_fallback"] = int((it < 0).sum())
        out["variants"][name] = v
    # per-matrix launch loop (the baseline the batched launch must beat)
    F.copy_(F0)
    G.copy_(G0)
    ipiv = torch.zeros(512, dtype=torch.int32, device=dev)
    inf1 = torch.zeros(1, dtype=torch.int32, device=dev)
    m = min(loop_sample, count)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(m):
        ni, ki = int(n[i]), int(k[i])
        L.flens_gb300_dgesv(ni, ki, ctypes.c_void_p(int(pa[i])), ni, ctypes.c_void_p(ipiv.data_ptr()),
                            ctypes.c_void_p(int(pb[i])), ni, ctypes.c_void_p(inf1.data_ptr()), sp)
    torch.cuda.synchronize()
    loop_s = (time.perf_counter() - t0) * count / m
    out["per_matrix_loop"] = {"solves_per_s": count / loop_s, "sample": f"first {m} matrices, scaled"}
    fp64 = out["variants"].get("fp64", {})
    if "solves_per_s" in fp64:
        out["speedup_vs_loop_fp64"] = fp64["solves_per_s"] / out["per_matrix_loop"]["solves_per_s"]
    del F0, F, G0, G, P
    torch.cuda.empty_cache()
    if not uniform:
        out["cpu_baseline"] = batched_cpu_baseline()
    return out


def e2e_dgesv(torch, fg, A0, b0, args):
    import ctypes
    import numpy as np
    n = A0.shape[0]
    hA0 = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    hA0.copy_(A0.t())                     # row-major storage of A^T == column-major A
    hb0 = b0.cpu()
    hA = torch.empty_like(hA0, pin_memory=True)
    hb = torch.empty((n,), dtype=torch.float64, pin_memory=True)
    hpiv = torch.zeros(n, dtype=torch.int32, pin_memory=True)
    L = fg.lib()
    i = lambda v: ctypes.byref(ctypes.c_int(v))
    dptr = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))
    iptr = ctypes.cast(hpiv.data_ptr(), ctypes.POINTER(ctypes.c_int))
    info = ctypes.c_int(0)
    times = []
    # the inputs are restored between steps by a single-threaded copy, so
    # that no worker threads of a parallel host copy are still busy on the
    # host cores while the timed call issues its launches
    nA, nA0, nb, nb0 = hA.numpy(), hA0.numpy(), hb.numpy(), hb0[:, 0].numpy()

    def restore():
        np.copyto(nA, nA0)
        np.copyto(nb, nb0)

    for s in range(args.warmup):
        restore()
        L.dgesv_(i(n), i(1), dptr(hA), i(n), iptr, dptr(hb), i(n), ctypes.byref(info))
    with ClockSampler(torch.cuda.current_device() if args.e2e_clocks else None) as clk:
        for s in range(args.steps):
            restore()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            L.dgesv_(i(n), i(1), dptr(hA), i(n), iptr, dptr(hb), i(n), ctypes.byref(info))
            times.append(time.perf_counter() - t0)
    x = hb.numpy()
    ok = info.value == 0 and bool(np.all(np.isfinite(x)))
    return {"value": len(times) / sum(times), "unit": UNIT,
            "h2d_bytes_per_step": 8 * n * n + 8 * n,
            "d2h_bytes_per_step": 8 * n * n + 8 * n + 4 * n,
            "api": "dgesv_ (Fortran ABI, host pointers, pinned)", "ok": ok,
            "ms_per_step": 1000.0 * sum(times) / len(times),
            "ms_per_step_min": 1000.0 * min(times),
            "ms_steps": [round(1000.0 * t, 2) for t in times], "clocks": clk.summary()}


def cpu_baseline(n):
    """The oracle restatement on 1 host thread: block steps spread over the
    n = 8192 factorisation, the whole dgetrf+dgetrs from their per-flop rates
    (lu_seconds_from_samples)."""
    import oracle
    port = oracle.Port()
    blocks = lu_sample_blocks(n)
    rates, spent = {}, 0.0
    for b in blocks:
        t, fl = port.time_dgetrf_step_at(n, b, 1, seed=5 + b)
        rates[b] = fl / t
        spent += t
    per_solve = lu_seconds_from_samples(n, rates)
    return {"value": 1.0 / per_solve, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": (f"block steps {blocks} (nb=64) of the n={n} LU on 1 thread ({spent:.1f} s); "
                       f"whole dgetrf+dgetrs from their per-flop rates interpolated over all "
                       f"{-(-n // NB)} block steps: {per_solve:.1f} s"),
            "rates_gflops": {str(b): round(r / 1e9, 4) for b, r in rates.items()}}


def only(args):
    """One sub-benchmark on its own, for ncu captures of a single kernel family."""
    import torch
    import flens_gb300 as fg
    dev = torch.device("cuda:0")
    if args.only == "tc_gemm":
        import ctypes
        m, n, k = (int(x) for x in args.tc_shape.split(","))
        g = torch.Generator(device=dev)
        g.manual_seed(1)
        A = torch.rand((k, m), generator=g, dtype=torch.float32, device=dev).t()
        B = torch.rand((n, k), generator=g, dtype=torch.float32, device=dev).t()
        C = torch.rand((n, m), generator=g, dtype=torch.float32, device=dev).t()
        f = fg.lib().flens_gb300_sgemm_tc
        f.argtypes = [ctypes.c_int, ctypes.c_char, ctypes.c_char] + [ctypes.c_int] * 3 + [
            ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
            ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        times = []
        for rep in range(1 + args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            st = f(1, b"N", b"N", m, n, k, -1.0, A.data_ptr(), m, B.data_ptr(), k, 1.0,
                   C.data_ptr(), m, s)
            e1.record()
            e1.synchronize()
            assert st == 0, fg.last_error()
            if rep:
                times.append(e0.elapsed_time(e1))
        ms = sum(times) / len(times)
        print(json.dumps({"only": "tc_gemm", "shape": [m, n, k], "precision": "bf16", "ms": ms,
                          "tflops": 2.0 * m * n * k / (ms * 1e-3) / 1e12,
                          "c_traffic_gbs": 8.0 * m * n / (ms * 1e-3) / 1e9}))
    elif args.only == "tc_kinds":
        print(json.dumps(tc_kinds_subbench(torch, fg, dev)))
    elif args.only == "batched":
        uni = tuple(int(v) for v in args.batch_uniform.split(",")) if args.batch_uniform else None
        out = batched_subbench(torch, fg, dev, count=args.batch_count, reps=1, loop_sample=50,
                               uniform=uni)
        print(json.dumps(out))
    elif args.only == "blas3":
        print(json.dumps(blas3_subbench(torch, fg, dev)))
    elif args.only == "cholesky":
        print(json.dumps(cholesky_subbench(torch, fg, dev, n=args.n, reps=args.steps)))
    elif args.only == "inverse":
        print(json.dumps(inverse_subbench(torch, fg, dev, n=args.n, reps=args.steps)))
    elif args.only == "split":
        out = split_subbench(torch, fg, dev, n=args.split_n, Es=(args.split_e,), reps=args.steps,
                             ref_slices=args.split_ref_slices)
        print(json.dumps(out))
    else:
        cases = set(args.mixed_cases.split(",")) if args.mixed_cases else None
        print(json.dumps(mixed_subbench(torch, fg, dev, n=args.mixed_n, reps=1, cases=cases,
                                        gen=args.mixed_gen)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--quick", action="store_true", help="skip peak and sub-benchmarks")
    ap.add_argument("--unshifted", action="store_true",
                    help="profiling only: omit the n/4 diagonal shift so that the LU interchanges rows "
                         "(the benchmark workload's pivots are the identity)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-e2e-clocks", dest="e2e_clocks", action="store_false",
                    help="no nvidia-smi sampling during the e2e leg")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--mixed-n", type=int, default=16384)
    ap.add_argument("--mixed-gen", choices=["svd", "uniform"], default="svd",
                    help="--only mixed input: U diag(s) V^T (default) or unshifted uniform (profiling)")
    ap.add_argument("--mixed-cases", default=None,
                    help="comma-separated factor precisions for --only mixed (e.g. bf16,fp8)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-split", action="store_true")
    ap.add_argument("--no-cholesky", action="store_true")
    ap.add_argument("--split-n", type=int, default=8192, help="n for --only split")
    ap.add_argument("--split-e", type=int, default=48, help="exponent range E for --only split")
    ap.add_argument("--split-ref-slices", type=int, default=14, help="reference slices for --only split")
    ap.add_argument("--batch-count", type=int, default=20000)
    ap.add_argument("--batch-uniform", default=None,
                    help="N,K: --only batched on count matrices of one size (for profiling)")
    ap.add_argument("--only", choices=["tc_gemm", "tc_kinds", "batched", "mixed", "split", "cholesky",
                                       "inverse", "blas3"],
                    help="run one sub-benchmark and print its JSON (for profiling)")
    ap.add_argument("--tc-shape", default="8192,8192,256", help="M,N,K for --only tc_gemm")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.only:
        only(args)
        return
    if args.impl == "reference":
        reference_arm(args, rank)
    else:
        our_arm(args, rank, world)


if __name__ == "__main__":
    main()
