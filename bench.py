"""Benchmark: exp(tA)v solves/s on the heat-equation workload (one GB300).

Workload (default): A = 2D Dirichlet Laplacian / h^2 on a 2048 x 2048 grid
(h = 1/2049, n = 4,194,304, nnz = 20,963,328, CSR int32/f64), v ~ U[0,1]
(seed 1), t = 1e-5, m = 30, tol = 1e-6, run to convergence. Synthetic,
seeded; the reference publishes no dataset for it.

A step is one full solve y = exp(tA)v. `value` is solves/s of the chosen
form (mixed precision when its result is within 1e-6 relative 2-norm error
of the FP64 path on this workload, else FP64) with v and y resident in HBM;
`e2e` is the same metric through the host-buffer C ABI call (mexk_expmv:
H2D of v and D2H of y inside the timed region). The basis (>= 520 MB) and
CSR (251 MB) exceed the 129 MB L2, so no extra flush runs between steps.

    python bench.py [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "matrix-exp-krylov_gb300"))

METRIC = "exp(tA)v solves/s at <=1e-6 rel err, chosen vs plain FP64 (1 GB300); SpMV HBM GB/s"
WORKLOAD = ("heat2048: A = 2D Dirichlet Laplacian / h^2 on a 2048^2 grid (h=1/2049), n=4194304, "
            "nnz=20963328, CSR int32/f64; v ~ U[0,1] seed 1; t=1e-5, m=30, tol=1e-6, max_restarts=0")
HEAT_GOLDEN = os.path.join(ROOT, "tests", "golden", "heat2048_reference.npz")


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples every 20 ms (clocks, power, throttle reasons),
    started before the timed region and waited on until its first sample;
    summary() keeps the samples whose timestamps fall inside the region
    marked by begin()/end() (all samples when none do)."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.file = None
        self.t_begin = self.t_end = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        deadline = time.time() + 5.0  # the first sample, so the timed region is covered
        while time.time() < deadline and self.proc.poll() is None:
            if os.path.getsize(self.file.name) > 0:
                break
            time.sleep(0.01)
        return self

    def begin(self):
        self.t_begin = time.time()

    def end(self):
        self.t_end = time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 10:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}

        def stamp(x):
            try:
                return datetime.datetime.strptime(x, "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                return None

        inside = [r for r in rows if self.t_begin is not None and self.t_end is not None and
                  stamp(r[0]) is not None and self.t_begin <= stamp(r[0]) <= self.t_end + 0.02]
        in_region = len(inside)
        if inside:
            rows = inside
        rows = [r[1:] for r in rows]

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "samples_in_timed_region": in_region}


# ------------------------------------------------------------------ bytes model
# DRAM bytes (read + written) of one spmv_stream_kernel<float, float> launch
# as ncu counted them on the 1536^2 heat grid (nnz = 11,790,336, n = 2,359,296):
# 89.87 MB read + 3.00 MB written (16-bit column offsets; the rest of y is
# still in L2 when the kernel ends). The same stencil's traffic grows with
# its nonzeros.
SPMV_F32_TRAFFIC_HEAT1536 = (89.869312e6 + 3.002624e6, 11790336)
# The same for the SpMV that also accumulates a step's dot products
# (spmv_stream_kernel<float, float, 1, 1>): 99.40 MB read (u_{j-1} too) +
# 3.27 MB written.
SPMV_DOTS_F32_TRAFFIC_HEAT1536 = (99.39968e6 + 3.26912e6, 11790336)
# ncu dram__bytes_read.sum + dram__bytes_write.sum of the row-pattern SpMV
# with dots on the 1536^2 heat grid (2,359,296 rows): (bytes, rows).
PAT_DOTS_F32_TRAFFIC_HEAT1536 = (11.843968e6, 2359296)

def kernel_bytes(kind, n, nnz, k, fp32, window=0, form="staged"):
    """Algorithmic HBM bytes of one launch (per-kernel minimum traffic); with a
    short-recurrence window the sweeps touch only the last `window` columns.
    The SpMV's matrix stream depends on its form: CSR (values, int32 columns,
    row pointers) or the row-pattern form (one id byte per row)."""
    s = 4 if fp32 else 8
    if window and kind in ("gram_dot", "gram_update"):
        k = min(k, window)
    if form == "pattern" and kind == "spmv":
        return n + 2 * n * s  # row ids, x once, y
    if form == "pattern" and kind == "spmv_dots":  # a window of 2 takes u_{j-1}.w from the update: no u_{j-1}
        return n + (2 if window == 2 else 3) * n * s
    if kind == "lanczos_cycle":
        # steps 1..k-1 of a window-2 basis in one launch: the row ids once, and
        # per step u_j (gathered once), u_{j-1} read and u_{j+1} written; w stays
        # on chip
        return n + (k - 1) * 3 * n * s
    if kind == "spmv":
        return nnz * (s + 4) + 4 * (n + 1) + 2 * n * s  # values+cols, row_ptr, x once, y
    if kind == "spmv_dots":  # the SpMV, then u_{j-1} read for the dots (u_j is x)
        return nnz * (s + 4) + 4 * (n + 1) + 3 * n * s
    if kind in ("gs_dot", "gram_dot"):
        return k * n * s + n * s  # V_k, w
    if kind in ("gs_upd_dot", "gs_upd_norm", "gram_update"):
        return k * n * s + 2 * n * s  # V_k, w read; w (or the next column) written
    if kind == "normalize":
        return 2 * n * s
    if kind == "gram_norm":
        return n * s
    if kind == "lift":
        return k * n * s + 8 * n
    return 0


def cgs2_step_bytes(n, k, fp32):
    """Bytes of one CGS2 Gram-Schmidt step as the hot-path scope counts them:
    two passes, each reading V_k twice and w twice and writing w once."""
    s = 4 if fp32 else 8
    return 2 * (2 * k * n * s + 3 * n * s)


STEP_KINDS = {"fp64": ["spmv", "gs_dot", "gs_upd_dot", "gs_upd_norm", "normalize"],
              "mixed": ["spmv", "gram_dot", "gram_update"]}


def step_kinds(precision, j, window=0, dots_in_spmv=True, fused=False):
    """Kernels of Arnoldi step j as a solve runs them: in mixed precision with
    the staged or the pattern SpMV a step j >= 1 over two columns (every step
    of a window of 2, step 1 of full Arnoldi) takes its dot products from the
    SpMV (spmv_dots) and needs no dot sweep; with the fused Lanczos form
    (window 2) steps 1..m-1 are one launch, counted at step 1."""
    if fused and precision == "mixed" and window == 2 and j >= 1:
        return ["lanczos_cycle"] if j == 1 else []
    if precision == "mixed" and dots_in_spmv:
        lo = max(0, j + 1 - window) if window else 0
        if j >= 1 and j + 1 - lo <= 2:
            return ["spmv_dots", "gram_update"]
    return STEP_KINDS[precision]


CYCLE_KINDS = {"fp64": ["controller", "lift"], "mixed": ["controller", "lift", "gram_norm"]}


def size_matched_copy(nbytes, stream, iters=20):
    """A plain device copy moving the same bytes as one launch of a kernel
    (half read, half written; torch's copy kernel), timed back to back with
    CUDA events: what a launch of that size reaches on this GPU, for reading
    the roofline fraction of a kernel whose launches are short."""
    import torch

    half = max(1, int(nbytes) // 8)  # floats per buffer
    with torch.cuda.stream(stream):  # the copies and the events on one stream
        a = torch.empty(half, dtype=torch.float32, device="cuda")
        b = torch.empty_like(a)
        a.fill_(1.0)
        for _ in range(3):
            b.copy_(a)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(iters):
            b.copy_(a)
        e1.record(stream)
    torch.cuda.synchronize()
    us = 1e3 * e0.elapsed_time(e1) / iters
    moved = 8 * half
    return {"bytes": moved, "us": round(us, 2), "gbs": round(moved / (us / 1e6) / 1e9, 1)}


def lanczos_fused(ctx, precision, window):
    return precision == "mixed" and window == 2 and ctx.lanczos_form() == "fused"


def profile_cycle(ctx, m, n, nnz, precision, iters=8, window=0):
    """CUDA-event timing of every kernel kind of one Krylov cycle (the sweeps
    as the context's last solve ran them: with its window, if any; a fused
    Lanczos basis as its one launch for steps 1..m-1), each kind and step
    as `iters` back-to-back launches after one untimed (a solve's steps
    follow one another the same way; two launches read about 15 % high)."""
    fp32 = precision == "mixed"
    once = CYCLE_KINDS[precision]
    form = ctx.spmv_form(precision)
    dots_in_spmv = form != "direct"
    fused = lanczos_fused(ctx, precision, window)
    per = {}

    def add(kind, j, k):
        if kind == "lanczos_cycle":  # steps 1..m-1: basis size m
            j, k = m - 1, m
        ms = ctx.profile_kernel(kind, j, iters, precision)
        p = per.setdefault(kind, {"ms": 0.0, "bytes": 0.0, "launches": 0})
        p["ms"] += ms
        p["bytes"] += kernel_bytes(kind, n, nnz, k, fp32, window, form)
        p["launches"] += 1

    # The controller first: it runs on the Hessenberg matrix the last solve left.
    for kind in once:
        add(kind, m - 1, m)
    for j in range(m):
        for kind in step_kinds(precision, j, window, dots_in_spmv, fused):
            add(kind, j, j + 1)
    return per


def launches_per_solve(ctx, precision, res, m, window=0):
    """Kernels one solve launches: the start vector (2), then per cycle its
    steps (SpMV + sweeps, step_kinds) and the cycle's controller, lift and
    restart (+ the mixed form's last-column norm). Cycle sizes come from the
    attempt log."""
    sizes = [int(s[3]) for s in ctx.steps()]
    if len(sizes) != res["cycles"]:  # rejects reuse their cycle's basis
        sizes = [m] * res["cycles"]
    per_cycle = 4 if precision == "mixed" else 3
    dots_in_spmv = ctx.spmv_form(precision) != "direct"
    fused = lanczos_fused(ctx, precision, window)
    return 2 + sum(sum(len(step_kinds(precision, j, window, dots_in_spmv, fused)) for j in range(k)) + per_cycle
                   for k in sizes)


def gs_cgs2_equivalent(per, n, m, precision):
    """Gram-Schmidt of one cycle against the CGS2 byte count: all GS kernel
    time of the cycle over sum_j cgs2_step_bytes."""
    fp32 = precision == "mixed"
    gs = [k for k in per if k.startswith("gs_") or k.startswith("gram_") or k == "normalize"]
    ms = sum(per[k]["ms"] for k in gs)
    b = sum(cgs2_step_bytes(n, j + 1, fp32) for j in range(m))
    return {"ms_per_cycle": round(ms, 4), "cgs2_bytes": b, "gbs": round(b / (ms / 1e3) / 1e9, 1),
            "moved_bytes": sum(per[k]["bytes"] for k in gs)}


# ------------------------------------------------------------------ CPU baseline
def cpu_cycle_seconds(A, v, t, m, cycles=1):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    if not os.path.exists(O.LIB_PATH):
        O.build(with_reference=False)
    t0 = time.perf_counter()
    O.expmv(A, v, t, m, max_cycles=cycles)
    return (time.perf_counter() - t0) / cycles


def whole_solve_check(N=1024):
    """The cycle x attempts model of the CPU baseline checked against a whole
    solve: the oracle port (bit-identical to main_cpu.cpp) solves the heat
    workload on an N^2 grid to convergence on one core, and the same
    problem's first cycle is timed alone. Returns the wall times, the
    attempts and measured / (cycle x attempts)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from mexk import synthetic as S

    if not os.path.exists(O.LIB_PATH):
        O.build(with_reference=False)
    P = S.config1(N=N)
    t0 = time.perf_counter()
    _, st, steps = O.expmv(P.A, P.v, P.t, P.m)
    whole = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.expmv(P.A, P.v, P.t, P.m, max_cycles=1)
    cycle = time.perf_counter() - t0
    out = {"grid": f"{N}^2", "n": P.A.n, "whole_solve_s": round(whole, 3), "cycle_s": round(cycle, 3),
           "attempts": len(steps), "converged": st["converged"],
           "measured_over_model": round(whole / (cycle * len(steps)), 3)}
    if os.path.exists(HEAT_GOLDEN):
        # the reference's own compiled main_cpu.cpp, full 2048^2 solve, one core of the x86 build machine
        out["reference_binary_heat2048_whole_solve_s"] = round(float(np.load(HEAT_GOLDEN)["wall_seconds"]), 1)
    return out


def reference_attempts():
    """Basis builds per solve of the reference: one per [STEP] attempt (it
    rebuilds the basis on every reject), from its own full-size run."""
    if os.path.exists(HEAT_GOLDEN):
        d = np.load(HEAT_GOLDEN)
        return int(len(d["step_lines"])), "reference run (tests/golden/heat2048_reference.npz)"
    return None, None


# ------------------------------------------------------------------ arms
def make_problem():
    from mexk import synthetic as S

    return S.config1()


def _reference_worker(_):
    """One Arnoldi cycle of the reference's CPU algorithm on its own copy of
    the workload (a spawned process: one host core)."""
    P = make_problem()
    return cpu_cycle_seconds(P.A, P.v, P.t, P.m, 1)


def run_reference(args, rank, world):
    """The reference's CPU implementation (the oracle port, bit-identical to
    main_cpu.cpp; single-threaded by construction) on all host cores: one
    independent solve per core, each timed for one Arnoldi cycle, aggregate
    solves/s = cores / (slowest cycle time x basis builds per solve)."""
    import multiprocessing as mp

    if rank != 0:
        return
    attempts, src = reference_attempts()
    if attempts is None:
        attempts = 1
        src = "unknown: one basis build counted as one solve"
    cores = max(1, os.cpu_count() or 1)
    walls = []
    for _ in range(max(1, args.steps)):
        with mp.get_context("spawn").Pool(cores) as pool:
            walls.append(max(pool.map(_reference_worker, range(cores))))
    t_cycle = statistics.median(walls)
    value = cores / (t_cycle * attempts)
    check = whole_solve_check()
    sample = (f"{len(walls)} x {cores} concurrent single-threaded solves (one per host core), each timed for "
              f"one Arnoldi cycle (m=30, n=4194304) of the reference's CPU algorithm (oracle port, bit-identical "
              f"to main_cpu.cpp); slowest cycle {t_cycle:.2f}s (median over rounds); a solve = {attempts} basis "
              f"builds ({src}). Model check on one core: a whole {check['grid']} heat solve took "
              f"{check['whole_solve_s']}s against {check['cycle_s']}s x {check['attempts']} attempts "
              f"(measured/model {check['measured_over_model']})")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_cycle * attempts * 1e3 / cores,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": f"reference CPU (FP64), {cores} concurrent solves"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample,
                             "whole_solve_check": check},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    from mexk import synthetic as S  # noqa: F401
    from mexk.api import Context

    torch.cuda.set_device(local_rank)
    P = make_problem()
    n, nnz, m = P.A.n, P.A.nnz, P.m
    # room for the Krylov dimensions the learned controller may choose (<= 60)
    ctx = Context(P.A, m_alloc=60, device=local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    v_d = torch.from_numpy(P.v).cuda()
    y64 = torch.zeros(n, dtype=torch.float64, device="cuda")
    y32 = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    # Plain FP64 with the reference's controller is the denominator; the
    # chosen form is the fastest candidate within 1e-6 of it.
    res64 = ctx.expmv_device(v_d.data_ptr(), y64.data_ptr(), P.t, m, precision="fp64")
    steps64 = ctx.steps()
    # (precision, controller, window): window 2 = Lanczos' short recurrence,
    # which the library accepts only for a symmetric matrix (refusals skipped).
    candidates = [("mixed", "search", 2), ("mixed", "learned", 2), ("mixed", "learned", 0), ("mixed", "search", 0),
                  ("mixed", "reference", 0), ("fp64", "search", 0), ("fp64", "reference", 2), ("fp64", "search", 2)]
    if args.precision != "auto":
        candidates = [(args.precision, args.controller, args.window)]
    checked = []
    from mexk._lib import MexkError
    for prec, ctrl, win in candidates:
        try:
            r = ctx.expmv_device(v_d.data_ptr(), y32.data_ptr(), P.t, m, precision=prec, controller=ctrl,
                                 window=win)
        except MexkError as exc:
            print(f"skipping {prec}+{ctrl}+w{win}: {exc}", file=sys.stderr)
            continue
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.expmv_device(v_d.data_ptr(), y32.data_ptr(), P.t, m, precision=prec, controller=ctrl, window=win)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        e = float(torch.linalg.norm(y32 - y64) / torch.linalg.norm(y64))
        checked.append({"precision": prec, "controller": ctrl, "window": win, "rel_err_vs_fp64": e,
                        "cycles": r["cycles"], "attempts": r["attempts"], "solve_ms": round(secs * 1e3, 2),
                        "steps": ctx.steps()})
    ok = [c for c in checked if c["rel_err_vs_fp64"] <= 1e-6] or [{"precision": "fp64", "controller": "reference",
                                                                  "window": 0, "rel_err_vs_fp64": 0.0,
                                                                  "cycles": res64["cycles"],
                                                                  "attempts": res64["attempts"], "solve_ms": 0.0,
                                                                  "steps": steps64}]
    chosen = min(ok, key=lambda c: c["solve_ms"])  # fastest single solve
    form, ctrl_form, rel_err = chosen["precision"], chosen["controller"], chosen["rel_err_vs_fp64"]
    win_form = chosen["window"]
    steps32 = chosen["steps"]

    def timed(precision, K, W, controller="reference", window=0):
        out = torch.zeros(n, dtype=torch.float64, device="cuda")
        res = None
        for _ in range(W):
            res = ctx.expmv_device(v_d.data_ptr(), out.data_ptr(), P.t, m, precision=precision, controller=controller,
                                   window=window)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        launches = 0
        with ClockSampler(local_rank) as clk:
            clk.begin()
            e0.record(stream)
            for _ in range(K):
                res = ctx.expmv_device(v_d.data_ptr(), out.data_ptr(), P.t, m, precision=precision,
                                       controller=controller, window=window)
                launches += launches_per_solve(ctx, precision, res, m, window)
            e1.record(stream)
            torch.cuda.synchronize()
            clk.end()
        ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            torch.distributed.barrier()
            ms = float(t.item())
        return ms, res, launches, clk.summary()

    ms_c, res_c, launches, clocks = timed(form, args.steps, args.warmup, ctrl_form, win_form)
    value = world * args.steps / (ms_c / 1e3)
    same = form == "fp64" and ctrl_form == "reference" and not win_form
    ms64, _, _, _ = timed("fp64", max(1, args.steps), 1) if not same else (ms_c, None, None, None)
    fp64_sps = world * max(1, args.steps) / (ms64 / 1e3)
    # the chosen form with the CSR SpMV (staged), for matrices the row-pattern form does not fit
    csr_sps = None
    if ctx.spmv_form(form) == "pattern":
        ctx.set_spmv_form("staged", form)
        ms_s, _, _, _ = timed(form, max(1, args.steps), 1, ctrl_form, win_form)
        csr_sps = world * max(1, args.steps) / (ms_s / 1e3)
        ctx.set_spmv_form("pattern", form)
        timed(form, 1, 1, ctrl_form, win_form)  # the pattern form's graphs again

    # e2e: host buffers through mexk_expmv (H2D v, solve, D2H y each step)
    v_pin = torch.from_numpy(P.v).pin_memory()
    y_pin = torch.zeros(n, dtype=torch.float64).pin_memory()
    import ctypes as C

    from mexk._lib import Result, check, lib
    from mexk.api import params as mkparams

    pr = mkparams(m, P.t, precision=form, controller=ctrl_form, window=win_form)
    r = Result()
    vp = C.cast(v_pin.data_ptr(), C.POINTER(C.c_double))
    yp = C.cast(y_pin.data_ptr(), C.POINTER(C.c_double))
    check(lib().mexk_expmv(ctx.handle, C.byref(pr), vp, yp, C.byref(r)), "mexk_expmv")
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        check(lib().mexk_expmv(ctx.handle, C.byref(pr), vp, yp, C.byref(r)), "mexk_expmv")
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * args.steps / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": 8 * n,
           "d2h_bytes_per_step": 8 * n}

    # kernel roofline from live CUDA-event timings of each kernel kind
    peak, peak_kind = measured_peaks()
    per = profile_cycle(ctx, m, n, nnz, form, window=win_form)
    tot_ms = sum(p["ms"] for p in per.values())
    dom = max(per, key=lambda k: per[k]["ms"])
    ach = per[dom]["bytes"] / (per[dom]["ms"] / 1e3) / 1e9
    traffic, tsrc = None, None
    if dom == "spmv_dots" and form != "fp64" and ctx.spmv_form(form) == "pattern":
        mb, rows = PAT_DOTS_F32_TRAFFIC_HEAT1536
        traffic = mb * n / rows
        tsrc = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the row-pattern spmv_dots kernel on the "
                "1536^2 heat grid (2,359,296 rows), scaled by rows")
    elif dom in ("spmv", "spmv_dots") and form != "fp64" and ctx.spmv_form(form) == "staged":
        mb, nz = SPMV_DOTS_F32_TRAFFIC_HEAT1536 if dom == "spmv_dots" else SPMV_F32_TRAFFIC_HEAT1536
        traffic = mb * nnz / nz
        tsrc = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of the {dom} kernel on the "
                "1536^2 heat grid (11,790,336 nonzeros), scaled by nonzeros")
    roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
            "traffic": traffic, "traffic_source": tsrc,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "size_matched_copy": size_matched_copy(per[dom]["bytes"] / per[dom]["launches"], stream)}
    sp = per["spmv"]
    spmv_gbs = sp["bytes"] / (sp["ms"] / 1e3) / 1e9
    if form != "fp64":
        ctx.expmv_device(v_d.data_ptr(), y64.data_ptr(), P.t, m, precision="fp64")
        per64 = profile_cycle(ctx, m, n, nnz, "fp64")
    else:
        per64 = per
    sp64 = per64["spmv"]

    cpu = None
    if rank == 0 and not args.no_cpu:
        attempts, src = reference_attempts()
        if attempts is None:
            attempts, src = len(steps64), "this run's FP64 decision sequence"
        t_cycle = cpu_cycle_seconds(P.A, P.v, P.t, m, 1)
        check = whole_solve_check()
        cpu = {"value": 1.0 / (t_cycle * attempts), "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": (f"one Arnoldi cycle (m=30, n=4194304) of the oracle port of main_cpu.cpp on 1 core "
                          f"took {t_cycle:.2f}s; a reference solve = {attempts} basis builds ({src}); "
                          f"model check: a whole {check['grid']} heat solve took {check['whole_solve_s']}s against "
                          f"{check['cycle_s']}s x {check['attempts']} attempts (measured/model "
                          f"{check['measured_over_model']})"),
               "whole_solve_check": check}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_c / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if form == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "form": f"{form} + {ctrl_form} controller" + (f" + window {win_form}" if win_form else ""),
                       "spmv_form": ctx.spmv_form(form),
                       "parallelism": f"replicas x{world}",
                       "l2": ("inputs larger than L2 (basis >= 520 MB; CSR 251 MB, of which the row-pattern "
                              "SpMV reads 4.2 MB of row ids); no flush")},
            "fp64_solves_per_s": fp64_sps, "chosen_rel_err_vs_fp64": rel_err,
            "chosen_form_csr_spmv_solves_per_s": csr_sps,
            "solve": {"attempts": res_c["attempts"], "cycles": res_c["cycles"],
                      "restarts_done": res_c["restarts_done"], "converged": res_c["converged"],
                      "fp64_attempts": res64["attempts"], "fp64_cycles": res64["cycles"]},
            "forms_checked": [{k: v for k, v in c.items() if k != "steps"} for c in checked],
            "spmv": {"gbs": spmv_gbs, "frac": spmv_gbs / peak, "precision": form, "form": ctx.spmv_form(form),
                     "us": 1e3 * sp["ms"] / sp["launches"],
                     "csr_bytes_gbs": kernel_bytes("spmv", n, nnz, 1, form != "fp64") * sp["launches"]
                     / (sp["ms"] / 1e3) / 1e9,
                     "fp64_gbs": sp64["bytes"] / (sp64["ms"] / 1e3) / 1e9,
                     "fp64_us": 1e3 * sp64["ms"] / sp64["launches"]},
            "kernel_share": {k: round(p["ms"] / tot_ms, 4) for k, p in per.items()},
            "kernels": {f: {k: {"ms_per_cycle": round(p["ms"], 4),
                                "gbs": round(p["bytes"] / (p["ms"] / 1e3) / 1e9, 1) if p["bytes"] else None}
                            for k, p in pp.items()} for f, pp in (("chosen", per), ("fp64", per64))},
            "gram_schmidt_vs_cgs2_bytes": {"chosen": gs_cgs2_equivalent(per, n, m, form) if not win_form else None,
                                           "fp64": gs_cgs2_equivalent(per64, n, m, "fp64")},
            "trace": {"fp64": [(round(s[1], 12), float(f"{s[2]:.3g}")) for s in steps64],
                      **{f"{c['precision']}+{c['controller']}" + (f"+w{c['window']}" if c["window"] else ""):
                         [(round(s[1], 12), float(f"{s[2]:.3g}"))
                                                                 for s in c["steps"]] for c in checked}},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    ctx.close()


# ------------------------------------------------------------------ batched workload
BATCH_METRIC = "batched exp(tA)v solves/s (256 problems x 16 RHS, mixed precision) vs serial plain FP64"
BATCH_WORKLOAD = ("batch256: 256 config-0-style matrices (n log-uniform in [1e4, 2e6], degree U{5..20}, "
                  "values U[-0.5,0.5], diagonal -(row |off| sum)-1; sizes seeded 100-355), 16 N(0,1) RHS each, "
                  "t ~ U[0.1,2], m=30, tol=1e-6, reference controller per RHS; FP32 values/bases, FP64 H")


def batch_kernel_bytes(kind, rows, nnz, k):
    """Algorithmic bytes of one first-wave launch (16 RHS x FP32 = 64 B per row)."""
    if kind == "spmm":
        return nnz * 8 + 8 * rows + 2 * 64 * rows  # cols+values, row_ptr, x once, y
    if kind == "dot":
        return (k + 1) * 64 * rows
    return (k + 2) * 64 * rows  # update


def run_batch(args):
    """Batched workload: one Batch over all problems, timed runs with inputs
    resident, e2e through add/upload/run/result, a sampled serial FP64
    baseline and accuracy check, and first-wave kernel rates."""
    import torch

    from mexk import synthetic as S
    from mexk.api import Context
    from mexk.batch import Batch

    torch.cuda.set_device(0)
    nprob = args.problems
    t0 = time.perf_counter()
    probs = [S.config3_generated(i) for i in range(nprob)]
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    torch.cuda.empty_cache()
    nsolves = sum(P.v.shape[0] for P in probs)

    # e2e through the public API: add + upload + run + results (H2D and D2H inside)
    t0 = time.perf_counter()
    b = Batch(m=30, tol=1e-6, autotune=True)
    for P in probs:
        b.add(P.A, P.v, P.t)
    b.upload()
    t_up = time.perf_counter() - t0
    b.run()  # first run: autotuning + graph capture
    ys = [b.result(i) for i in range(nprob)]
    t_e2e = time.perf_counter() - t0
    info = b.info()
    h2d = sum(P.A.nnz * 12 + (P.A.n + 1) * 4 + P.v.size * 8 for P in probs)
    d2h = sum(P.v.size * 8 for P in probs)

    for _ in range(max(0, args.warmup - 1)):
        b.run()
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        clk.begin()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            b.run()
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        clk.end()
    clocks = clk.summary()
    value = nsolves * args.steps / secs
    cycles = info["cycles"]
    info = b.info()
    ys = [b.result(i) for i in range(nprob)]

    # first-wave kernel rates at a mid step
    kern = {}
    for kind, j in (("spmm", 0), ("dot", 14), ("update", 14)):
        ms, rows, nnz = b.profile(kind, j, 5)
        kern[kind] = {"j": j, "ms": round(ms, 4),
                      "gbs": round(batch_kernel_bytes(kind, rows, nnz, j + 1) / (ms / 1e3) / 1e9, 1)}
    b.close()

    # serial plain FP64 on a size-stratified subset (every RHS of args.sample
    # problems): measured solve by solve, and the same subset as one batch
    order = np.argsort([P.A.n for P in probs])
    sample = sorted(set(int(order[int(i)]) for i in np.linspace(0, nprob - 1, min(args.sample, nprob)).round()))
    pts, worst, serial_s = [], 0.0, 0.0
    for i in sample:
        P = probs[i]
        with Context(P.A, m_alloc=30) as ctx:
            ctx.expmv(P.v[0], P.t, 30, precision="fp64")  # graph capture
            for r in range(P.v.shape[0]):
                ts = time.perf_counter()
                y64, _ = ctx.expmv(P.v[r], P.t, 30, precision="fp64")
                dt = time.perf_counter() - ts
                serial_s += dt
                pts.append((P.A.n, dt))
                err = np.linalg.norm(ys[i][0][r] - y64) / max(np.linalg.norm(y64), 1e-300)
                worst = max(worst, err)
    sub_solves = len(pts)
    with Batch(m=30, tol=1e-6, autotune=True) as bs:
        for i in sample:
            bs.add(probs[i].A, probs[i].v, probs[i].t)
        bs.upload()
        bs.run()  # autotune and graph capture
        torch.cuda.synchronize()
        ts = time.perf_counter()
        for _ in range(3):
            bs.run()
        torch.cuda.synchronize()
        batch_sub_s = (time.perf_counter() - ts) / 3
    nn = np.array([p[0] for p in pts], float)
    tt = np.array([p[1] for p in pts], float)
    slope, icept = np.polyfit(nn, tt, 1)
    icept = max(icept, 0.0)
    est = sum(P.v.shape[0] * max(icept + slope * P.A.n, 0.0) for P in probs)
    serial_sps = nsolves / est

    peak, peak_kind = measured_peaks()
    dom = max(kern, key=lambda k: kern[k]["ms"])
    line = {
        "metric": BATCH_METRIC, "value": value, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD, "problems": nprob, "solves_per_step": nsolves,
                   "rows_padded": info["rows"], "nnz": info["nnz"], "waves": info["waves"],
                   "schedule": {"tile_rows": info["tile_rows"], "dot_columns": info["dot_columns"],
                                "spmm_unroll": info["spmm_unroll"], "tune_ms": round(info["tune_ms"], 1)},
                   "cycles_per_step": cycles, "generator": "torch Philox on the GPU, seeds 100+i",
                   "l2": "inputs far larger than L2 (bases > 100 GB); no flush"},
        "serial_fp64": {"measured_subset": {"problems": len(sample), "solves": sub_solves,
                                            "serial_s": round(serial_s, 3), "batch_s": round(batch_sub_s, 4),
                                            "serial_solves_per_s": sub_solves / serial_s,
                                            "batch_solves_per_s": sub_solves / batch_sub_s,
                                            "speedup": serial_s / batch_sub_s},
                        "extrapolated_all": {"solves_per_s": serial_sps, "speedup": value / serial_sps,
                                             "how": f"time per serial solve fitted as a + b*n on the subset and "
                                                    f"summed over all {nsolves} solves"},
                        "sample": f"every RHS of {len(sample)} size-stratified problems ({sub_solves} plain-FP64 "
                                  f"solves, each timed), and the same problems as one batch"},
        "max_rel_err_vs_fp64_sample": worst,
        "setup": {"generate_s": round(t_gen, 2), "upload_s": round(t_up, 2)},
        "kernels_first_wave": kern,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": kern[dom]["gbs"], "peak": peak, "unit": "GB/s",
                     "frac": kern[dom]["gbs"] / peak, "traffic": None, "peak_source": peak_kind},
        "e2e": {"value": nsolves / t_e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "note": "add + upload + first run (autotune, graph capture) + results"},
        "cpu_baseline": None, "clocks": clocks,
        # per wave cycle: m x (SpMM, dot, update) + last norm, controller, lift, restart, status
        "gpu_launches": info["cycles"] * (3 * 30 + 5) * args.steps // max(1, args.steps),
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ learned-controller workload
CONV_METRIC = ("exp(tA)v solves/s and SpMVs of the learned controller vs the plain restart heuristic "
               "(128^3 convection-diffusion, Pe 1-1000)")


def run_convdiff(args):
    """Config-4 workload: for each Peclet number, the same solve under the plain
    heuristic (FP64 and mixed), the candidate-step search and the learned
    controller (mixed); SpMVs, cycles, CUDA-event time and error vs FP64."""
    import torch

    from mexk import synthetic as S
    from mexk.api import Context
    from mexk.controller import CONVDIFF_T

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    forms = (("fp64", "reference"), ("mixed", "reference"), ("mixed", "search"), ("mixed", "learned"))
    per_pe, tot = [], {f"{p}+{c}": {"ms": 0.0, "spmv": 0, "cycles": 0} for p, c in forms}
    for pe, t in CONVDIFF_T.items():
        P = S.config4(128, pe)
        entry = {"pe": pe, "t": t, "n": P.A.n, "nnz": P.A.nnz}
        with Context(P.A, m_alloc=60) as ctx:
            v_d = torch.from_numpy(P.v).cuda()
            y64 = torch.zeros_like(v_d)
            y = torch.zeros_like(v_d)
            for prec, ctrl in forms:
                out = y64 if (prec, ctrl) == forms[0] else y
                res = ctx.expmv_device(v_d.data_ptr(), out.data_ptr(), t, 30, precision=prec, controller=ctrl)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(args.steps):
                    res = ctx.expmv_device(v_d.data_ptr(), out.data_ptr(), t, 30, precision=prec, controller=ctrl)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / args.steps
                err = float(torch.linalg.norm(out - y64) / torch.linalg.norm(y64)) if out is y else 0.0
                key = f"{prec}+{ctrl}"
                entry[key] = {"ms": round(ms, 2), "spmv": res["spmv_count"], "cycles": res["cycles"],
                              "attempts": res["attempts"], "converged": res["converged"], "rel_err_vs_fp64": err}
                tot[key]["ms"] += ms
                tot[key]["spmv"] += res["spmv_count"]
                tot[key]["cycles"] += res["cycles"]
        per_pe.append(entry)
    nprob = len(per_pe)
    learned, plain = tot["mixed+learned"], tot["mixed+reference"]
    line = {
        "metric": CONV_METRIC, "value": nprob / (learned["ms"] / 1e3), "unit": "solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": 1, "ms_per_step": learned["ms"] / nprob, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": ("convdiff128: 3D 7-point convection-diffusion, 128^3 grid, h = 1/129, upwinded "
                                "velocity (1,0.5,0.25)*Pe, Pe in {1,10,100,1000}; v ~ U[0,1] seed 4; "
                                "t per Pe = " + json.dumps(CONVDIFF_T) + "; m = 30 (learned: chosen per cycle), "
                                "tol 1e-6")},
        "learned_vs_plain_heuristic": {"solves_per_s": nprob / (learned["ms"] / 1e3),
                                       "plain_solves_per_s": nprob / (plain["ms"] / 1e3),
                                       "speedup": plain["ms"] / learned["ms"],
                                       "spmv": learned["spmv"], "plain_spmv": plain["spmv"],
                                       "spmv_ratio": plain["spmv"] / max(learned["spmv"], 1)},
        # the same candidate search without the network (the method the network centres)
        "learned_vs_search": {"search_solves_per_s": nprob / (tot["mixed+search"]["ms"] / 1e3),
                              "speedup": tot["mixed+search"]["ms"] / learned["ms"],
                              "spmv": learned["spmv"], "search_spmv": tot["mixed+search"]["spmv"],
                              "spmv_ratio": tot["mixed+search"]["spmv"] / max(learned["spmv"], 1)},
        "totals": {k: {"ms": round(v["ms"], 2), "spmv": v["spmv"], "cycles": v["cycles"]} for k, v in tot.items()},
        "per_pe": per_pe,
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ power-law workload
PL_METRIC = "exp(tA)v solves/s at <=1e-6 rel err, mixed precision vs plain FP64 (irregular power-law rows)"


def run_powerlaw(args):
    """Config-2 workload: power-law rows (Zipf 1.8, 2..2048 off-diagonals),
    n = 8,388,608, t = 0.5, m = 40; each form timed after one untimed solve,
    error vs FP64, SpMV rates from CUDA events."""
    import torch

    from mexk import synthetic as S
    from mexk.api import Context

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    P = S.config2()
    t_gen = time.perf_counter() - t0
    n, nnz = P.A.n, P.A.nnz
    forms = (("fp64", "reference"), ("mixed", "reference"), ("mixed", "search"), ("mixed", "learned"))
    out = {}
    with Context(P.A, m_alloc=P.m) as ctx:
        v_d = torch.from_numpy(P.v).cuda()
        y64 = torch.zeros_like(v_d)
        y = torch.zeros_like(v_d)
        for prec, ctrl in forms:
            dst = y64 if (prec, ctrl) == forms[0] else y
            res = ctx.expmv_device(v_d.data_ptr(), dst.data_ptr(), P.t, P.m, precision=prec, controller=ctrl)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                res = ctx.expmv_device(v_d.data_ptr(), dst.data_ptr(), P.t, P.m, precision=prec, controller=ctrl)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            err = float(torch.linalg.norm(dst - y64) / torch.linalg.norm(y64)) if dst is y else 0.0
            out[f"{prec}+{ctrl}"] = {"ms": round(ms, 2), "solves_per_s": 1e3 / ms, "rel_err_vs_fp64": err,
                                     "cycles": res["cycles"], "attempts": res["attempts"],
                                     "spmv": res["spmv_count"], "converged": res["converged"]}
        spmv = {}
        for prec in ("mixed", "fp64"):
            chosen = ctx.spmv_form(prec)
            b = kernel_bytes("spmv", n, nnz, 1, prec == "mixed")
            spmv[prec] = {"form": chosen}
            for f in ("staged", "direct"):  # both forms, then the context's own choice back
                ctx.set_spmv_form(f, prec)
                ms = min(ctx.profile_kernel("spmv", j, 5, prec) for j in (0, 10, 20))
                spmv[prec][f] = {"us": round(ms * 1e3, 1), "gbs": round(b / (ms / 1e3) / 1e9, 1)}
            ctx.set_spmv_form(chosen, prec)
            spmv[prec].update(spmv[prec][chosen])
    ok = {k: v for k, v in out.items() if k != "fp64+reference" and v["rel_err_vs_fp64"] <= 1e-6}
    best = min(ok, key=lambda k: out[k]["ms"]) if ok else "fp64+reference"
    peak, _ = measured_peaks()
    row_len = np.diff(P.A.row_ptr)
    line = {
        "metric": PL_METRIC, "value": out[best]["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": 1, "ms_per_step": out[best]["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": ("powerlaw: n = 8,388,608, seed 2, row off-diagonal counts ~ Zipf(1.8) clipped to "
                                "[2, 2048], uniform distinct columns, values U[-1,1], diagonal -(row |off| sum)-0.5; "
                                "v ~ N(0,1); t = 0.5, m = 40, tol 1e-6"),
                   "nnz": nnz, "row_len_mean": float(row_len.mean()), "row_len_max": int(row_len.max()),
                   "chosen": best, "generate_s": round(t_gen, 1)},
        "fp64_solves_per_s": out["fp64+reference"]["solves_per_s"],
        "speedup_vs_fp64": out[best]["solves_per_s"] / out["fp64+reference"]["solves_per_s"],
        "forms": out,
        "spmv": {k: dict(v, frac=round(v["gbs"] / peak, 3)) for k, v in spmv.items()},
    }
    print(json.dumps(line), flush=True)


def run_batch_once(args):
    """One untimed batch run over problems [first, first + problems) of the
    batched workload (autotuning off): the command ncu captures."""
    import torch

    from mexk import synthetic as S
    from mexk.batch import Batch

    torch.cuda.set_device(0)
    probs = [S.config3_generated(i) for i in range(args.first, args.first + args.problems)]
    with Batch(m=30, tol=1e-6, autotune=False) as b:
        for P in probs:
            b.add(P.A, P.v, P.t)
        b.upload()
        b.run()
        print(json.dumps(b.info()), flush=True)


def run_solve_once(local_rank, grid=2048, spmv_form=None, controller="learned"):
    """One solve in the headline form (mixed precision, window 2: the heat
    matrix is symmetric; the learned controller unless `controller` names
    another) and one plain FP64 solve of the heat equation on a grid x grid
    mesh, untimed: the command ncu captures. spmv_form: run that SpMV form
    instead of the context's choice (the row-pattern form on this matrix)."""
    import torch

    from mexk import synthetic as S
    from mexk.api import Context

    torch.cuda.set_device(local_rank)
    P = make_problem() if grid == 2048 else S.config1(N=grid)
    # room for the Krylov dimensions the learned controller may choose (<= 60)
    with Context(P.A, m_alloc=60, device=local_rank) as ctx:
        if spmv_form is not None:
            for prec in ("mixed", "fp64"):
                ctx.set_spmv_form(spmv_form, prec)
        for prec, ctrl, window in (("mixed", controller, 2), ("fp64", "reference", 0)):
            _, res = ctx.expmv(P.v, P.t, P.m, precision=prec, controller=ctrl, window=window)
            print(prec, ctrl, window, res, flush=True)


def run_load(args):
    """The .bincsr load path: the heat2048 matrix (u32 indices, f64 values, as
    the reference's generator writes it) and the config-2 power-law matrix
    (u32, f32 values), written to a temporary directory (so read from the
    page cache), loaded by the host loader + upload (CSRHost::from_binary_csr
    then mexk_context_upload_csr, timed by csr_tool --time) and straight into
    a context (mexk_context_load_bincsr). Best of `steps` loads each."""
    import shutil
    import subprocess
    import tempfile

    from mexk import bincsr as B
    from mexk import synthetic as S
    from mexk._lib import BUILD
    from mexk.api import Context

    tool = os.path.join(BUILD, "csr_tool")
    tmp = tempfile.mkdtemp(prefix="mexk_load_")
    out = {}
    try:
        for name, make, idt, vdt in (("heat2048", lambda: S.laplacian_2d(2048), "u32", "f64"),
                                     ("powerlaw_cfg2", lambda: S.config2().A, "u32", "f32")):
            A = make()
            path = os.path.join(tmp, name + ".bincsr")
            B.write_bincsr(path, A.row_ptr, A.col_idx, A.values, index_dtype=idt, value_dtype=vdt)
            size = os.path.getsize(path)
            del A
            host, fast, fast_inner = [], [], []
            for _ in range(max(1, args.steps)):
                r = subprocess.run([tool, path, "--time"], capture_output=True, text=True, check=True)
                kv = dict(x.split("=") for x in r.stdout.split() if "=" in x)
                host.append((float(kv["host_load_s"]), float(kv["upload_s"])))
                t0 = time.perf_counter()
                with Context.from_bincsr(path, m_alloc=30) as ctx:
                    fast_inner.append(ctx.load_info["seconds"])
                fast.append(time.perf_counter() - t0)
            h = min(host, key=lambda x: x[0] + x[1])
            out[name] = {"file_bytes": size, "index_dtype": idt, "value_dtype": vdt,
                         "host_loader_s": round(h[0], 4), "host_upload_s": round(h[1], 4),
                         "host_total_s": round(h[0] + h[1], 4),
                         "direct_s": round(min(fast_inner), 4), "direct_with_context_s": round(min(fast), 4),
                         "direct_gbs": round(size / min(fast_inner) / 1e9, 2),
                         "speedup": round((h[0] + h[1]) / min(fast_inner), 1)}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    h = out["heat2048"]
    print(json.dumps({"metric": "bincsr load GB/s (file bytes / wall s, page-cache resident)",
                      "value": h["direct_gbs"], "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
                      "higher_is_better": True, "data": "synthetic", "config": {"workload": "load"},
                      "files": out, "host_cores": os.cpu_count()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--controller", default="search", choices=["reference", "search", "learned"])
    ap.add_argument("--window", type=int, default=0, help="with --precision: short-recurrence window (0 = Arnoldi)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--solve-once", action="store_true", help="one untimed FP64 + mixed solve (for ncu)")
    ap.add_argument("--workload", default="heat2048",
                    choices=["heat2048", "batch", "convdiff", "powerlaw", "load"])
    ap.add_argument("--problems", type=int, default=256, help="batch workload: number of problems")
    ap.add_argument("--sample", type=int, default=16,
                    help="batch workload: problems (all their RHS) in the measured serial FP64 subset")
    ap.add_argument("--grid", type=int, default=2048, help="--solve-once: heat-equation grid size")
    ap.add_argument("--spmv-form", choices=["staged", "direct", "pattern"], default=None,
                    help="--solve-once: SpMV form to run instead of the context's choice")
    ap.add_argument("--first", type=int, default=0, help="batch --solve-once: index of the first problem")
    args = ap.parse_args()
    if args.solve_once and args.workload == "batch":
        run_batch_once(args)
        return
    if args.solve_once:
        run_solve_once(int(os.environ.get("LOCAL_RANK", "0")), args.grid, args.spmv_form,
                       args.controller if args.precision != "auto" else "learned")
        return
    if args.workload == "batch" and args.impl == "ours":
        run_batch(args)
        return
    if args.workload == "convdiff" and args.impl == "ours":
        run_convdiff(args)
        return
    if args.workload == "powerlaw" and args.impl == "ours":
        run_powerlaw(args)
        return
    if args.workload == "load" and args.impl == "ours":
        run_load(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
