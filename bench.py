"""Benchmark of the H*X hot path on GB300.

One step = one FP64 H*X application (MYHX, TA1) to a block of 16 vectors on
the 96 x 96 x 64 Jacobi-DVR grid (589,824 points) -- the "bare FP64 H*X on 1
and 16 vectors" of the plain-FP64 GPU workload.  Inputs are seeded N(0,1)
vectors already resident in HBM; two input/output sets (2 x 151 MB, larger
than the 129 MB L2) alternate between steps.  `e2e` repeats the measurement
through the host-buffer C ABI (scalit_hx), host<->device copies included.

The PIST leg (default: the 200 lowest levels of the 160 x 160 x 120 problem,
3,072,000 points) times preconditioner build + PIST to convergence + the FP64
residual check twice: FP64 inner solves, and the mixed path (FP32 inner solves,
FP32 first Gram-Schmidt pass), and reports every level's difference.

N > 1 (torchrun): replicas -- every rank runs the same workload on its own GPU,
no collective on the data path; value = all ranks' applications / slowest rank.

--impl reference: the oracle's FP64 restatement of the reference's serial
MYHX (C, OpenMP over all host cores), timed on a bounded sample of the same
workload; rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "H*X apps/s & %roofline; PIST time to 200 levels (mixed vs FP64 GPU)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tri-96x96x64")
    ap.add_argument("--nvec", type=int, default=16)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--pist-workload", default="tri-160x160x120",
                    help="grid of the PIST leg ('none' skips it)")
    ap.add_argument("--pist-levels", type=int, default=200)
    ap.add_argument("--pist-arms", default="fp64,fp32",
                    help="PIST arms to run: fp64 (FP64 inner solves), fp32 (mixed)")
    ap.add_argument("--pist-warmup", type=int, default=1,
                    help="untimed small-grid PIST before the timed arms (0 skips it)")
    ap.add_argument("--batch-problems", type=int, default=0,
                    help="shifted-QMR leg over this many uneven problems (0 skips it)")
    ap.add_argument("--batch-shifts", type=int, default=16)
    return ap.parse_args()


# ---------------------------------------------------------------- helpers --
def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def reduce_max(value: float, world: int) -> float:
    """Max of a per-rank float over all ranks (identity for one rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(units_per_rank: float, world: int, max_seconds: float) -> float:
    return units_per_rank * world / max_seconds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        smax = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(self.samples)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def profiled_traffic(workload, level):
    """DRAM bytes per single-vector launch of the tensor-core level kernel, from
    the committed ncu summary of this workload (None when not profiled)."""
    import re
    path = os.path.join(ROOT, "profiles", f"tc_level_kernel_{workload}.md")
    try:
        with open(path) as f:
            m = re.search(rf"traffic_per_launch_level{level}_nvec1:\s*(\d+)", f.read())
        return int(m.group(1)) if m else None
    except OSError:
        return None


def hx_units(sizes):
    """Algorithmic flops and bytes of one FP64 H*X application, and per level.

    flops: 2 N n_l per level plus the diagonal (V - E0) X and the level sums (5N).
    bytes of a level launch: read X, write Y, and read Y when accumulating
    (levels 2..sF), plus the small level matrix; DEP and V where used.
    """
    n = list(sizes)
    N = int(np.prod(n))
    w = 8
    levels = []
    for l, nl in enumerate(n):
        flops = 2.0 * N * nl
        byts = (2 + (1 if l > 0 else 0)) * N * w + nl * nl * w
        if l == 0:
            byts += N * w            # V for the fused diagonal term
            flops += 3.0 * N
        if l == len(n) - 1:
            byts += (N // nl) * w    # DEP factors c(r, R)
            flops += N
        levels.append({"flops": flops, "bytes": byts})
    total_flops = sum(x["flops"] for x in levels) + N
    total_bytes = 3 * N * w + sum(m * m for m in n) * w + (N // n[-1]) * w
    return total_flops, total_bytes, levels


# ------------------------------------------------------------- reference --
def cpu_baseline(problem, e0, seconds, nvec_cap=64):
    """The oracle's MYHX on the host cores: applications per second on a bounded sample."""
    from oracle import oracle as orc
    op = orc.Operator.from_problem(problem, E0=e0)
    x = np.random.default_rng(0).standard_normal(problem.N)
    op.hx(x, 1)
    t0 = time.perf_counter()
    op.hx(x, 1)
    one = time.perf_counter() - t0
    reps = max(1, min(nvec_cap, int(seconds / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(reps):
        op.hx(x, 1)
    dt = time.perf_counter() - t0
    return {"value": reps / dt, "unit": "H*X apps/s", "cores": orc.num_threads(), "kind": "port",
            "sample": f"{reps} FP64 H*X applications (TA1) on the {problem.sizes[0]}x"
                      f"{problem.sizes[1]}x{problem.sizes[2]} grid, oracle C restatement of MYHX "
                      f"(osb.hx.h:71-110), OpenMP over blocks"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from scalit_gb300 import hamiltonian as hm
    p = hm.workload(args.workload)
    e0 = float(p.RES.min())
    from oracle import oracle as orc
    op = orc.Operator.from_problem(p, E0=e0)
    x = np.random.default_rng(0).standard_normal(p.N)
    op.hx(x, 1)
    t0 = time.perf_counter()
    op.hx(x, 1)
    one = time.perf_counter() - t0
    # each step is a bounded sample: nvec applications, capped so the run stays short
    per_step = max(1, min(args.nvec, int(6.0 / max(one, 1e-6))))
    for _ in range(args.warmup):
        op.hx(x, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for _ in range(per_step):
            op.hx(x, 1)
    dt = time.perf_counter() - t0
    value = args.steps * per_step / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "H*X apps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "grid": list(p.sizes), "npoints": p.N,
                   "vectors_per_step": per_step, "operator": "MYHX TA1"},
        "cpu_baseline": {"value": value, "unit": "H*X apps/s", "cores": orc.num_threads(),
                         "kind": "port",
                         "sample": f"{per_step} applications per step, oracle C restatement of MYHX"},
        "e2e": {"value": value, "unit": "H*X apps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------- PIST --
def pist_leg(workload, levels, device, capi, hm, arms=("fp64", "fp32"), warmup=True):
    """Wall time from the preconditioner build to converged eigenvalues, with
    FP64 and with FP32 QMR inner solves (basis, HMAT and Ritz values in FP64)."""
    # untimed warm-up on the small grid with the same number of levels (so the
    # same Krylov sizes): the first solve of a process loads the kernels of
    # the eigensolver library for each matrix size class it meets (lazy module
    # loading, seconds in all), which would otherwise land on whichever arm
    # runs first
    pw = hm.workload("tri-24x32x20")
    for prec, orth in ((capi.PREC_FP64, 1), (capi.PREC_FP32, 2)) if warmup else ():
        with capi.Context.from_problem(pw, e0=float(pw.RES.min()), device=device) as ctx:
            ctx.build_osb(20, 1e-4)
            if prec == capi.PREC_FP32:
                ctx.set_fp32_mode(capi.FP32_TENSOR_PX)
            ctx.pist(np.random.default_rng(0).random(pw.N), levels, float(pw.RES.min()), 1e-11,
                     m_max=max(8 * levels, 400), qmr_max=2000, qmr_tol=1e-4, precision=prec, orth=orth,
                     residuals=True)
    p = hm.workload(workload)
    e0 = float(p.RES.min())
    x0 = np.random.default_rng(0).random(p.N)
    out = {"workload": workload, "levels": levels}
    eigs = {}
    # mixed leg: FP32 inner solves (H*X on the CUDA cores, the preconditioner's
    # rotations in split-BF16 x3 on the tensor cores) and an FP32 first
    # Gram-Schmidt pass (the re-orthogonalisation's projections, HMAT and the
    # Ritz solves stay FP64; its update streams the basis' FP32 copy with
    # coefficients split into two FP32 parts)
    for name, prec, orth in (("fp64", capi.PREC_FP64, 1), ("fp32", capi.PREC_FP32, 2)):
        if name not in arms:
            continue
        with capi.Context.from_problem(p, e0=e0, device=device) as ctx:
            if prec == capi.PREC_FP32:
                ctx.set_fp32_mode(capi.FP32_TENSOR_PX)
            t0 = time.perf_counter()
            stats = ctx.build_osb(20, 1e-4)
            t1 = time.perf_counter()
            build_levels = [float(v) for v in ctx.build_times()]
            st, eig, res, info = ctx.pist(x0, levels, e0, 1e-11, m_max=max(8 * levels, 400),
                                          qmr_max=2000, qmr_tol=1e-4, precision=prec, orth=orth,
                                          residuals=True)
            t2 = time.perf_counter()
        eigs[name] = eig
        out[name] = {"status": st, "orth": orth, "seconds": t2 - t0, "build_s": t1 - t0, "pist_s": t2 - t1,
                     "fp32_engine": ("H*X CUDA cores, preconditioner rotations split-BF16 x3 tensor cores"
                                     if prec == capi.PREC_FP32 else None),
                     "build_levels_s": build_levels,
                     "sweeps_per_block": [float(stats[l, 4] / int(np.prod(p.sizes[l + 1:])))
                                          for l in range(len(p.sizes))],
                     "levels_per_s": levels / (t2 - t0), "krylov": info["krylov"],
                     "qmr_iterations": info["qmr_total"], "qmr_solves": info["qmr_solves"],
                     "t_qmr": info["t_qmr"], "t_orth": info["t_orth"], "t_hmat": info["t_hmat"],
                     "t_ritz": info["t_ritz"], "t_resid": info["t_resid"],
                     "max_residual_eh": float(np.max(info["resid"]))}
    if "fp64" in eigs and "fp32" in eigs:
        out["speedup_fp32_inner"] = out["fp64"]["seconds"] / out["fp32"]["seconds"]
        out["speedup_excluding_build"] = out["fp64"]["pist_s"] / out["fp32"]["pist_s"]
        diff = np.abs(eigs["fp32"] - eigs["fp64"]) * hm.HARTREE_CM
        out["max_abs_diff_cm"] = float(diff.max())
        out["per_level_diff_cm"] = [float(f"{d:.3g}") for d in diff]
    out["lowest_eigenvalues_eh"] = [float(v) for v in next(iter(eigs.values()))[:5]] if eigs else []
    return out


def batch_leg(nprob, nrhs, device, capi, hm):
    """Uneven problems (n_R, n_r in [24, 96], n_theta in [16, 64], PES +-10%),
    each with nrhs shifts over its lowest 0.02 Eh and one FP32 QMR on all of
    them, every problem advanced by one CUDA graph; then the same problems one
    after another for comparison."""
    import torch
    probs = hm.batched_problems(nprob, seed=0)
    ctxs = [capi.Context.from_problem(p, e0=0.0, device=device) for p in probs]
    try:
        t0 = time.perf_counter()
        for c in ctxs:
            c.set_precond(capi.TOSBD1, 0.002, 0.0)
            c.build_osb(20, 1e-4)
        build_s = time.perf_counter() - t0
        rng = np.random.default_rng(7)
        shifts = np.stack([float(p.RES.min()) + 0.02 * (np.arange(nrhs) + 0.5) / nrhs for p in probs])
        dBs = [torch.tensor(rng.standard_normal((nrhs, p.N)), device=f"cuda:{device}") for p in probs]
        dXs = [torch.zeros_like(b) for b in dBs]
        capi.qmr_shifts_batch(ctxs[:1], shifts[:1], dBs[:1], dXs[:1], 2000, 1e-4)      # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        codes, res, dev_s = capi.qmr_shifts_batch(ctxs, shifts, dBs, dXs, 2000, 1e-4,
                                                  precision=capi.PREC_FP32)
        wall = time.perf_counter() - t0
        its = np.abs(codes).astype(np.int64)
        points = np.array([p.N for p in probs])
        hx_apps = int((2 * its).sum())                      # QMR_MPI type -1: 2 H*X per iteration
        hx_points = float((2 * its * points[:, None]).sum())
        t0 = time.perf_counter()
        for k, c in enumerate(ctxs):
            c.qmr_shifts_device(dBs[k], torch.zeros_like(dBs[k]), shifts[k], 2000, 1e-4,
                                precision=capi.PREC_FP32)
        torch.cuda.synchronize()
        seq = time.perf_counter() - t0
        return {"problems": nprob, "shifts": nrhs, "points_total": int(points.sum()),
                "points_min": int(points.min()), "points_max": int(points.max()),
                "build_s": build_s, "solve_wall_s": wall, "solve_device_s": dev_s,
                "converged": int((codes > 0).sum()), "systems": int(codes.size),
                "qmr_iterations_total": int(its.sum()), "hx_apps": hx_apps,
                "hx_apps_per_s": hx_apps / wall, "hx_points_per_s": hx_points / wall,
                "one_by_one_wall_s": seq, "batch_speedup": seq / wall}
    finally:
        for c in ctxs:
            c.close()


# ------------------------------------------------------------------- ours --
def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    from scalit_gb300 import capi, hamiltonian as hm
    capi.load(build_if_missing=True)
    p = hm.workload(args.workload)
    e0 = float(p.RES.min())
    N, nvec = p.N, args.nvec
    ctx = capi.Context.from_problem(p, e0=e0, device=local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    gen = torch.Generator(device=f"cuda:{local}").manual_seed(1234 + rank)
    X = [torch.randn(nvec, N, dtype=torch.float64, device=f"cuda:{local}", generator=gen) for _ in range(2)]
    Y = [torch.empty_like(X[0]) for _ in range(2)]
    torch.cuda.synchronize()

    def step(i):
        ctx.hx_device(X[i % 2], Y[i % 2], nvec, capi.TA1)

    for i in range(max(args.warmup, 3)):
        step(i)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for i in range(args.steps):
                step(i)
            ev1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = ev0.elapsed_time(ev1)
    ms_max = reduce_max(ms, world)
    value = replicas_value(args.steps * nvec, world, ms_max / 1e3)

    # per-level kernel timing (the strided GEMM launches of one application)
    total_flops, total_bytes, lv = hx_units(p.sizes)
    level_ms = []
    reps = 20
    for l in range(len(p.sizes)):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            for i in range(3):
                ctx.level_device(l + 1, X[i % 2][i], Y[i % 2][i], accumulate=l > 0)
            a.record(stream)
            for i in range(reps):
                ctx.level_device(l + 1, X[i % 2][i % nvec], Y[i % 2][i % nvec], accumulate=l > 0)
            b.record(stream)
        torch.cuda.synchronize()
        level_ms.append(a.elapsed_time(b) / reps)
    dom = int(np.argmax(level_ms))
    hbm, bf16, peak_src = load_peaks()
    ach_gbs = lv[dom]["bytes"] / (level_ms[dom] / 1e3) / 1e9
    ach_tf = lv[dom]["flops"] / (level_ms[dom] / 1e3) / 1e12

    # FP64 reference rate: cuBLAS DGEMM measured live (the FP64 unit this path runs on)
    fp64_peak = None
    try:
        m = 4096
        A = torch.randn(m, m, dtype=torch.float64, device=f"cuda:{local}")
        B = torch.randn(m, m, dtype=torch.float64, device=f"cuda:{local}")
        for _ in range(2):
            A @ B
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(3):
            A @ B
        b.record()
        torch.cuda.synchronize()
        fp64_peak = 2.0 * m ** 3 * 3 / (a.elapsed_time(b) / 1e3) / 1e12
        del A, B
    except Exception:
        fp64_peak = None

    # FP32 (the inner-solve arithmetic) on the same block, both FP32 engines
    X32 = [x.float() for x in X]
    Y32 = [torch.empty_like(x) for x in X32]

    def time_f32(fn):
        with torch.cuda.stream(stream):
            for i in range(3):
                fn(X32[i % 2], Y32[i % 2], nvec, capi.TA1)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            for i in range(args.steps):
                fn(X32[i % 2], Y32[i % 2], nvec, capi.TA1)
            b.record(stream)
        torch.cuda.synchronize()
        return args.steps * nvec / (a.elapsed_time(b) / 1e3)

    fp32_engines = {}
    for name, mode in (("simt", capi.FP32_SIMT), ("tensor_bf16x3", capi.FP32_TENSOR)):
        ctx.set_fp32_mode(mode)
        fp32_engines[name] = time_f32(ctx.hx_f32_device)
    ctx.set_fp32_mode(capi.FP32_SIMT)
    fp32_apps = max(fp32_engines.values())

    # P*X (MYPX, TA1) of the same block in FP64 and FP32, after one preconditioner build
    t0 = time.perf_counter()
    ctx.build_osb(20, 1e-4)
    build_s = time.perf_counter() - t0
    build_levels = [float(v) for v in ctx.build_times()]
    px_apps = {}
    for name, xs, ys, fn in (("fp64", X, Y, ctx.px_device), ("fp32", X32, Y32, ctx.px_f32_device)):
        with torch.cuda.stream(stream):
            for i in range(3):
                fn(xs[i % 2], ys[i % 2], nvec, capi.TA1)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            for i in range(args.steps):
                fn(xs[i % 2], ys[i % 2], nvec, capi.TA1)
            b.record(stream)
        torch.cuda.synchronize()
        px_apps[name] = args.steps * nvec / (a.elapsed_time(b) / 1e3)
    ctx.set_fp32_mode(capi.FP32_TENSOR)
    px_apps["fp32_tensor_bf16x3"] = time_f32(ctx.px_f32_device)
    ctx.set_fp32_mode(capi.FP32_SIMT)
    del X32, Y32

    # end to end through the host-buffer ABI (pinned host memory)
    Xh = X[0].cpu().pin_memory()
    Yh = torch.empty_like(Xh).pin_memory()
    xh, yh = Xh.numpy(), Yh.numpy()
    ctx.hx(xh, capi.TA1)
    e2e_steps = max(3, args.steps // 4)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.hx(xh, capi.TA1, out=yh)
    e2e_s = time.perf_counter() - t0
    e2e_s = reduce_max(e2e_s, world)
    e2e_value = replicas_value(e2e_steps * nvec, world, e2e_s)

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(p, e0, args.cpu_seconds)
    pist = None
    if args.pist_workload != "none" and args.pist_levels > 0:
        pist = pist_leg(args.pist_workload, args.pist_levels, local, capi, hm,
                        arms=tuple(a.strip() for a in args.pist_arms.split(",")), warmup=args.pist_warmup > 0)
    batch = None
    if args.batch_problems > 0:
        batch = batch_leg(args.batch_problems, args.batch_shifts, local, capi, hm)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "H*X apps/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": args.workload, "grid": list(p.sizes), "npoints": N,
                       "vectors_per_step": nvec, "operator": "MYHX TA1 (H - E0) X",
                       "parallelism": f"replicas{world}",
                       "l2": "two alternating 2x151 MB input/output sets (> 129 MB L2)"},
            "roofline": {"bound": "hbm", "achieved": ach_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": ach_gbs / hbm, "traffic": profiled_traffic(args.workload, dom + 1),
                         "kernel": f"tc_level_kernel level {dom + 1}",
                         "peak_source": peak_src,
                         "algorithmic_bytes_per_launch": lv[dom]["bytes"],
                         "launch_ms": level_ms[dom]},
            "fp64_roofline": {"bound": "fp64", "achieved": ach_tf, "unit": "TFLOP/s",
                              "peak": fp64_peak, "frac": (ach_tf / fp64_peak) if fp64_peak else None,
                              "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                              "algorithmic_flops_per_launch": lv[dom]["flops"]},
            "level_ms": level_ms,
            "hx_flops_per_app": total_flops, "hx_bytes_per_app": total_bytes,
            "fp32_apps_per_s": fp32_apps, "fp32_engines_apps_per_s": fp32_engines,
            "px_apps_per_s": px_apps,
            "osb_build": {"seconds": build_s, "levels_s": build_levels},
            "e2e": {"value": e2e_value, "unit": "H*X apps/s",
                    "h2d_bytes_per_step": int(nvec * N * 8), "d2h_bytes_per_step": int(nvec * N * 8)},
            "gpu_launches": args.steps * len(p.sizes),
            "clocks": clk.summary(),
        }
        if base is not None:
            line["cpu_baseline"] = base
        if pist is not None:
            line["pist"] = pist
        if batch is not None:
            line["batch"] = batch
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
