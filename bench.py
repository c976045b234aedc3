"""Benchmark of the H*X / PIST hot path on GB300.

One step = one FP64 H*X application (MYHX, TA1) to a block of 16 vectors on
the 160 x 160 x 120 Jacobi-DVR grid (3,072,000 points), the grid the metric's
PIST leg is quoted on.  Inputs are seeded N(0,1) vectors already resident in
HBM; two input/output sets (2 x 786 MB, far larger than the 129 MB L2)
alternate between steps.  `e2e` repeats the measurement through the
host-buffer C ABI (scalit_hx), host<->device copies included.  The roofline
object describes the dominant level launch of that same 16-vector step, timed
with CUDA events on the context's stream; `hx_fp32` does the same for the FP32
H*X of the precision form (both FP32 engines).

Legs (each reported in the JSON line): P*X FP64/FP32; PIST on 24x32x20 (20
levels) and 96x96x64 (100 levels) against the oracle's level fixtures in
tests/golden; PIST on 160x160x120 (200 levels) with FP64 and with mixed inner
solves, per-level differences; the batched shifted QMR over 48 uneven
problems; the CPU baseline (the oracle's MYHX and PIST on the host cores).

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

# the 200-level PIST leg: the FP64 residual its levels are taken to (Eh), the
# cap on basis extensions after the eigenvalue-change test, and the inner
# solves' tolerance that makes the residual target reachable
REFINE_TOL, REFINE_STEPS, PIST_QMR_TOL = 1e-8, 20, 1e-6

# FP32 H*X engines timed by the bench, and the kernel each runs
FP32_ENGINES = (("simt", 0), ("tensor_bf16x3", 1), ("tensor_f16x3", 3))
FP32_KERNEL = {"simt": "gemm_kernel<float>", "tensor_bf16x3": "tc32p_level_kernel<false>",
               "tensor_f16x3": "tc32p_level_kernel<true>"}
FP32_PROFILE = {"simt": "gemm_kernel_f32", "tensor_bf16x3": "tc32p_level_kernel",
                "tensor_f16x3": "tc32p_level_kernel"}
# the engine of the mixed arms' FP32 inner solves: H*X in split-FP16 x3 on the
# tensor cores (the accuracy of the CUDA-core GEMM), the preconditioner's
# rotations in split-BF16 x3
MIXED_FP32_MODE = 3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tri-160x160x120")
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
    ap.add_argument("--batch-problems", type=int, default=48,
                    help="shifted-QMR leg over this many uneven problems (0 skips it)")
    ap.add_argument("--golden-pist", default="tri-24x32x20,tri-96x96x64",
                    help="PIST legs compared with the oracle's level fixtures ('none' skips them)")
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


def profiled_traffic(kernel, workload, level, nvec):
    """DRAM bytes (read + write) of one nvec-vector launch of a level kernel,
    from the committed ncu summary of this workload: the summary lists the
    bytes of one vector's share (a smaller capture scaled by its vectors),
    multiplied here by nvec (None when not profiled)."""
    import re
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        with open(path) as f:
            m = re.search(rf"traffic_per_vector_level{level}:\s*(\d+)", f.read())
        return int(m.group(1)) * nvec if m else None
    except OSError:
        return None


def hx_units(sizes, w=8, diag_level=0):
    """Algorithmic flops and bytes of one H*X application (one vector), and per level.

    flops: 2 N n_l per level plus the diagonal (V - E0) X and the level sums (5N).
    bytes of a level launch: read X, write Y, and read Y when accumulating
    (levels 2..sF), plus the small level matrix; DEP and V where used (V on
    the level that carries the diagonal term: the first on the FP64 engines,
    the last on the persistent FP32 kernel).
    w: bytes per value (8 FP64, 4 FP32).
    """
    n = list(sizes)
    N = int(np.prod(n))
    levels = []
    for l, nl in enumerate(n):
        flops = 2.0 * N * nl
        byts = (2 + (1 if l > 0 else 0)) * N * w + nl * nl * w
        if l == diag_level:
            byts += N * w            # V for the fused diagonal term
            flops += 3.0 * N
        if l == len(n) - 1:
            byts += (N // nl) * w    # DEP factors c(r, R)
            flops += N
        levels.append({"flops": flops, "bytes": byts})
    total_flops = sum(x["flops"] for x in levels) + N
    total_bytes = 3 * N * w + sum(m * m for m in n) * w + (N // n[-1]) * w
    return total_flops, total_bytes, levels


def hx_config(p, nvec, operator="MYHX TA1 (H - E0) X", world=1):
    """The `config` of both arms' JSON lines (identical by construction)."""
    return {"workload": f"tri-{p.sizes[0]}x{p.sizes[1]}x{p.sizes[2]}", "grid": list(p.sizes), "npoints": p.N,
            "vectors_per_step": nvec, "operator": operator, "parallelism": f"replicas{world}",
            "l2": "inputs larger than the 129 MB L2 (16 FP64 vectors of 24.6 MB per block)"}


# ------------------------------------------------------------- reference --
def cpu_hx_rate(op, N, seconds, cap=64):
    """The oracle's MYHX (TA1) applications per second on a bounded sample."""
    x = np.random.default_rng(0).standard_normal(N)
    op.hx(x, 1)
    t0 = time.perf_counter()
    op.hx(x, 1)
    one = time.perf_counter() - t0
    reps = max(1, min(cap, int(seconds / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(reps):
        op.hx(x, 1)
    return reps, reps / (time.perf_counter() - t0)


def cpu_pist_baseline(hm, seconds_capped=8.0):
    """The oracle's PIST on the host cores: the 24x32x20 problem in full (20
    levels, its level fixture's parameters), and on 96x96x64 the rates of a
    capped run -- QMR iterations per second and seconds per Krylov step (QMR
    solve + re-orthogonalised Gram-Schmidt + HMAT column) -- next to the
    committed fixture's full CPU run (tests/golden)."""
    from oracle import oracle as orc
    out = {"cores": orc.num_threads(), "kind": "port"}
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min())
    op = orc.Operator.from_problem(p, E0=e0)
    t0 = time.perf_counter()
    op.build_osb(20, 1e-4)
    t1 = time.perf_counter()
    x0 = orc.start_vector(p.N, 0)

    def lin(v):
        rc, X, _, _ = op.qmr(v, 2000, 1e-4)
        return rc, X

    st, eig, _, _ = orc.pist_conv(e0, 1e-11, 0, x0, 40, 5, 1, 20, 400, lambda v: op.hx(v, 0), lin, orth=1)
    t2 = time.perf_counter()
    out["tri-24x32x20"] = {"levels": 20, "status": int(st), "build_s": t1 - t0, "pist_s": t2 - t1,
                           "seconds": t2 - t0, "levels_per_s": 20 / (t2 - t0)}
    return out


def cpu_baseline(problem, e0, seconds, hm, with_pist=True):
    """The oracle on the host cores: MYHX applications per second on a bounded
    sample of the bench's grid, and the PIST baseline."""
    from oracle import oracle as orc
    op = orc.Operator.from_problem(problem, E0=e0)
    reps, value = cpu_hx_rate(op, problem.N, seconds)
    out = {"value": value, "unit": "H*X apps/s", "cores": orc.num_threads(), "kind": "port",
           "sample": f"{reps} FP64 H*X applications (TA1) on the {problem.sizes[0]}x"
                     f"{problem.sizes[1]}x{problem.sizes[2]} grid, oracle C restatement of MYHX "
                     f"(osb.hx.h:71-110), OpenMP over blocks"}
    if with_pist:
        out["pist"] = cpu_pist_baseline(hm)
    return out


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
    # each step is a bounded sample of the nvec-vector step, capped so the run stays short
    per_step = max(1, min(args.nvec, int(2.0 / max(one, 1e-6))))
    for _ in range(min(args.warmup, 3)):
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
        "config": hx_config(p, args.nvec, world=world),
        "cpu_baseline": {"value": value, "unit": "H*X apps/s", "cores": orc.num_threads(),
                         "kind": "port",
                         "sample": f"{per_step} of the step's {args.nvec} applications per step, oracle C "
                                   f"restatement of MYHX (osb.hx.h:71-110)"},
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
    for prec, orth in ((capi.PREC_FP64, 1), (capi.PREC_FP32_REFINED, 3)) if warmup else ():
        with capi.Context.from_problem(pw, e0=float(pw.RES.min()), device=device) as ctx:
            if prec != capi.PREC_FP64:
                ctx.set_fp32_mode(MIXED_FP32_MODE)
                ctx.set_build_precision(capi.PREC_FP32)
                ctx.set_fp32_px_storage(16)
            ctx.build_osb(20, 1e-4)
            ctx.pist(np.random.default_rng(0).random(pw.N), levels, float(pw.RES.min()), 1e-11,
                     m_max=max(8 * levels, 400), qmr_max=2000, qmr_tol=PIST_QMR_TOL, precision=prec, orth=orth,
                     refine_tol=REFINE_TOL, refine_steps=REFINE_STEPS)
    p = hm.workload(workload)
    e0 = float(p.RES.min())
    x0 = np.random.default_rng(0).random(p.N)
    out = {"workload": workload, "levels": levels}
    eigs = {}
    # mixed leg: FP32 inner solves (H*X in split-FP16 x3 and the preconditioner's
    # rotations in split-BF16 x3 on the tensor cores) on a preconditioner whose
    # first-level Jacobi sweeps run in FP32 and whose first-level matrices the
    # FP32 P*X streams in FP16 (it only feeds those solves), and
    # an FP32 first Gram-Schmidt pass (the re-orthogonalisation's projections,
    # HMAT and the Ritz solves stay FP64; its update streams the basis' FP32
    # copy with coefficients split into two FP32 parts)
    for name, prec, orth in (("fp64", capi.PREC_FP64, 1), ("fp32", capi.PREC_FP32_REFINED, 3)):
        if name not in arms:
            continue
        with capi.Context.from_problem(p, e0=e0, device=device) as ctx:
            if prec != capi.PREC_FP64:
                ctx.set_fp32_mode(MIXED_FP32_MODE)
                ctx.set_build_precision(capi.PREC_FP32)
                ctx.set_fp32_px_storage(16)
            t0 = time.perf_counter()
            stats = ctx.build_osb(20, 1e-4)
            t1 = time.perf_counter()
            build_levels = [float(v) for v in ctx.build_times()]
            st, eig, res, info = ctx.pist(x0, levels, e0, 1e-11, m_max=max(8 * levels, 400),
                                          qmr_max=2000, qmr_tol=PIST_QMR_TOL, precision=prec, orth=orth,
                                          refine_tol=REFINE_TOL, refine_steps=REFINE_STEPS)
            t2 = time.perf_counter()
        eigs[name] = eig
        out[name] = {"status": st, "orth": orth, "seconds": t2 - t0, "build_s": t1 - t0, "pist_s": t2 - t1,
                     "build_sweeps": "FP32 on the first level" if prec != capi.PREC_FP64 else "FP64",
                     "px_level1_storage": "FP16" if prec != capi.PREC_FP64 else "FP64",
                     "inner_solves": ("FP32 QMR under FP64 iterative refinement (H*X split-FP16 x3 "
                                      "tensor cores, preconditioner rotations split-BF16 x3 tensor cores)"
                                      if prec != capi.PREC_FP64 else "FP64 QMR"),
                     "qmr_tol": PIST_QMR_TOL,
                     "build_levels_s": build_levels,
                     "sweeps_per_block": [float(stats[l, 4] / int(np.prod(p.sizes[l + 1:])))
                                          for l in range(len(p.sizes))],
                     "levels_per_s": levels / (t2 - t0), "krylov": info["krylov"],
                     "qmr_iterations": info["qmr_total"], "qmr_solves": info["qmr_solves"],
                     "t_qmr": info["t_qmr"], "t_orth": info["t_orth"], "t_hmat": info["t_hmat"],
                     "t_ritz": info["t_ritz"], "t_resid_and_refine": info["t_resid"],
                     "refine_steps": info["refine_steps"], "refine_tol_eh": REFINE_TOL,
                     "max_residual_eh": float(np.max(info["resid"])),
                     "residuals_eh": [float(f"{r:.3g}") for r in info["resid"]]}
    fx = load_fixture(workload)
    if fx is not None and fx.get("levels") == levels:
        ref = np.array(fx["eigenvalues_eh"])
        for name, eig in eigs.items():
            err = np.abs(eig - ref) * hm.HARTREE_CM
            out[name]["max_err_vs_oracle_cm"] = float(err.max())
            out[name]["per_level_err_vs_oracle_cm"] = [float(f"{d:.3g}") for d in err]
    if "fp64" in eigs and "fp32" in eigs:
        out["speedup_fp32_inner"] = out["fp64"]["seconds"] / out["fp32"]["seconds"]
        out["speedup_excluding_build"] = out["fp64"]["pist_s"] / out["fp32"]["pist_s"]
        diff = np.abs(eigs["fp32"] - eigs["fp64"]) * hm.HARTREE_CM
        out["max_abs_diff_cm"] = float(diff.max())
        out["per_level_diff_cm"] = [float(f"{d:.3g}") for d in diff]
    out["lowest_eigenvalues_eh"] = [float(v) for v in next(iter(eigs.values()))[:5]] if eigs else []
    return out


def load_fixture(workload):
    path = os.path.join(ROOT, "tests", "golden", f"pist_{workload}.json")
    try:
        with open(path) as f:
            return json.load(f)
    except OSError:
        return None


def golden_pist_leg(workload, device, capi, hm):
    """PIST with FP64 and with mixed inner solves on a workload whose oracle
    levels are committed (tests/golden), with the fixture's parameters: wall
    time from the build, levels/s and the largest level error against the
    FP64 oracle, next to the oracle's own CPU time for the same solve."""
    fx = load_fixture(workload)
    if fx is None:
        return None
    p = hm.workload(workload)
    x0 = np.random.default_rng(fx["seed"]).random(p.N)
    out = {"levels": fx["levels"], "oracle_krylov": fx["status"], "oracle_qmr_iterations": fx["qmr_iterations"],
           "oracle_cpu_seconds": fx["build_s"] + fx["pist_s"], "oracle_cpu_threads": fx["threads"]}
    ref = np.array(fx["eigenvalues_eh"])
    for name, prec, orth in (("fp64", capi.PREC_FP64, 1), ("fp32", capi.PREC_FP32, 2)):
        with capi.Context.from_problem(p, e0=fx["e0"], device=device) as ctx:
            if prec == capi.PREC_FP32:
                ctx.set_fp32_mode(MIXED_FP32_MODE)
                ctx.set_build_precision(capi.PREC_FP32)
                ctx.set_fp32_px_storage(16)
            t0 = time.perf_counter()
            ctx.build_osb(20, 1e-4)
            st, eig, _, info = ctx.pist(x0, fx["levels"], fx["e0"], fx["etol"], startcnt=fx["startcnt"],
                                        stepcnt=fx["stepcnt"], m_max=fx["m_max"], qmr_max=fx["qmr_max"],
                                        qmr_tol=fx["qmr_tol"], precision=prec, orth=orth, residuals=True)
            dt = time.perf_counter() - t0
        err = np.abs(eig - ref) * hm.HARTREE_CM
        out[name] = {"status": st, "seconds": dt, "levels_per_s": fx["levels"] / dt,
                     "qmr_iterations": info["qmr_total"], "max_err_vs_oracle_cm": float(err.max()),
                     "max_residual_eh": float(np.max(info["resid"]))}
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
            torch.cuda.nvtx.range_push("hx_fp64_step")    # names the launches for ncu --nvtx-include
            ev0.record(stream)
            for i in range(args.steps):
                step(i)
            ev1.record(stream)
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = ev0.elapsed_time(ev1)
    ms_max = reduce_max(ms, world)
    value = replicas_value(args.steps * nvec, world, ms_max / 1e3)

    # the dominant level launch of the same 16-vector step: CUDA events between
    # the step's level launches on the context's stream (the 16-vector block
    # of 393 MB does not fit the 129 MB L2, so every launch streams from HBM)
    # the persistent FP64 kernel carries the diagonal term on the last level
    total_flops, total_bytes, lv = hx_units(p.sizes, 8, diag_level=len(p.sizes) - 1)
    level_ms = ctx.hx_level_times(X[0], Y[0], nvec, reps=10)
    dom = int(np.argmax(level_ms))
    hbm, bf16, peak_src = load_peaks()
    dom_bytes = nvec * lv[dom]["bytes"]
    ach_gbs = dom_bytes / (level_ms[dom] / 1e3) / 1e9
    ach_tf = nvec * lv[dom]["flops"] / (level_ms[dom] / 1e3) / 1e12

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

    # FP32 H*X of the precision form (the QMR inner solves' arithmetic) on the
    # same block, both FP32 engines, with the dominant level's HBM roofline
    X32 = [x.float() for x in X]
    Y32 = [torch.empty_like(x) for x in X32]

    def time_f32(fn, steps=args.steps, label="fp32"):
        with torch.cuda.stream(stream):
            for i in range(3):
                fn(X32[i % 2], Y32[i % 2], nvec, capi.TA1)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            torch.cuda.nvtx.range_push(label)
            a.record(stream)
            for i in range(steps):
                fn(X32[i % 2], Y32[i % 2], nvec, capi.TA1)
            b.record(stream)
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        return steps * nvec / (a.elapsed_time(b) / 1e3)

    _, bytes32, lv32 = hx_units(p.sizes, 4, diag_level=len(p.sizes) - 1)
    fp32 = {"dtype": "f32", "engines_apps_per_s": {}, "engines_level_ms": {}}
    for name, mode in FP32_ENGINES:
        ctx.set_fp32_mode(mode)
        fp32["engines_apps_per_s"][name] = time_f32(ctx.hx_f32_device, label=f"hx_fp32_{name}")
        fp32["engines_level_ms"][name] = ctx.hx_level_times(X32[0], Y32[0], nvec, reps=10)
    # the roofline of the engine the mixed arms' inner solves run (split-FP16 x3:
    # the CUDA-core GEMM's accuracy); the split-BF16 x3 rate is listed beside it
    best = "tensor_f16x3"
    lms = fp32["engines_level_ms"][best]
    d32 = int(np.argmax(lms))
    a32 = nvec * lv32[d32]["bytes"] / (lms[d32] / 1e3) / 1e9
    fp32.update({"apps_per_s": fp32["engines_apps_per_s"][best], "engine": best,
                 "hbm_fraction_whole_step": fp32["engines_apps_per_s"][best] * bytes32 / 1e9 / hbm,
                 "roofline": {"bound": "hbm", "achieved": a32, "peak": hbm, "unit": "GB/s", "frac": a32 / hbm,
                              "kernel": f"{FP32_KERNEL[best]} level {d32 + 1}",
                              "algorithmic_bytes_per_launch": nvec * lv32[d32]["bytes"], "launch_ms": lms[d32],
                              "traffic": profiled_traffic(FP32_PROFILE[best], args.workload, d32 + 1, nvec),
                              "peak_source": peak_src}})
    ctx.set_fp32_mode(capi.FP32_SIMT)

    # P*X (MYPX, TA1) of the same block in FP64 and FP32, after one preconditioner build
    t0 = time.perf_counter()
    ctx.build_osb(20, 1e-4)
    build_s = time.perf_counter() - t0
    build_levels = [float(v) for v in ctx.build_times()]
    px_apps = {}
    for name, xs, ys, fn in (("fp64", X, Y, ctx.px_device), ("fp32", X32, Y32, ctx.px_f32_device)):
        with torch.cuda.stream(stream):
            for i in range(2):
                fn(xs[i % 2], ys[i % 2], nvec, capi.TA1)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(2, args.steps // 4)
        with torch.cuda.stream(stream):
            a.record(stream)
            for i in range(reps):
                fn(xs[i % 2], ys[i % 2], nvec, capi.TA1)
            b.record(stream)
        torch.cuda.synchronize()
        px_apps[name] = reps * nvec / (a.elapsed_time(b) / 1e3)
    ctx.set_fp32_mode(capi.FP32_TENSOR_PX)
    px_apps["fp32_tensor_rotations"] = time_f32(ctx.px_f32_device, max(2, args.steps // 4))
    ctx.set_fp32_mode(capi.FP32_SIMT)
    del X32, Y32

    # end to end through the host-buffer ABI (pinned host memory)
    Xh = X[0].cpu().pin_memory()
    Yh = torch.empty_like(Xh).pin_memory()
    xh, yh = Xh.numpy(), Yh.numpy()
    ctx.hx(xh, capi.TA1, out=yh)
    e2e_steps = max(3, args.steps // 4)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.hx(xh, capi.TA1, out=yh)
    e2e_s = time.perf_counter() - t0
    e2e_s = reduce_max(e2e_s, world)
    e2e_value = replicas_value(e2e_steps * nvec, world, e2e_s)
    ctx.close()
    del X, Y, Xh, Yh
    torch.cuda.empty_cache()

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(p, e0, args.cpu_seconds, hm)
    golden = {}
    if args.golden_pist != "none":
        for wl in (w.strip() for w in args.golden_pist.split(",") if w.strip()):
            g = golden_pist_leg(wl, local, capi, hm)
            if g is not None:
                golden[wl] = g
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
            "config": hx_config(p, nvec, world=world),
            "roofline": {"bound": "hbm", "achieved": ach_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": ach_gbs / hbm, "traffic": profiled_traffic("tc64p_level_kernel", args.workload,
                                                                           dom + 1, nvec),
                         "kernel": f"tc64p_level_kernel level {dom + 1}",
                         "peak_source": peak_src,
                         "algorithmic_bytes_per_launch": dom_bytes,
                         "launch_ms": level_ms[dom], "vectors_per_launch": nvec},
            "fp64_roofline": {"bound": "fp64", "achieved": ach_tf, "unit": "TFLOP/s",
                              "peak": fp64_peak, "frac": (ach_tf / fp64_peak) if fp64_peak else None,
                              "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                              "algorithmic_flops_per_launch": nvec * lv[dom]["flops"]},
            "level_ms": level_ms,
            "hx_flops_per_app": total_flops, "hx_bytes_per_app": total_bytes,
            "hx_fp32": fp32,
            "px_apps_per_s": px_apps,
            "osb_build": {"seconds": build_s, "levels_s": build_levels},
            "e2e": {"value": e2e_value, "unit": "H*X apps/s",
                    "h2d_bytes_per_step": int(nvec * N * 8), "d2h_bytes_per_step": int(nvec * N * 8)},
            # per level: the row-exponent pass and the level product
            "gpu_launches": args.steps * 2 * len(p.sizes),
            "clocks": clk.summary(),
        }
        if base is not None:
            line["cpu_baseline"] = base
        if golden:
            line["pist_vs_oracle"] = golden
        if pist is not None:
            line["pist"] = pist
        if batch is not None:
            line["batch"] = batch
        print(json.dumps(line), flush=True)
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
