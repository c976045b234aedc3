"""Generate the PIST eigenvalue fixtures of the oracle (CPU, FP64).

Runs the oracle's restatement of the reference's PIST_CONV (pist.f90:7-98,
pistH0 pistHij.f90:70-125, with classical Gram-Schmidt applied twice as the
orthogonalisation, the library's default), its QMR inner solves (qmr.f90:5-175)
and its block-Jacobi preconditioner build (hosbdiag.f90:5-75) on a named
workload, and writes the converged levels with the run's parameters to
tests/golden/pist_<workload>[_<tag>].json.  The GPU tests compare the device
PIST (FP64 and mixed inner solves) with these files.

    python tests/golden/make_pist_levels.py tri-96x96x64 --levels 100 --m-max 2000

The start vector is the seeded uniform(0, 1) vector the tests and the bench
use (the reference draws it with random_number).  Expect minutes for the
589,824-point grid on a few cores; the file records the wall time.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def run(workload, levels, m_max, qmr_tol, qmr_max, etol, osb_kind, osb_de, start, step, seed, log):
    from oracle import oracle as orc
    from scalit_gb300 import hamiltonian as hm

    p = hm.workload(workload)
    e0 = float(p.RES.min())
    op = orc.Operator.from_problem(p, E0=e0)
    t0 = time.perf_counter()
    op.build_osb(20, 1e-4)
    t1 = time.perf_counter()
    x0 = orc.start_vector(p.N, seed)
    counts = {"solves": 0, "iters": 0}

    def lin(v):
        rc, X, _, _ = op.qmr(v, qmr_max, qmr_tol, nosb=osb_kind, de=osb_de)
        counts["solves"] += 1
        counts["iters"] += abs(rc)
        return rc, X

    st, eig, res, info = orc.pist_conv(e0, etol, 0, x0, start, step, 1, levels, m_max,
                                       lambda v: op.hx(v, 0), lin, log=log, orth=1)
    t2 = time.perf_counter()
    return {
        "workload": workload, "grid": list(p.sizes), "npoints": int(p.N), "levels": levels,
        "e0": e0, "etol": etol, "qmr_tol": qmr_tol, "qmr_max": qmr_max, "m_max": m_max,
        "startcnt": start, "stepcnt": step, "stepeig": 1, "orth": "classical Gram-Schmidt twice",
        "osb_kind": osb_kind, "osb_de": osb_de, "seed": seed,
        "status": int(st), "res": float(res), "krylov": int(abs(st)),
        "qmr_solves": counts["solves"], "qmr_iterations": counts["iters"],
        "build_s": t1 - t0, "pist_s": t2 - t1, "threads": orc.num_threads(),
        "eigenvalues_eh": [float(v) for v in eig],
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload")
    ap.add_argument("--levels", type=int, required=True)
    ap.add_argument("--m-max", type=int, default=0, help="default: 8 x levels, at least 400")
    ap.add_argument("--start", type=int, default=0, help="default: 2 x levels (setPISTConvParam)")
    ap.add_argument("--step", type=int, default=5)
    ap.add_argument("--qmr-tol", type=float, default=1e-4)
    ap.add_argument("--qmr-max", type=int, default=2000)
    ap.add_argument("--etol", type=float, default=1e-11)
    ap.add_argument("--osb-kind", type=int, default=1, help="1 TOSB, 2 TOSBD1")
    ap.add_argument("--osb-de", type=float, default=0.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--tag", default="")
    a = ap.parse_args()
    m_max = a.m_max or max(8 * a.levels, 400)
    start = a.start or 2 * a.levels
    out = run(a.workload, a.levels, m_max, a.qmr_tol, a.qmr_max, a.etol, a.osb_kind, a.osb_de, start, a.step,
              a.seed, log=lambda s: print(s, flush=True))
    name = f"pist_{a.workload}{'_' + a.tag if a.tag else ''}.json"
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {name}: status {out['status']}, {out['qmr_iterations']} QMR iterations, "
          f"{out['pist_s']:.1f} s", flush=True)


if __name__ == "__main__":
    main()
