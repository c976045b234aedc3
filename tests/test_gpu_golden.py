"""Device PIST against the oracle's committed level fixtures
(tests/golden/pist_*.json, made by tests/golden/make_pist_levels.py): the
24x32x20 problem with the plain (TOSB) and the windowed (TOSBD1, DE = 0.05 Eh)
preconditioner, and the 96x96x64 problem (100 levels, QMR tolerance 1e-4,
at most 2000 Krylov vectors), each with FP64 and with mixed inner solves.
Every level must lie within 1e-4 cm^-1 of the oracle's.
"""
import json
import os

import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

CM_TOL = 1e-4
HERE = os.path.dirname(os.path.abspath(__file__))


def fixture(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def run_pist(fx, prec, orth):
    p = hm.workload(fx["workload"])
    x0 = np.random.default_rng(fx["seed"]).random(p.N)
    with capi.Context.from_problem(p, e0=fx["e0"]) as ctx:
        if fx["osb_kind"] != capi.TOSB:
            ctx.set_precond(fx["osb_kind"], fx["osb_de"], 0.0)
        if prec == capi.PREC_FP32:
            ctx.set_fp32_mode(capi.FP32_TENSOR_PX)
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, fx["levels"], fx["e0"], fx["etol"], startcnt=fx["startcnt"],
                                      stepcnt=fx["stepcnt"], m_max=fx["m_max"], qmr_max=fx["qmr_max"],
                                      qmr_tol=fx["qmr_tol"], precision=prec, orth=orth)
    return st, eig, info


ARMS = [(capi.PREC_FP64, 1), (capi.PREC_FP32, 2)]


@pytest.mark.parametrize("name", ["pist_tri-24x32x20.json", "pist_tri-24x32x20_osbd1.json"])
@pytest.mark.parametrize("prec,orth", ARMS)
def test_pist_c0_fixture(lib, name, prec, orth):
    fx = fixture(name)
    st, eig, _ = run_pist(fx, prec, orth)
    assert st > 0 and fx["status"] > 0
    err = np.abs(eig - np.array(fx["eigenvalues_eh"])) * hm.HARTREE_CM
    print(f"{name} prec={prec}: max |dE| = {err.max():.2e} cm^-1, Krylov {st} (oracle {fx['status']})")
    assert err.max() < CM_TOL


@pytest.mark.slow
@pytest.mark.parametrize("prec,orth", ARMS)
def test_pist_c1_fixture(lib, prec, orth):
    """96x96x64, 100 levels: the plain-FP64 GPU workload's PIST."""
    fx = fixture("pist_tri-96x96x64.json")
    st, eig, info = run_pist(fx, prec, orth)
    assert st > 0 and fx["status"] > 0
    err = np.abs(eig - np.array(fx["eigenvalues_eh"])) * hm.HARTREE_CM
    print(f"C1 prec={prec}: max |dE| = {err.max():.2e} cm^-1, Krylov {st} (oracle {fx['status']}), "
          f"QMR iterations {info['qmr_total']} (oracle {fx['qmr_iterations']})")
    assert err.max() < CM_TOL
