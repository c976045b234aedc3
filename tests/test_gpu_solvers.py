"""QMR and PIST on the GPU against the oracle.

QMR (qmr.f90 / qmr_mpi.f90): same iteration count and status code as the
oracle; solution within 1e-8 norm-wise (FP64).  PIST (pist.f90): eigenvalues
within 1e-4 cm^-1 of the oracle's PIST (HARTREE_CM from sinc.f90:27).
"""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

CM_TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def c0():
    return hm.workload("tri-24x32x20")


@pytest.mark.parametrize("ntype", [-1, -2, 0])
def test_qmr_matches_oracle(lib, orc, c0, ntype):
    e0 = float(c0.RES.min()) - 1e-3
    ref = orc.Operator.from_problem(c0, E0=e0)
    ref.build_osb(20, 1e-4)
    b = np.random.default_rng(0).random(c0.N)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        code, X, res, it = ctx.qmr(b, 300, 1e-9, ntype=ntype)
    code_r, X_r, res_r, it_r = ref.qmr(b, 300, 1e-9, ntype=ntype)
    assert code == code_r
    assert rel(X, X_r) < 1e-8
    # RES ratios near convergence involve |UX|/|X| ~ 1e-10, which carries the
    # rounding of the last update: compare it loosely, the iterates tightly.
    assert res < 1e-9 and res_r < 1e-9
    assert abs(res - res_r) <= 0.05 * res_r


def test_qmr_fp32_converges(lib, c0):
    e0 = float(c0.RES.min()) - 1e-3
    b = np.random.default_rng(1).random(c0.N)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        code, X, res, it = ctx.qmr(b, 300, 1e-4, precision=capi.PREC_FP32)
        r = ctx.hx(X, capi.TA1) - b
    assert code > 0
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-3


def test_qmr_not_converged_code(lib, orc, c0):
    e0 = float(c0.RES.min()) - 1e-3
    b = np.random.default_rng(2).random(c0.N)
    ref = orc.Operator.from_problem(c0, E0=e0)
    ref.build_osb(20, 1e-4)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        code, X, res, it = ctx.qmr(b, 2, 1e-15)
    assert code == -2 == ref.qmr(b, 2, 1e-15)[0]


def test_qmr_zero_rhs_breakdown(lib, c0):
    """B = 0 gives VNRM = 0: QMR_MPI's code -1 (qmr_mpi.f90:82-85)."""
    with capi.Context.from_problem(c0, e0=0.0) as ctx:
        ctx.build_osb(20, 1e-4)
        code, X, res, it = ctx.qmr(np.zeros(c0.N), 10, 1e-8)
    assert code == -1
    assert not X.any()


def test_pist_c0_matches_oracle(lib, orc, c0):
    e0 = float(c0.RES.min())
    ref = orc.Operator.from_problem(c0, E0=e0)
    ref.build_osb(20, 1e-4)
    x0 = orc.start_vector(c0.N, 0)
    M, etol = 20, 1e-11

    def linsolv(v):
        rc, X, _, _ = ref.qmr(v, 500, 1e-4)
        return rc, X

    st_r, eig_r, res_r, info_r = orc.pist_conv(e0, etol, 0, x0, 40, 5, 1, M, 400,
                                               lambda v: ref.hx(v, 0), linsolv)
    assert st_r > 0
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, M, e0, etol, m_max=400, qmr_max=500, qmr_tol=1e-4)
    assert st > 0
    err_cm = np.abs(eig - eig_r).max() * hm.HARTREE_CM
    assert err_cm < CM_TOL, err_cm


def test_pist_fp32_inner(lib, orc, c0):
    """Mixed precision: FP32 QMR inner solves, FP64 basis / HMAT / Ritz."""
    import scipy.sparse.linalg as sla
    e0 = float(c0.RES.min())
    ref = orc.Operator.from_problem(c0, E0=e0)
    exact = np.sort(sla.eigsh(sla.LinearOperator((c0.N, c0.N), matvec=lambda v: ref.hx(v, 0)),
                              k=20, which="SA", tol=1e-13)[0])
    x0 = orc.start_vector(c0.N, 0)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, 20, e0, 1e-11, m_max=400, qmr_max=500, qmr_tol=1e-4,
                                      precision=capi.PREC_FP32)
    assert st > 0
    assert np.abs(eig - exact).max() * hm.HARTREE_CM < CM_TOL


def test_pist_bad_params(lib, c0):
    """stepEig >= M_MAX returns 0 before any work (pist.f90:38-40)."""
    with capi.Context.from_problem(c0, e0=0.0) as ctx:
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(np.ones(c0.N), 5, 0.0, 1e-8, m_max=100, gap=200)
    assert st == 0
    assert info["qmr_solves"] == 0
