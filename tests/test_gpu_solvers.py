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
    """Same recurrence as the oracle (QMR_MPI); iteration count within one."""
    e0 = float(c0.RES.min()) - 1e-3
    ref = orc.Operator.from_problem(c0, E0=e0)
    ref.build_osb(20, 1e-4)
    b = np.random.default_rng(0).random(c0.N)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        code, X, res, it = ctx.qmr(b, 300, 1e-9, ntype=ntype)
    code_r, X_r, res_r, it_r = ref.qmr(b, 300, 1e-9, ntype=ntype)
    # the FP64 H*X engines differ from the oracle at 1e-14; a test that crosses
    # its tolerance at the same iteration within one step is the same recurrence
    assert abs(code - code_r) <= 1 and code > 0
    assert rel(X, X_r) < 1e-7
    assert res < 1e-9 and res_r < 1e-9


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


@pytest.mark.parametrize("orth", [0, 1, 2])
def test_pist_c0_matches_oracle(lib, orc, c0, orth):
    e0 = float(c0.RES.min())
    ref = orc.Operator.from_problem(c0, E0=e0)
    ref.build_osb(20, 1e-4)
    x0 = orc.start_vector(c0.N, 0)
    M, etol = 20, 1e-11

    def linsolv(v):
        rc, X, _, _ = ref.qmr(v, 500, 1e-4)
        return rc, X

    st_r, eig_r, res_r, info_r = orc.pist_conv(e0, etol, 0, x0, 40, 5, 1, M, 400,
                                               lambda v: ref.hx(v, 0), linsolv, orth=min(orth, 1))
    assert st_r > 0
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, M, e0, etol, m_max=400, qmr_max=500, qmr_tol=1e-4, orth=orth)
    assert st > 0
    err_cm = np.abs(eig - eig_r).max() * hm.HARTREE_CM
    assert err_cm < CM_TOL, err_cm


def test_pist_long_run_orthogonality(lib, orc):
    """48x48x32, 50 levels (~200 Krylov vectors).  The reference's single MGS
    pass loses orthogonality here and reports a spurious ~0 Eh level -- the
    oracle and the GPU agree on that (orth=0); with classical Gram-Schmidt
    twice (orth=1) the GPU's levels equal the oracle's re-orthogonalised PIST."""
    p = hm.build_problem(hm.Grid3(48, 48, 32), hm.PES())
    e0 = float(p.RES.min())
    ref = orc.Operator.from_problem(p, E0=e0)
    ref.build_osb(20, 1e-4)
    x0 = orc.start_vector(p.N, 0)

    def linsolv(v):
        rc, X, _, _ = ref.qmr(v, 2000, 1e-4)
        return rc, X

    st_r, eig_r, _, _ = orc.pist_conv(e0, 1e-11, 0, x0, 100, 5, 1, 50, 1000, lambda v: ref.hx(v, 0),
                                      linsolv, orth=1)
    assert st_r > 0 and eig_r[0] > 1e-3          # no spurious level with re-orthogonalisation
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        st0, eig0, _, _ = ctx.pist(x0, 50, e0, 1e-11, m_max=1000, qmr_max=2000, qmr_tol=1e-4, orth=0)
        st1, eig1, _, info1 = ctx.pist(x0, 50, e0, 1e-11, m_max=1000, qmr_max=2000, qmr_tol=1e-4, orth=1)
        # the mixed path: FP32 inner solves and an FP32 first Gram-Schmidt pass
        st2, eig2, _, _ = ctx.pist(x0, 50, e0, 1e-11, m_max=1000, qmr_max=2000, qmr_tol=1e-4, orth=2,
                                   precision=capi.PREC_FP32)
    assert st0 > 0 and eig0[0] < 1e-9            # the reference's MGS: spurious ~0 level
    assert st1 > 0 and st2 > 0
    assert np.abs(eig1 - eig_r).max() * hm.HARTREE_CM < CM_TOL
    assert np.abs(eig2 - eig_r).max() * hm.HARTREE_CM < CM_TOL


ORTH_TOL = 3e-15   # max |V^T V - I|: FP64 round-off; an FP32-rounded update coefficient gives ~1e-14


@pytest.mark.parametrize("orth", [1, 2, 3])
def test_pist_basis_orthogonality(lib, orc, c0, orth):
    """The Krylov basis after classical Gram-Schmidt twice is orthonormal to FP64
    round-off, in FP64 (orth=1) and in the mixed form (orth=2: FP32 first pass,
    FP64 projections and an FP32-streamed update with split coefficients)."""
    e0 = float(c0.RES.min())
    x0 = orc.start_vector(c0.N, 0)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, 20, e0, 1e-11, m_max=400, qmr_max=500, qmr_tol=1e-4,
                                      precision=capi.PREC_FP32, orth=orth, basis=True)
    V = info["vj"]
    assert st > 0 and V.shape[1] > 40
    G = V.T @ V
    err = np.abs(G - np.eye(G.shape[0])).max()
    print(f"orth={orth} basis {V.shape[1]} vectors: max|V^T V - I| = {err:.3e}")
    assert err < ORTH_TOL


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
        with pytest.raises(capi.ScalitError):
            ctx.pist(np.ones(c0.N), 5, 0.0, 1e-8, m_max=100, orth=4)


def test_qmr_matches_oracle_iteration_for_iteration(lib, orc, c0):
    """With the FP64-pipe H*X engine the status code equals the oracle's exactly."""
    e0 = float(c0.RES.min()) - 1e-3
    ref = orc.Operator.from_problem(c0, E0=e0)
    ref.build_osb(20, 1e-4)
    b = np.random.default_rng(0).random(c0.N)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.set_fp64_mode(capi.FP64_DFMA)
        ctx.build_osb(20, 1e-4)
        code, X, res, it = ctx.qmr(b, 300, 1e-9, ntype=-1)
    code_r, X_r, res_r, it_r = ref.qmr(b, 300, 1e-9, ntype=-1)
    assert code == code_r
    assert rel(X, X_r) < 1e-8


def test_pist_residuals_match_host_check(lib, orc, c0):
    """The device residual check |H psi - E psi| equals the oracle's H*X applied
    to the returned Ritz vectors, and is small for converged levels."""
    e0 = float(c0.RES.min())
    ref = orc.Operator.from_problem(c0, E0=e0)
    x0 = orc.start_vector(c0.N, 0)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        st, eig, _, info = ctx.pist(x0, 20, e0, 1e-11, m_max=400, qmr_max=500, qmr_tol=1e-4, residuals=True)
        st_v, eig_v, _, info_v = ctx.pist(x0, 20, e0, 1e-11, m_max=400, qmr_max=500, qmr_tol=1e-4, vectors=True)
    assert st > 0 and st_v == st
    np.testing.assert_array_equal(eig, eig_v)
    psi = info_v["vectors"]
    host = np.array([np.linalg.norm(ref.hx(psi[k], 0) - eig[k] * psi[k]) for k in range(20)])
    np.testing.assert_allclose(info["resid"], host, rtol=1e-6, atol=1e-14)
    assert info["resid"].max() < 1e-3
    # the Ritz vectors (basis x eigenvectors, an FP64 product on the digit
    # engine) are orthonormal and reproduce the eigenvalues to FP64 accuracy
    gram = psi @ psi.T
    assert np.abs(gram - np.eye(len(psi))).max() < 1e-12
    rq = np.array([psi[k] @ ref.hx(psi[k], 0) for k in range(20)])
    np.testing.assert_allclose(rq, eig, rtol=1e-12, atol=0)


def test_pist_mixed_tensor_fp32(lib, orc, c0):
    """The mixed path with the FP32 tensor-core engine (split-BF16 x3 H*X and
    rotations in the inner solves): eigenvalues still equal the exact ones."""
    import scipy.sparse.linalg as sla
    e0 = float(c0.RES.min())
    ref = orc.Operator.from_problem(c0, E0=e0)
    exact = np.sort(sla.eigsh(sla.LinearOperator((c0.N, c0.N), matvec=lambda v: ref.hx(v, 0)),
                              k=20, which="SA", tol=1e-13)[0])
    x0 = orc.start_vector(c0.N, 0)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.set_fp32_mode(capi.FP32_TENSOR)
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, 20, e0, 1e-11, m_max=400, qmr_max=500, qmr_tol=1e-4,
                                      precision=capi.PREC_FP32, orth=2)
    assert st > 0
    assert np.abs(eig - exact).max() * hm.HARTREE_CM < CM_TOL
