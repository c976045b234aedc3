"""The oracle pinned against the reference's known-answer test patterns and
independent mathematics (no GPU).

* QMR recovers x0(i) = i for a random symmetric 23x23 H with the Jacobi
  preconditioner (src/iterate/libiterate/qmr/testing/qmr.drv.f90:7-51).
* PIST eigenvalues near E0 equal a direct dense eigen-solve of a random
  symmetric 100x100 matrix (src/iterate/libiterate/pist/testing/pist.drv.f90).
* MYHX equals the explicit Kronecker-sum Hamiltonian.
* With one level the block-Jacobi build is an exact eigen-decomposition.
"""
import numpy as np
import pytest

from scalit_gb300 import hamiltonian as hm


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_qmr_known_solution(orc):
    rng = np.random.default_rng(0)
    n = 23
    a = rng.random((n, n))
    H = np.tril(a) + np.tril(a, -1).T + n * np.eye(n)   # diagonally dominant like the driver's intent
    x0 = np.arange(1, n + 1, dtype=np.float64)
    b = H @ x0
    code, x, res = orc.qmr_dense(H, b, 1000, 1e-12, ntype=0)
    assert code > 0
    assert np.max(np.abs((x0 - x) / x0)) < 1e-10


def test_qmr_serial_and_mpi_breakdown_codes(orc):
    H = np.eye(5)
    code, x, res = orc.qmr_dense(H, np.zeros(5), 10, 1e-8, ntype=0, mpi_codes=False)
    assert code == 0                        # serial QMR leaves 0 (qmr.f90:57)
    code, x, res = orc.qmr_dense(H, np.zeros(5), 10, 1e-8, ntype=0, mpi_codes=True)
    assert code == -1                       # QMR_MPI (qmr_mpi.f90:82-85)


def test_pist_dense_known_answer(orc):
    rng = np.random.default_rng(1)
    n = 100
    a = rng.standard_normal((n, n))
    H = (a + a.T) / 2
    E0, M = 0.0, 6
    exact = np.linalg.eigvalsh(H)
    Hs = H - E0 * np.eye(n)

    def linsolv(v):
        return 1, np.linalg.solve(Hs, v)

    st, eig, res, info = orc.pist_conv(E0, 1e-12, 0, rng.random(n), 12, 5, 1, M, 100,
                                       lambda v: H @ v, linsolv)
    assert st > 0
    near = np.sort(exact[np.argsort(np.abs(exact - E0))[:M]])
    np.testing.assert_allclose(eig, near, atol=1e-10)


def test_myhx_equals_dense(orc):
    p = hm.build_problem(hm.Grid3(6, 7, 5), hm.PES())
    H = hm.dense_hamiltonian(p, shift=0.01)
    op = orc.Operator.from_problem(p, E0=0.01)
    x = np.random.default_rng(2).standard_normal(p.N)
    assert rel(op.hx(x, 1), H @ x) < 1e-14
    assert rel(op.hx(x, 0), (H + 0.01 * np.eye(p.N)) @ x) < 1e-14


def test_one_level_build_is_exact(orc):
    rng = np.random.default_rng(3)
    n = 30
    a = rng.standard_normal((n, n))
    H1 = (a + a.T) / 2
    res = rng.standard_normal(n)
    op = orc.Operator((n,), (False,), H1.ravel(order="F"), res, None, E0=-20.0)
    op.build_osb(50, 1e-14)
    np.testing.assert_allclose(np.sort(op.EIG0), np.linalg.eigvalsh(H1 + np.diag(res)), atol=1e-12)
    x = rng.standard_normal(n)
    assert rel(op.px(op.hx(x, 1)), x) < 1e-11


def test_vx_vtx_are_inverse(orc):
    rng = np.random.default_rng(4)
    nin, nout, blk = 3, 5, 4
    V = np.concatenate([np.linalg.qr(rng.standard_normal((nout, nout)))[0].ravel(order="F")
                        for _ in range(blk)])
    x = rng.standard_normal(nin * nout * blk)
    assert rel(orc.vx(nin, nout, blk, V, orc.vtx(nin, nout, blk, V, x)), x) < 1e-14


def test_h1x_layout(orc):
    """H1X_XYZ: Y(a, i, b) = sum_j H(i, j) X(a, j, b) in column-major order."""
    rng = np.random.default_rng(5)
    nin, nout, blk = 3, 4, 2
    H = rng.standard_normal((nout, nout))
    X = rng.standard_normal((nin, nout, blk))
    Y = orc.h1x_xyz(nin, nout, blk, H.ravel(order="F"), X.ravel(order="F"))
    np.testing.assert_allclose(Y.reshape((nin, nout, blk), order="F"),
                               np.einsum("ij,ajb->aib", H, X), rtol=1e-14, atol=1e-14)
    c = rng.uniform(1, 2, nin)
    Yd = orc.h1x_dep(nin, nout, blk, H.ravel(order="F"), c, X.ravel(order="F"))
    np.testing.assert_allclose(Yd.reshape((nin, nout, blk), order="F"),
                               c[:, None, None] * np.einsum("ij,ajb->aib", H, X), rtol=1e-13)


def test_oracle_pist_c0_levels(orc):
    """20 lowest levels of the 24x32x20 problem against ARPACK (1e-4 cm^-1)."""
    import scipy.sparse.linalg as sla
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min())
    op = orc.Operator.from_problem(p, E0=e0)
    op.build_osb(20, 1e-4)

    def linsolv(v):
        rc, X, _, _ = op.qmr(v, 500, 1e-4)
        return rc, X

    st, eig, res, info = orc.pist_conv(e0, 1e-11, 0, orc.start_vector(p.N, 0), 40, 5, 1, 20, 400,
                                       lambda v: op.hx(v, 0), linsolv)
    assert st > 0
    ex = np.sort(sla.eigsh(sla.LinearOperator((p.N, p.N), matvec=lambda v: op.hx(v, 0)),
                           k=20, which="SA", tol=1e-13)[0])
    assert np.abs(eig - ex).max() * hm.HARTREE_CM < 1e-4


def test_window_and_convergence_helpers(orc):
    v = np.array([5.0, -1.0, 2.0, 2.0, 0.5])
    np.testing.assert_array_equal(orc.get_window(1.0, v, 3), [0.5, 2.0, 2.0])
    assert orc.get_diff_max([1, 2, 3], [1, 2.5, 2]) == 1.0
    assert orc.get_sep_max([0.0, 1.0], [0.1, 0.95, 3.0]) == pytest.approx(0.1)
    p = orc.pist_params(20, (0.0, 1e-8, 0, 0, 0, 20, 0))
    assert (p["startcnt"], p["stepcnt"], p["stepeig"], p["m_max"]) == (40, 5, 1, 60)


def test_oracle_ndvr_matches_dense(orc):
    """The oracle's sNDVR path (H3X as the outer level, OUTH as the outer
    block-Jacobi blocks) equals the explicit matrix, and one more level of the
    same Hamiltonian in per-point form changes nothing when the coupling is 0."""
    from scalit_gb300 import hamiltonian as hm
    p = hm.build_problem(hm.Grid3(8, 7, 6), hm.PES())
    q0 = hm.ndvr_problem(p, coupling=0.0)
    H0 = hm.dense_ndvr(q0)
    assert np.abs(H0 - hm.dense_hamiltonian(p)).max() < 1e-15
    q = hm.ndvr_problem(p, coupling=2e-4, seed=3)
    op = orc.Operator(q.sizes, q.dep, q.H0, q.RES, None, E0=0.0, ndvr=True, OUTH=q.OUTH)
    x = np.random.default_rng(4).standard_normal(q.N)
    H = hm.dense_ndvr(q)
    assert np.linalg.norm(op.hx(x, 0) - H @ x) / np.linalg.norm(H @ x) < 1e-14
    # the build's outer blocks are OUTH: with one level left, P*X is (H - E0)^-1 on it
    op.build_osb(50, 1e-14)
    assert np.all(np.isfinite(op.EIG0))
