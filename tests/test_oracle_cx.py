"""The oracle's complex (absorbing-potential) forms against dense complex algebra (CPU).

MYHX_DX (src/iterate/module/osb.hxdx.h:178-240), MYPX_DX
(src/iterate/module/osb.mypxdx.h), QMR_CX
(src/iterate/libiterate/qmr/qmrcx.f90:4-175) and PIST_CONV_SX
(src/iterate/libiterate/pist/pist_sx.f90:4-96) carry no known answers in the
reference; the restatement is pinned to its definition: H*X is the dense
(H - E0 +- i A) X, P*X is V diag(1/(kernel)) V^T X, QMR_CX recovers a known
solution of a complex symmetric system (the pattern of the reference's real
QMR driver, qmr.drv.f90:24-47), and PIST_CONV_SX returns the eigenvalues
ZGEEV gives for the dense operator.
"""
import numpy as np
import pytest

from scalit_gb300 import hamiltonian as hm


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def cxcase(orc):
    p = hm.build_problem(hm.Grid3(6, 7, 5), hm.PES())
    op = orc.Operator.from_problem(p, E0=0.0)
    op.build_osb(30, 1e-12)
    e0 = float(np.sort(op.EIG0)[10]) + 2e-4
    op.set_e0(e0)
    rng = np.random.default_rng(0)
    app = rng.uniform(0.0, 2e-3, p.N)
    apr = rng.uniform(0.0, 1e-3, p.N)
    cx = orc.CxOperator(op, app, apr)
    sizes = op.sizes
    vs = orc.vosb_starts(sizes)
    dims = np.cumprod((1,) + sizes[:-1])
    V = np.zeros((op.N, op.N))
    for j in range(op.N):
        y = np.zeros(op.N)
        y[j] = 1.0
        for l, n in enumerate(sizes):
            blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
            y = orc.vx(int(dims[l]), n, blk, op.VOSB[vs[l]:vs[l] + blk * n * n], y)
        V[:, j] = y
    H = hm.dense_hamiltonian(p, shift=0.0)
    return p, op, cx, V, H, e0


ALL = [0, 1, 2, 3, 100, 101, 102, 200, 201, 202]


@pytest.mark.parametrize("ntype", ALL)
def test_cx_hx_is_dense(orc, cxcase, ntype):
    p, op, cx, V, H, e0 = cxcase
    use_e0, sign, which = orc.cx_terms(ntype)
    A = {"AP": cx.AP, "APP": cx.APP, "APR": cx.APR}.get(which, np.zeros(p.N))
    M = H - (e0 if use_e0 else 0.0) * np.eye(p.N) + 1j * sign * np.diag(A)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(p.N) + 1j * rng.standard_normal(p.N)
    assert rel(cx.hx(x, ntype), M @ x) < 1e-14
    np.testing.assert_allclose(cx.AP, cx.APP + cx.APR, rtol=0, atol=0)


@pytest.mark.parametrize("nosb,ntype", [(1, 1), (1, 0), (1, 2), (1, 100), (1, 201), (2, 102), (3, 200), (3, 1)])
def test_cx_px_is_dense(orc, cxcase, nosb, ntype):
    p, op, cx, V, H, e0 = cxcase
    de, beta = 3e-3, 0.5
    use_e0, sign, which = orc.cx_terms(ntype)
    A = {"AP": cx.AP, "APP": cx.APP, "APR": cx.APR}.get(which, np.zeros(p.N))
    shift = 0.0 if ntype in (0, 2, 3) else e0
    ade = op.EIG0 - shift
    inside = np.abs(ade) <= de
    if nosb == 2:
        ade = np.where(inside, np.sign(ade) * de + (ade == 0) * de, ade)
    elif nosb == 3:
        ade = np.where(inside, -beta * de + (1 + beta) * ade, ade)
    kern = 1.0 / (ade + 1j * sign * A)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(p.N) + 1j * rng.standard_normal(p.N)
    got = cx.px(x, nosb=nosb, ntype=ntype, de=de, beta=beta)
    assert rel(got, V @ (kern * (V.T @ x))) < 1e-12


def test_cx_qmr_known_solution(orc):
    """A complex symmetric matrix H + i diag(a) with the Jacobi preconditioner:
    the solution x0(i) = i is recovered."""
    rng = np.random.default_rng(3)
    n = 80
    a = rng.standard_normal((n, n))
    H = (a + a.T) / 2 + np.diag(np.arange(n) * 0.5 + 5.0)
    M = H + 1j * np.diag(rng.uniform(0.1, 1.0, n))
    x0 = np.arange(1, n + 1).astype(np.complex128)
    b = M @ x0
    d = np.diag(M)
    code, x, res = orc.qmr_cx(lambda v: M @ v, lambda v: v / d, b, 500, 1e-12)
    assert code > 0 and res < 1e-12
    assert rel(x, x0) < 1e-9


@pytest.mark.parametrize("nosb", [1, 2])
def test_cx_qmr_on_the_osb_operator(orc, cxcase, nosb):
    """(H - E0 + i AP) x = b through the complex OSB preconditioner (TAAP)."""
    p, op, cx, V, H, e0 = cxcase
    M = H - e0 * np.eye(p.N) + 1j * np.diag(cx.AP)
    b = np.random.default_rng(4).standard_normal(p.N) + 0j
    code, x, res = orc.qmr_cx(lambda v: cx.hx(v, orc.TAAP),
                              lambda v: cx.px(v, nosb=nosb, ntype=orc.TAAP, de=3e-3), b, 500, 1e-10)
    assert code > 0
    assert rel(M @ x, b) < 1e-8


def test_get_op_cx_and_window(orc):
    z = np.array([1 - 2j, -3 + 0.5j, 0.25 + 0.25j])
    np.testing.assert_array_equal(orc.get_op_cx(1, z), z.real)
    np.testing.assert_array_equal(orc.get_op_cx(6, z), z.real ** 2 + z.imag ** 2)
    np.testing.assert_array_equal(orc.get_op_cx(11, z), np.abs(z.imag - z.real))
    np.testing.assert_array_equal(orc.get_window_cx(0.3, 1, z, 2), z[[2, 0]])
    np.testing.assert_array_equal(orc.reorder_cx(1, z), z[[1, 2, 0]])


def test_pist_sx_dense_known_answer(orc):
    """PIST_CONV_SX with exact shift-and-invert solves on a complex symmetric
    matrix returns its eigenvalues nearest E0 (by the real part), as ZGEEV does."""
    rng = np.random.default_rng(5)
    n = 60
    a = rng.standard_normal((n, n))
    M = (a + a.T) / 2 + np.diag(np.linspace(0.0, 6.0, n)) - 1j * np.diag(rng.uniform(0.01, 0.1, n))
    E0 = 3.0
    exact = np.linalg.eigvals(M)
    want = np.sort_complex(exact[np.argsort(np.abs(exact.real - E0))[:5]])
    inv = np.linalg.inv(M - E0 * np.eye(n))
    x0 = rng.random(n) + 0j
    st, eig, res = orc.pist_conv_sx(E0, 1e-12, 0, x0, 0, 5, 1, 5, n, lambda v: M @ v, lambda v: (1, inv @ v))
    assert st > 0 and res <= 1e-12
    np.testing.assert_allclose(eig[np.argsort(eig.real)], want[np.argsort(want.real)], atol=1e-9)
    with pytest.raises(ValueError):
        orc.pist_conv_sx(E0, 1e-12, 1, x0, 0, 5, 1, 5, n, lambda v: M @ v, lambda v: (1, inv @ v))


def test_pist_sx_on_the_osb_operator(orc, cxcase):
    """Complex levels of H - i AP nearest E0 through QMR_CX solves with the
    complex OSB preconditioner (TMAP) against the dense eigenvalues."""
    p, op, cx, V, H, e0 = cxcase
    Heff = H - 1j * np.diag(cx.AP)
    exact = np.linalg.eigvals(Heff)
    want = exact[np.argsort(np.abs(exact.real - e0))[:6]]

    def linsolv(v):
        code, x, _ = orc.qmr_cx(lambda u: cx.hx(u, orc.TMAP), lambda u: cx.px(u, 1, orc.TMAP), v, 500, 1e-12)
        return code, x

    x0 = np.random.default_rng(6).random(p.N) + 0j
    st, eig, res = orc.pist_conv_sx(e0, 1e-11, 0, x0, 0, 5, 1, 6, 150, lambda v: cx.hx(v, orc.TMAP0), linsolv)
    assert st > 0
    np.testing.assert_allclose(np.sort(eig.real), np.sort(want.real), atol=1e-8)
    np.testing.assert_allclose(eig.imag[np.argsort(eig.real)], want.imag[np.argsort(want.real)], atol=1e-8)


def test_lan_dx_hermitian(orc):
    """LAN_DX on a Hermitian matrix: n steps give its whole spectrum."""
    rng = np.random.default_rng(7)
    n = 30
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = (a + a.conj().T) / 2
    st, eig = orc.lan_dx(rng.random(n) + 1j * rng.random(n), n, lambda v: A @ v)
    assert st == n
    np.testing.assert_allclose(np.sort(eig), np.linalg.eigvalsh(A), atol=1e-10)


def test_crp_equals_dense_trace(orc, cxcase):
    """With APR on r points the CRP operator has rank <= r, so r + 1 Lanczos
    steps give its trace: N(E) = 4 Tr[sqrt(APR) G+ APP G- sqrt(APR)]."""
    p, op, cx0, V, H, e0 = cxcase
    rng = np.random.default_rng(8)
    apr = np.zeros(p.N)
    pts = rng.choice(p.N, 12, replace=False)
    apr[pts] = rng.uniform(1e-3, 3e-3, 12)
    app = np.where(apr == 0.0, rng.uniform(0.0, 2e-3, p.N), 0.0)
    cx = orc.CxOperator(op, app, apr)
    E = e0
    G = lambda s: np.linalg.inv(H - E * np.eye(p.N) + s * 1j * np.diag(cx.AP))
    sq = np.diag(np.sqrt(apr))
    dense = 4.0 * np.real(np.trace(sq @ G(1) @ np.diag(app) @ G(-1) @ sq))
    x0 = rng.random(p.N) + 1j * rng.random(p.N)
    got = orc.osb_crp(cx, [E], 13, [x0], 1000, 1e-13)[0]
    assert dense > 0.0
    assert abs(got - dense) / dense < 1e-6


@pytest.mark.parametrize("ntype", [1, 0, 2, 100, 201])
def test_cx_window_px_is_dense(orc, cxcase, ntype):
    """MYPX_DX with TOSBW: the window block of the kernel is the inverse of
    HW - E0 +- i A(WIND) (createWH_DXCX), the rest 1/(EIG0 - E0 +- i A)."""
    p, op, cx, V, H, e0 = cxcase
    win = orc.OSBW(op, e0, 20, 1e-4)
    use_e0, sign, which = orc.cx_terms(ntype)
    A = {"AP": cx.AP, "APP": cx.APP, "APR": cx.APR}.get(which, np.zeros(p.N))
    shift = 0.0 if ntype in (0, 2, 3) else e0
    M = np.diag(1.0 / (op.EIG0 - shift + 1j * sign * A))
    Wm = win.HW - shift * np.eye(20) + 1j * sign * np.diag(A[win.ind])
    M[np.ix_(win.ind, win.ind)] = np.linalg.inv(Wm)
    x = np.random.default_rng(11).standard_normal(p.N) + 1j * np.random.default_rng(12).standard_normal(p.N)
    got = cx.px(x, nosb=orc.TOSBW, ntype=ntype, win=win)
    assert rel(got, V @ M @ V.T @ x) < 1e-10


def test_pist_cx_conjugate_dense(orc):
    """PIST_CONV_CX (the conjugate product) returns the same eigenvalues of a
    non-Hermitian matrix as ZGEEV, with exact shift-and-invert solves."""
    rng = np.random.default_rng(16)
    n = 50
    a = rng.standard_normal((n, n))
    M = (a + a.T) / 2 + np.diag(np.linspace(0.0, 5.0, n)) - 1j * np.diag(rng.uniform(0.01, 0.1, n))
    E0 = 2.5
    exact = np.linalg.eigvals(M)
    want = exact[np.argsort(np.abs(exact.real - E0))[:4]]
    want = want[np.argsort(want.real)]
    inv = np.linalg.inv(M - E0 * np.eye(n))
    x0 = rng.random(n) + 1j * rng.random(n)
    st, eig, res = orc.pist_conv_sx(E0, 1e-12, 0, x0, 0, 5, 1, 4, n, lambda v: M @ v, lambda v: (1, inv @ v),
                                    conj=True)
    assert st > 0
    np.testing.assert_allclose(eig, want, atol=1e-9)


def _complex_hamiltonian(p, seed):
    """Complex symmetric level matrices K_l + i S_l (small symmetric S_l),
    complex DEP factors, for the complex-Hamiltonian job (sCX)."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, n in enumerate(p.sizes):
        K = p.level_matrix(l + 1)
        S = rng.standard_normal((n, n)) * 1e-4
        parts.append((K + 1j * (S + S.T)).ravel(order="F"))
    H0CX = np.concatenate(parts)
    DEPCX = p.DEP * (1.0 + 1j * rng.uniform(-0.05, 0.05, p.DEP.size))
    return H0CX, DEPCX


def _dense_cx(p, H0CX, DEPCX, RES, shift=0.0):
    sizes = p.sizes
    N = int(np.prod(sizes))
    H = np.diag(RES - shift).astype(np.complex128)
    h0, dp = 0, 0
    for l, n in enumerate(sizes):
        nin = int(np.prod(sizes[:l], dtype=np.int64))
        blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
        Hl = H0CX[h0:h0 + n * n].reshape((n, n), order="F")
        h0 += n * n
        if p.dep[l]:
            D = np.diag(DEPCX[dp:dp + nin])
            dp += nin
        else:
            D = np.eye(nin)
        H = H + np.kron(np.eye(blk), np.kron(Hl, D))
    assert H.shape == (N, N)
    return H


@pytest.mark.parametrize("ntype", [0, 1, 201])
def test_cx_hamiltonian_hx_is_dense(orc, ntype):
    """MYHX_CX (osb.hxcx.h:191-261) with complex level matrices and DEP: the
    oracle's level sum equals the dense complex Kronecker sum."""
    p = hm.build_problem(hm.Grid3(6, 5, 4), hm.PES())
    op = orc.Operator.from_problem(p, E0=1e-3)
    app = np.random.default_rng(1).uniform(0.0, 2e-3, p.N)
    cx = orc.CxOperator(op, app)
    H0CX, DEPCX = _complex_hamiltonian(p, 2)
    cx.set_complex_h0(H0CX, DEPCX)
    shift = op.E0 if ntype != 0 else 0.0
    H = _dense_cx(p, H0CX, DEPCX, p.RES, shift)
    if ntype == 201:                                   # TMAP: H - i AP - E0
        H = H - 1j * np.diag(app)
    x = np.random.default_rng(3).standard_normal(p.N) + 1j * np.random.default_rng(4).standard_normal(p.N)
    assert rel(cx.hx(x, ntype), H @ x) < 1e-13
