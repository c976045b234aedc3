"""The oracle's complex (absorbing-potential) forms against dense complex algebra (CPU).

MYHX_DX (src/iterate/module/osb.hxdx.h:178-240), MYPX_DX
(src/iterate/module/osb.mypxdx.h) and QMR_CX
(src/iterate/libiterate/qmr/qmrcx.f90:4-175) carry no known answers in the
reference; the restatement is pinned to its definition: H*X is the dense
(H - E0 +- i A) X, P*X is V diag(1/(kernel)) V^T X, and QMR_CX recovers a
known solution of a complex symmetric system (the pattern of the reference's
real QMR driver, qmr.drv.f90:24-47).
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
