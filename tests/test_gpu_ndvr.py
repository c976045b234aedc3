"""The sNDVR form on the GPU: the outermost layer as per-point matrices OUTH
(H3X, src/libutil/serial/base/matrix.f90:188-203), through the whole-operator
path -- MYHX (osb.hx.h:71-110) with H3X as its last level, the block-Jacobi
build whose outer blocks are OUTH itself (myDiagInit, osb.diag.h:19-30), P*X,
QMR and PIST -- against the oracle and the explicit matrix.
"""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

CM_TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def case(sizes=(12, 10, 8)):
    p = hm.build_problem(hm.Grid3(*sizes), hm.PES())
    return hm.ndvr_problem(p, coupling=2e-4, seed=3)


def oracle_op(orc, q, e0):
    return orc.Operator(q.sizes, q.dep, q.H0, q.RES, None, E0=e0, ndvr=True, OUTH=q.OUTH)


def context(q, e0):
    ctx = capi.Context(q.sizes, q.dep, ndvr=True)
    ctx.load(q.H0, q.RES, None, q.OUTH)
    ctx.set_shift(e0)
    return ctx


@pytest.mark.parametrize("mode", [capi.FP64_TENSOR, capi.FP64_DFMA])
def test_ndvr_hx(lib, orc, mode):
    q = case()
    H = hm.dense_ndvr(q)
    e0 = 0.004
    ref = oracle_op(orc, q, e0)
    X = np.random.default_rng(0).standard_normal((4, q.N))
    with context(q, e0) as ctx:
        ctx.set_fp64_mode(mode)
        for ntype in (capi.TA0, capi.TA1):
            Y = ctx.hx(X, ntype)
            for v in range(X.shape[0]):
                want = ref.hx(X[v], ntype)
                assert rel(Y[v], want) < 1e-12
                dense = H @ X[v] - (e0 * X[v] if ntype == capi.TA1 else 0.0)
                assert rel(Y[v], dense) < 1e-12


def test_ndvr_hx_fp32(lib, orc):
    import torch
    q = case()
    ref = oracle_op(orc, q, 0.0)
    x = np.random.default_rng(1).standard_normal(q.N)
    with context(q, 0.0) as ctx:
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dy = torch.empty_like(dx)
        ctx.hx_f32_device(dx, dy, 1, capi.TA0)
        torch.cuda.synchronize()
        assert rel(dy.double().cpu().numpy(), ref.hx(x, 0)) < 2e-6


def test_ndvr_build_px_qmr(lib, orc):
    q = case()
    e0 = 0.0045
    ref = oracle_op(orc, q, e0)
    st_ref = ref.build_osb(20, 1e-4)
    x = np.random.default_rng(2).standard_normal(q.N)
    with context(q, e0) as ctx:
        st = ctx.build_osb(20, 1e-4)
        V, E = ctx.get_osb()
        z = ctx.px(x)
        code, X, res, it = ctx.qmr(x, 300, 1e-9)
    assert rel(E, ref.EIG0) < 1e-11
    assert rel(V, ref.VOSB) < 1e-9
    np.testing.assert_array_equal(st[:, 4], st_ref[:, 4])
    assert rel(z, ref.px(x)) < 1e-9
    code_r, X_r, _, _ = ref.qmr(x, 300, 1e-9)
    assert code > 0 and abs(code - code_r) <= 1
    assert rel(X, X_r) < 1e-7


@pytest.mark.parametrize("prec,orth", [(capi.PREC_FP64, 1), (capi.PREC_FP32, 2)])
def test_ndvr_pist(lib, orc, prec, orth):
    """20 lowest levels of the sNDVR problem: the oracle's PIST, the dense
    eigenvalues and the device PIST (FP64 and mixed inner solves) agree."""
    q = case()
    exact = np.linalg.eigvalsh(hm.dense_ndvr(q))[:20]
    e0 = float(exact[0]) - 1e-4
    ref = oracle_op(orc, q, e0)
    ref.build_osb(20, 1e-4)
    x0 = orc.start_vector(q.N, 0)

    def lin(v):
        rc, X, _, _ = ref.qmr(v, 500, 1e-4)
        return rc, X

    st_r, eig_r, _, _ = orc.pist_conv(e0, 1e-11, 0, x0, 40, 5, 1, 20, 400, lambda v: ref.hx(v, 0), lin, orth=1)
    assert st_r > 0
    assert np.abs(eig_r - exact).max() * hm.HARTREE_CM < CM_TOL
    with context(q, e0) as ctx:
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, 20, e0, 1e-11, m_max=400, qmr_max=500, qmr_tol=1e-4,
                                      precision=prec, orth=orth)
    assert st > 0
    assert np.abs(eig - eig_r).max() * hm.HARTREE_CM < CM_TOL
    assert np.abs(eig - exact).max() * hm.HARTREE_CM < CM_TOL
