"""Differentiation: adjoint H*X (with respect to X, the potential grid and the
kinetic matrices) and Hellmann-Feynman eigenvalue gradients, checked against
dense FP64 references and central finite differences (relative step 1e-6).
A torch.autograd.Function wraps the adjoint for the gradcheck (test harness only)."""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_adjoint_against_dense(lib):
    p = hm.build_problem(hm.Grid3(7, 6, 5), hm.PES())
    rng = np.random.default_rng(0)
    x, yb = rng.standard_normal(p.N), rng.standard_normal(p.N)
    n_r, n_R, n_t = p.sizes
    Kr, KR, Kt = (p.level_matrix(l) for l in (1, 2, 3))
    X = x.reshape(p.sizes, order="F")
    Yb = yb.reshape(p.sizes, order="F")
    c = p.DEP.reshape(n_r, n_R, order="F")
    with capi.Context.from_problem(p, e0=0.01) as ctx:
        xb, vb, hb = ctx.hx_adjoint(x, yb, capi.TA1)
        y = ctx.hx(x, capi.TA1)
    H = hm.dense_hamiltonian(p, shift=0.01)
    assert rel(xb, H.T @ yb) < 1e-13
    np.testing.assert_allclose(vb, yb * x, rtol=1e-14)
    gKr = np.einsum("ibt,jbt->ij", Yb, X)
    gKR = np.einsum("aib,ajb->ij", Yb, X)
    gKt = np.einsum("ab,abi,abj->ij", c, Yb, X)
    off = [0, n_r ** 2, n_r ** 2 + n_R ** 2]
    assert rel(hb[off[0]:off[1]].reshape(n_r, n_r, order="F"), gKr) < 1e-13
    assert rel(hb[off[1]:off[2]].reshape(n_R, n_R, order="F"), gKR) < 1e-13
    assert rel(hb[off[2]:].reshape(n_t, n_t, order="F"), gKt) < 1e-13
    # <Ybar, H X> = <H^T Ybar, X>
    assert abs(yb @ y - xb @ x) < 1e-12 * abs(yb @ y)


def test_adjoint_f32(lib):
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-24x32x20")
    rng = np.random.default_rng(1)
    x, yb = rng.standard_normal(p.N), rng.standard_normal(p.N)
    with capi.Context.from_problem(p, e0=0.0) as ctx:
        xb64, vb64, hb64 = ctx.hx_adjoint(x, yb)
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dy = torch.tensor(yb, dtype=torch.float32, device="cuda")
        dxb, dvb = torch.empty_like(dx), torch.empty_like(dx)
        dhb = torch.empty(hb64.size, dtype=torch.float32, device="cuda")
        ctx.hx_adjoint_device(dx, dy, dxb, dvb, dhb, f32=True)
        torch.cuda.ExternalStream(ctx.stream).synchronize()
    assert rel(dxb.double().cpu().numpy(), xb64) < 2e-6
    assert rel(dvb.double().cpu().numpy(), vb64) < 1e-6
    assert rel(dhb.double().cpu().numpy(), hb64) < 1e-4


def test_autograd_gradcheck(lib):
    """torch.autograd.Function over the C ABI, gradcheck in FP64."""
    torch = pytest.importorskip("torch")
    p = hm.build_problem(hm.Grid3(5, 4, 3), hm.PES())
    ctx = capi.Context.from_problem(p, e0=0.0)

    class HX(torch.autograd.Function):
        @staticmethod
        def forward(fctx, x):
            fctx.save_for_backward(x)
            return torch.from_numpy(ctx.hx(x.detach().numpy(), capi.TA1))

        @staticmethod
        def backward(fctx, g):
            (x,) = fctx.saved_tensors
            xb, _, _ = ctx.hx_adjoint(x.detach().numpy(), g.detach().numpy(), want=("x",))
            return torch.from_numpy(xb)

    x = torch.randn(p.N, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(HX.apply, (x,), eps=1e-6, atol=1e-8, rtol=1e-6)
    ctx.close()


def test_hellmann_feynman_vs_finite_differences(lib):
    """dE_k/dp for the lowest levels of a small problem: Hellmann-Feynman with
    the PIST Ritz vectors against central differences of PIST eigenvalues."""
    grid = hm.Grid3(16, 20, 12)
    pes = hm.PES(amp1=0.001, amp3=0.0005, width1=1.2, width3=0.8)
    M = 6
    p = hm.build_problem(grid, pes)
    r, R, cth = p.grids["r"], p.grids["R"], p.grids["cos_theta"]
    dv = hm.potential_grad(r[:, None, None], R[None, :, None], cth[None, None, :], pes)
    dvdp = np.stack([np.ascontiguousarray(g).ravel(order="F") for g in dv])
    x0 = np.random.default_rng(0).random(p.N)

    def levels(pp, vectors=False):
        prob = hm.build_problem(grid, pp)
        e0 = float(prob.RES.min())
        with capi.Context.from_problem(prob, e0=e0) as ctx:
            ctx.build_osb(20, 1e-4)
            st, eig, res, info = ctx.pist(x0, M, e0, 1e-12, m_max=400, qmr_max=500, qmr_tol=1e-6,
                                          vectors=vectors)
            assert st > 0
            g = ctx.hf_gradients(info["vectors"], dvdp) if vectors else None
        return eig, g

    eig0, g = levels(pes, vectors=True)
    base = pes.params()
    for j in (0, 1, 3, 4, 6, 7):   # Morse depths / ranges and the P1, P2 amplitudes
        h = 1e-6 * max(abs(base[j]), 1.0)
        pp, pm = base.copy(), base.copy()
        pp[j] += h
        pm[j] -= h
        fd = (levels(pes.with_params(pp))[0] - levels(pes.with_params(pm))[0]) / (2 * h)
        np.testing.assert_allclose(g[:, j], fd, rtol=2e-3, atol=2e-7)


@pytest.mark.slow
def test_differentiation_form_128x128x96(lib, orc):
    """The differentiation workload at its stated size (1,572,864 points).

    Adjoint H*X with respect to X, the V grid and K_R, K_r, K_theta in FP64
    against the FP64 CPU reference gradient (the oracle's H applied to Ybar,
    Ybar * X, and the contractions of Ybar with X per level), and in FP32
    against the FP64 result; then Hellmann-Feynman dE_k/dp for the 50 lowest
    levels and all 12 PES parameters against central differences of the
    levels with relative step 1e-6 (levels taken to an FP64 residual of 1e-9
    Eh, so their error, ~r^2/gap, is far below the differences)."""
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-128x128x96")
    n_r, n_R, n_t = p.sizes
    rng = np.random.default_rng(12)
    x, yb = rng.standard_normal(p.N), rng.standard_normal(p.N)
    e0 = float(p.RES.min())
    ref = orc.Operator.from_problem(p, E0=e0)
    X = x.reshape(p.sizes, order="F")
    Yb = yb.reshape(p.sizes, order="F")
    c = p.DEP.reshape(n_r, n_R, order="F")
    with capi.Context.from_problem(p, e0=e0) as ctx:
        xb, vb, hb = ctx.hx_adjoint(x, yb, capi.TA1)
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dy = torch.tensor(yb, dtype=torch.float32, device="cuda")
        dxb, dvb = torch.empty_like(dx), torch.empty_like(dx)
        dhb = torch.empty(hb.size, dtype=torch.float32, device="cuda")
        ctx.hx_adjoint_device(dx, dy, dxb, dvb, dhb, f32=True)
        torch.cuda.ExternalStream(ctx.stream).synchronize()
    assert rel(xb, ref.hx(yb, 1)) < 1e-12           # H - E0 is symmetric: Xbar = (H - E0) Ybar
    np.testing.assert_allclose(vb, yb * x, rtol=1e-14)
    off = [0, n_r ** 2, n_r ** 2 + n_R ** 2]
    gKr = np.einsum("ibt,jbt->ij", Yb, X)
    gKR = np.einsum("aib,ajb->ij", Yb, X)
    gKt = np.einsum("ab,abi,abj->ij", c, Yb, X)
    assert rel(hb[off[0]:off[1]].reshape(n_r, n_r, order="F"), gKr) < 1e-12
    assert rel(hb[off[1]:off[2]].reshape(n_R, n_R, order="F"), gKR) < 1e-12
    assert rel(hb[off[2]:].reshape(n_t, n_t, order="F"), gKt) < 1e-12
    assert rel(dxb.double().cpu().numpy(), xb) < 2e-6
    assert rel(dvb.double().cpu().numpy(), vb) < 1e-6
    assert rel(dhb.double().cpu().numpy(), hb) < 1e-4

    # Hellmann-Feynman, 50 levels x 12 parameters
    M = 50
    grid, pes = hm.WORKLOADS["tri-128x128x96"]
    rr, RR, cth = p.grids["r"], p.grids["R"], p.grids["cos_theta"]
    dv = hm.potential_grad(rr[:, None, None], RR[None, :, None], cth[None, None, :], pes)
    dvdp = np.stack([np.ascontiguousarray(g).ravel(order="F") for g in dv])
    x0 = np.random.default_rng(0).random(p.N)

    def levels(pp, vectors=False):
        prob = hm.build_problem(grid, pp)
        with capi.Context.from_problem(prob, e0=e0) as cx:
            cx.build_osb(20, 1e-4)
            st, eig, _, info = cx.pist(x0, M, e0, 1e-12, m_max=800, qmr_max=2000, qmr_tol=1e-7,
                                       refine_tol=1e-9, refine_steps=20, vectors=vectors)
            assert st > 0 and np.max(info["resid"]) <= 1e-9
            g = cx.hf_gradients(info["vectors"], dvdp) if vectors else None
        return eig, g

    eig0, g = levels(pes, vectors=True)
    base = pes.params()
    worst = 0.0
    for j in range(12):
        h = 1e-6 * abs(base[j])
        pp, pm = base.copy(), base.copy()
        pp[j] += h
        pm[j] -= h
        fd = (levels(pes.with_params(pp))[0] - levels(pes.with_params(pm))[0]) / (2 * h)
        err = np.abs(g[:, j] - fd) / (np.abs(fd) + 1e-6 * np.abs(fd).max() + 1e-12)
        worst = max(worst, float(err.max()))
        np.testing.assert_allclose(g[:, j], fd, rtol=1e-3, atol=1e-5 * np.abs(fd).max() + 1e-9)
    print(f"HF vs central differences, 50 levels x 12 parameters: worst relative difference {worst:.2e}")
