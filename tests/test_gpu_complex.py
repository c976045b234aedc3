"""Complex forms with absorbing potentials on the GPU against the oracle
(MYHX_DX, src/iterate/module/osb.hxdx.h:178-240; MYPX_DX,
src/iterate/module/osb.mypxdx.h; QMR_CX, src/iterate/libiterate/qmr/qmrcx.f90:4-175).

The context takes the oracle's VOSB / EIG0 (set_osb).  Tolerances: complex
H*X 1e-12 norm-wise (the real level products of the FP64 engine, 1e-16, on
both halves); P*X 1e-9 as the real P*X; QMR_CX's solution 1e-7 of the
oracle's and its residual against the dense operator 1e-8.
"""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case(orc):
    p = hm.build_problem(hm.Grid3(12, 10, 8), hm.PES())
    ref = orc.Operator.from_problem(p, E0=0.0)
    ref.build_osb(20, 1e-4)
    e0 = float(np.sort(ref.EIG0)[15]) + 2e-4
    ref.set_e0(e0)
    rng = np.random.default_rng(0)
    app = rng.uniform(0.0, 2e-3, p.N)
    apr = rng.uniform(0.0, 1e-3, p.N)
    return p, ref, e0, app, apr


def context(p, ref, e0, app, apr):
    ctx = capi.Context.from_problem(p, e0=e0)
    ctx.set_osb(ref.VOSB, ref.EIG0)
    ctx.set_absorbing(app, apr)
    return ctx


def cvec(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("ntype", [0, 1, 2, 3, 100, 101, 102, 200, 201, 202])
def test_hx_cx_matches_oracle(lib, orc, case, ntype):
    p, ref, e0, app, apr = case
    cx = orc.CxOperator(ref, app, apr)
    X = cvec(np.random.default_rng(1), (2, p.N))
    with context(p, ref, e0, app, apr) as ctx:
        Y = ctx.hx_cx(X, ntype)
    for v in range(2):
        assert rel(Y[v], cx.hx(X[v], ntype)) < 1e-12


@pytest.mark.parametrize("kind,ntype", [(1, 1), (1, 0), (1, 2), (1, 100), (1, 202), (2, 101), (3, 200)])
def test_px_cx_matches_oracle(lib, orc, case, kind, ntype):
    p, ref, e0, app, apr = case
    cx = orc.CxOperator(ref, app, apr)
    de, beta = 3e-3, 0.5
    x = cvec(np.random.default_rng(2), p.N)
    with context(p, ref, e0, app, apr) as ctx:
        ctx.set_precond(kind, de, beta)
        z = ctx.px_cx(x, ntype)
    assert rel(z, cx.px(x, nosb=kind, ntype=ntype, de=de, beta=beta)) < 1e-9


def test_resonance_job_uses_app_only(lib, orc, case):
    """JOB_RES1/2: APR = 0 and AP = APP."""
    p, ref, e0, app, apr = case
    cx = orc.CxOperator(ref, app)
    x = cvec(np.random.default_rng(3), p.N)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.set_osb(ref.VOSB, ref.EIG0)
        ctx.set_absorbing(app)
        y = ctx.hx_cx(x, capi.TAAP)
        y0 = ctx.hx_cx(x, capi.TAAPR)
    assert rel(y, cx.hx(x, capi.TAAP)) < 1e-12
    assert rel(y0, cx.hx(x, capi.TA1)) < 1e-12        # APR = 0


def test_qmr_cx_matches_oracle(lib, orc, case):
    p, ref, e0, app, apr = case
    cx = orc.CxOperator(ref, app, apr)
    b = cvec(np.random.default_rng(4), p.N)
    code_r, x_r, res_r = orc.qmr_cx(lambda v: cx.hx(v, orc.TAAP), lambda v: cx.px(v, 1, orc.TAAP), b, 500, 1e-10)
    with context(p, ref, e0, app, apr) as ctx:
        ctx.set_fp64_mode(capi.FP64_DFMA)
        code, x, res = ctx.qmr_cx(b, 500, 1e-10, ntype=capi.TAAP)
    assert code_r > 0 and code > 0
    assert abs(code - code_r) <= 1
    assert rel(x, x_r) < 1e-7
    assert rel(cx.hx(x, orc.TAAP), b) < 1e-8


def test_errors(lib, case):
    p, ref, e0, app, apr = case
    x = np.zeros(p.N, dtype=np.complex128)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        with pytest.raises(capi.ScalitError) as e:
            ctx.hx_cx(x, capi.TAAP)                  # no absorbing potential yet
        assert e.value.code == -104
        ctx.set_absorbing(app, apr)
        with pytest.raises(capi.ScalitError) as e:
            ctx.px_cx(x, capi.TAAP)                  # no preconditioner yet
        assert e.value.code == -104
        bad = app.copy()
        bad[3] = np.inf
        with pytest.raises(capi.ScalitError) as e:
            ctx.set_absorbing(bad)
        assert e.value.code == -106


def test_crp_matches_oracle_and_dense_trace(lib, orc, case):
    """osbCRP: with APR on r points, r + 1 Lanczos steps give the trace
    4 Tr[sqrt(APR) G+ APP G- sqrt(APR)] (computed densely here)."""
    p, ref, e0, app0, apr0 = case
    rng = np.random.default_rng(9)
    apr = np.zeros(p.N)
    pts = rng.choice(p.N, 10, replace=False)
    apr[pts] = rng.uniform(1e-3, 3e-3, 10)
    app = np.where(apr == 0.0, rng.uniform(0.0, 2e-3, p.N), 0.0)
    cx = orc.CxOperator(ref, app, apr)
    H = hm.dense_hamiltonian(p, shift=0.0)
    G = lambda s: np.linalg.inv(H - e0 * np.eye(p.N) + s * 1j * np.diag(cx.AP))
    sq = np.diag(np.sqrt(apr))
    dense = 4.0 * np.real(np.trace(sq @ G(1) @ np.diag(app) @ G(-1) @ sq))
    x0 = rng.random(p.N) + 1j * rng.random(p.N)
    with context(p, ref, e0, app, apr) as ctx:
        got = ctx.crp([e0], 11, qmrmax=2000, qmrtol=1e-12, X0=x0[None, :])[0]
    want = orc.osb_crp(cx, [e0], 11, [x0], 2000, 1e-12)[0]
    assert dense > 0.0
    assert abs(got - dense) / dense < 1e-5
    assert abs(got - want) / want < 1e-5


def test_pist_cx_levels_of_h_minus_i_ap(lib, orc, case):
    """PIST_CONV_SX through QMR_CX solves (TMAP) returns the complex levels of
    H - i AP nearest E0: against the dense eigenvalues and the oracle."""
    p, ref, e0, app, apr = case
    cx = orc.CxOperator(ref, app, apr)
    H = hm.dense_hamiltonian(p, shift=0.0)
    exact = np.linalg.eigvals(H - 1j * np.diag(cx.AP))
    want = exact[np.argsort(np.abs(exact.real - e0))[:6]]
    want = want[np.argsort(want.real)]
    x0 = np.random.default_rng(10).random(p.N) + 0j
    with context(p, ref, e0, app, apr) as ctx:
        st, eig, res = ctx.pist_cx(x0, 6, e0, 1e-11, 200, qmrmax=1000, qmrtol=1e-12)
    assert st > 0
    np.testing.assert_allclose(eig.real, want.real, atol=1e-8)
    np.testing.assert_allclose(eig.imag, want.imag, atol=1e-8)

    def linsolv(v):
        code, x, _ = orc.qmr_cx(lambda u: cx.hx(u, orc.TMAP), lambda u: cx.px(u, 1, orc.TMAP), v, 1000, 1e-12)
        return code, x

    st_r, eig_r, _ = orc.pist_conv_sx(e0, 1e-11, 0, x0, 0, 5, 1, 6, 200, lambda v: cx.hx(v, orc.TMAP0), linsolv)
    assert st_r > 0
    np.testing.assert_allclose(eig, eig_r, atol=1e-8)


@pytest.mark.parametrize("ntype", [1, 0, 2, 100, 201])
def test_px_cx_window_matches_oracle(lib, orc, case, ntype):
    """MYPX_DX with TOSBW: the window's complex matrix (createWH_DXCX) inverted
    by LU on the device against the oracle's solve."""
    p, ref, e0, app, apr = case
    cx = orc.CxOperator(ref, app, apr)
    win = orc.OSBW(ref, e0, 30, 1e-4)
    x = cvec(np.random.default_rng(13), p.N)
    with context(p, ref, e0, app, apr) as ctx:
        ctx.build_osbw(e0, 30, 1e-4)
        z = ctx.px_cx(x, ntype)
        z2 = ctx.px_cx(x, ntype)                 # the cached inverse
    want = cx.px(x, nosb=orc.TOSBW, ntype=ntype, win=win)
    assert rel(z, want) < 1e-9
    np.testing.assert_array_equal(z2, z)


def test_fortran_externals_with_callbacks(lib, orc):
    """qmr_cx_ and pist_conv_sx_ with caller callbacks on COMPLEX*16 arrays
    (a dense complex symmetric matrix, the reference drivers' pattern)."""
    import ctypes as C
    FOP = C.CFUNCTYPE(None, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double))
    FLIN = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double),
                       C.POINTER(C.c_double))
    I, D, ref = C.c_int, C.c_double, C.byref

    def dp(a):
        return a.ctypes.data_as(C.POINTER(C.c_double))

    def cview(ptr, k):
        return np.ctypeslib.as_array(ptr, shape=(2 * k,)).view(np.complex128)

    rng = np.random.default_rng(14)
    n = 40
    a = rng.standard_normal((n, n))
    M = (a + a.T) / 2 + np.diag(np.linspace(1.0, 6.0, n)) - 1j * np.diag(rng.uniform(0.01, 0.1, n))
    d = np.diag(M).copy()

    @FOP
    def hmult(pn, px, py):
        k = pn[0]
        cview(py, k)[:] = M @ cview(px, k)

    @FOP
    def pmult(pn, px, py):
        k = pn[0]
        cview(py, k)[:] = cview(px, k) / d

    x0 = np.arange(1, n + 1).astype(np.complex128)
    b = M @ x0
    x = np.zeros(n, np.complex128)
    res = D(0.0)
    code = lib.qmr_cx_(ref(I(0)), ref(I(1000)), ref(D(1e-12)), ref(I(n)), dp(b.view(np.float64)),
                       C.cast(hmult, C.c_void_p), C.cast(pmult, C.c_void_p), dp(x.view(np.float64)), ref(res))
    code_r, x_r, _ = orc.qmr_cx(lambda v: M @ v, lambda v: v / d, b, 1000, 1e-12)
    assert code > 0 and abs(code - code_r) <= 1
    assert np.abs(x - x0).max() / n < 1e-9

    E0 = 3.0
    inv = np.linalg.inv(M - E0 * np.eye(n))

    @FLIN
    def linsolv(pn, pb, px, pres):
        k = pn[0]
        cview(px, k)[:] = inv @ cview(pb, k)
        return 1

    xs = rng.random(n) + 0j
    eig = np.zeros(5, np.complex128)
    st = lib.pist_conv_sx_(ref(D(E0)), ref(D(1e-12)), ref(I(0)), ref(I(n)), dp(xs.view(np.float64)), ref(I(0)),
                           ref(I(5)), ref(I(1)), ref(I(5)), ref(I(n)), C.cast(hmult, C.c_void_p),
                           C.cast(linsolv, C.c_void_p), dp(eig.view(np.float64)), ref(res))
    st_r, eig_r, _ = orc.pist_conv_sx(E0, 1e-12, 0, xs, 0, 5, 1, 5, n, lambda v: M @ v, lambda v: (1, inv @ v))
    assert st > 0 and st_r > 0
    np.testing.assert_allclose(eig, eig_r, atol=1e-9)


def test_driver_resonance_and_crp_jobs(lib, tmp_path):
    """The driver flow on reference-format files for JOB_RES1 (OSB_PISTCONVDX1:
    resonances of H - i AP) and JOB_CRP (osbCRP at mE0 + (i-1) mTol)."""
    from scalit_gb300 import osb, refio
    p = hm.build_problem(hm.Grid3(12, 10, 8), hm.PES())
    H = hm.dense_hamiltonian(p, shift=0.0)
    rng = np.random.default_rng(15)
    apr = np.zeros(p.N)
    pts = rng.choice(p.N, 8, replace=False)
    apr[pts] = rng.uniform(1e-3, 3e-3, 8)
    app = np.where(apr == 0.0, rng.uniform(0.0, 2e-3, p.N), 0.0)
    refio.save_data_dir(tmp_path / "APP.dat", app)
    refio.save_data_dir(tmp_path / "APR.dat", apr)
    exact = np.linalg.eigvals(H)
    e0 = float(np.sort(exact.real)[12]) + 3e-4

    inp = refio.OSBInput(sJOB=refio.JOB_RES1, sAP=True, sBJ=(20, 1e-4), sQMR=(1000, 1e-12),
                         sConv=(e0, 1e-11, 0, 5, 200, 4, 1), sOSBW=(e0, 0.0, 0.0, 0),
                         APPFile=str(tmp_path / "APP.dat"))
    inp = refio.write_problem_files(p, tmp_path, inp)
    o = osb.OSB.read((tmp_path / "input.txt").read_text())
    assert o.load_init_data()
    o.prog_diag(log=None)
    st, eig, res, _ = o.prog_pist_eig(log=None)
    o.close()
    cx = np.linalg.eigvals(H - 1j * np.diag(app))
    want = cx[np.argsort(np.abs(cx.real - e0))[:4]]
    want = want[np.argsort(want.real)]
    assert st > 0
    np.testing.assert_allclose(eig, want, atol=1e-7)

    inp2 = refio.OSBInput(sJOB=refio.JOB_CRP, sAP=True, sBJ=(20, 1e-4), sQMR=(2000, 1e-12),
                          sConv=(e0, 1e-3, 0, 5, 0, 2, 9), sOSBW=(e0, 0.0, 0.0, 0),
                          APPFile=str(tmp_path / "APP.dat"), APRFile=str(tmp_path / "APR.dat"))
    inp2 = refio.write_problem_files(p, tmp_path, inp2)
    o2 = osb.OSB.read((tmp_path / "input.txt").read_text())
    assert o2.load_init_data()
    o2.prog_diag(log=None)
    n, crp, _, info = o2.prog_pist_eig(log=None)
    o2.close()
    ap = app + apr
    sq = np.diag(np.sqrt(apr))
    for E, got in zip(info["energies"], crp):
        G = lambda s: np.linalg.inv(H - E * np.eye(p.N) + s * 1j * np.diag(ap))
        dense = 4.0 * np.real(np.trace(sq @ G(1) @ np.diag(app) @ G(-1) @ sq))
        assert abs(got - dense) / dense < 1e-5


def test_pist_cx_conjugate_levels(lib, orc, case):
    """PIST_CONV_CX (JOB_RES2, the conjugated product) reaches the same complex
    levels of H - i AP as the dense eigenvalues and the oracle."""
    p, ref, e0, app, apr = case
    cx = orc.CxOperator(ref, app, apr)
    H = hm.dense_hamiltonian(p, shift=0.0)
    exact = np.linalg.eigvals(H - 1j * np.diag(cx.AP))
    want = exact[np.argsort(np.abs(exact.real - e0))[:4]]
    want = want[np.argsort(want.real)]
    x0 = np.random.default_rng(17).random(p.N) + 1j * np.random.default_rng(18).random(p.N)
    with context(p, ref, e0, app, apr) as ctx:
        st, eig, res = ctx.pist_cx(x0, 4, e0, 1e-11, 200, qmrmax=1000, qmrtol=1e-12, conjugate=True)
    assert st > 0
    np.testing.assert_allclose(eig, want, atol=1e-8)


def _cx_hamiltonian(p, seed):
    rng = np.random.default_rng(seed)
    parts = []
    for l, n in enumerate(p.sizes):
        K = p.level_matrix(l + 1)
        S = rng.standard_normal((n, n)) * 1e-4
        parts.append((K + 1j * (S + S.T)).ravel(order="F"))
    return np.concatenate(parts), p.DEP * (1.0 + 1j * rng.uniform(-0.05, 0.05, p.DEP.size))


@pytest.mark.parametrize("sizes", [(12, 10, 8), (32, 24, 20)])
def test_complex_hamiltonian_hx(lib, orc, sizes):
    """The complex-Hamiltonian job (sCX): MYHX_CX with complex level matrices
    and complex DEP (osb.hxcx.h:191-261) against the oracle, 1e-12, for the
    plain, shifted and absorbing forms; the real entry points see the real
    parts, and a real load drops the imaginary ones."""
    p = hm.build_problem(hm.Grid3(*sizes), hm.PES())
    e0 = float(p.RES.min()) + 1e-3
    ref = orc.Operator.from_problem(p, E0=e0)
    app = np.random.default_rng(5).uniform(0.0, 2e-3, p.N)
    cx = orc.CxOperator(ref, app)
    H0CX, DEPCX = _cx_hamiltonian(p, 6)
    cx.set_complex_h0(H0CX, DEPCX)
    X = cvec(np.random.default_rng(7), (2, p.N))
    with capi.Context(p.sizes, p.dep) as ctx:
        ctx.load_cx(H0CX, p.RES, DEPCX)
        ctx.set_shift(e0)
        ctx.set_absorbing(app)
        for ntype in (capi.TA0, capi.TA1, capi.TMAP):
            Y = ctx.hx_cx(X, ntype)
            for v in range(2):
                assert rel(Y[v], cx.hx(X[v], ntype)) < 1e-12, (ntype, v)
        # the real H*X of the same context: the real parts
        xr = X[0].real.copy()
        real = orc.Operator(p.sizes, p.dep, H0CX.real, p.RES, DEPCX.real, E0=e0)
        assert rel(ctx.hx(xr, capi.TA1), real.hx(xr, 1)) < 1e-12
        ctx.load(p.H0, p.RES, p.DEP)
        ctx.set_absorbing(app)
        plain = orc.CxOperator(ref, app)
        assert rel(ctx.hx_cx(X[0], capi.TA1), plain.hx(X[0], capi.TA1)) < 1e-12


def test_complex_hamiltonian_qmr_and_pist(lib, orc):
    """QMR_CX and the complex symmetric PIST on a complex Hamiltonian: the
    solution of (H - E0 - i AP) x = b against the dense solve, and the levels
    of H - i AP nearest E0 against the dense eigenvalues (the preconditioner
    is built from the real parts: it sets the convergence, not the result)."""
    p = hm.build_problem(hm.Grid3(12, 10, 8), hm.PES())
    H0CX, DEPCX = _cx_hamiltonian(p, 8)
    app = np.random.default_rng(9).uniform(0.0, 2e-3, p.N)
    sizes, N = p.sizes, p.N
    H = np.diag(p.RES).astype(np.complex128)
    h0, dp = 0, 0
    for l, n in enumerate(sizes):
        nin = int(np.prod(sizes[:l], dtype=np.int64))
        blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
        Hl = H0CX[h0:h0 + n * n].reshape((n, n), order="F")
        h0 += n * n
        D = np.diag(DEPCX[dp:dp + nin]) if p.dep[l] else np.eye(nin)
        dp += nin if p.dep[l] else 0
        H = H + np.kron(np.eye(blk), np.kron(Hl, D))
    Hm = H - 1j * np.diag(app)
    ev = np.linalg.eigvals(Hm)
    e0 = float(np.sort(ev.real)[12]) + 3e-4
    b = cvec(np.random.default_rng(10), N)
    with capi.Context(p.sizes, p.dep) as ctx:
        ctx.load_cx(H0CX, p.RES, DEPCX)
        ctx.set_shift(e0)
        ctx.set_absorbing(app)
        ctx.build_osb(20, 1e-4)
        code, x, res = ctx.qmr_cx(b, 2000, 1e-10, ntype=capi.TMAP)
        assert code > 0
        x_dense = np.linalg.solve(Hm - e0 * np.eye(N), b)
        assert rel(x, x_dense) < 1e-7
        x0 = np.random.default_rng(11).random(N) + 1j * np.random.default_rng(12).random(N)
        st, eig, res = ctx.pist_cx(x0, 4, e0, 1e-11, 200, qmrmax=1000, qmrtol=1e-12)
    assert st > 0
    want = ev[np.argsort(np.abs(ev.real - e0))[:4]]
    want = want[np.argsort(want.real)]
    np.testing.assert_allclose(np.sort_complex(eig), np.sort_complex(want), atol=1e-8)


def test_driver_complex_hamiltonian_job(lib, tmp_path):
    """The driver flow with sCX: H0 and DEP as COMPLEX*16 files (loadData_CX,
    loadDataDir_CX; osb.io.h:46-54,211-222), JOB_RES1: the levels of
    H_complex - i AP nearest E0 against the dense eigenvalues."""
    import dataclasses
    from scalit_gb300 import osb, refio
    p = hm.build_problem(hm.Grid3(12, 10, 8), hm.PES())
    H0CX, DEPCX = _cx_hamiltonian(p, 13)
    app = np.random.default_rng(14).uniform(0.0, 2e-3, p.N)
    sizes = p.sizes
    H = np.diag(p.RES).astype(np.complex128)
    h0, dp = 0, 0
    for l, n in enumerate(sizes):
        nin = int(np.prod(sizes[:l], dtype=np.int64))
        blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
        Hl = H0CX[h0:h0 + n * n].reshape((n, n), order="F")
        h0 += n * n
        D = np.diag(DEPCX[dp:dp + nin]) if p.dep[l] else np.eye(nin)
        dp += nin if p.dep[l] else 0
        H = H + np.kron(np.eye(blk), np.kron(Hl, D))
    ev = np.linalg.eigvals(H - 1j * np.diag(app))
    e0 = float(np.sort(ev.real)[12]) + 3e-4
    refio.save_data_dir(tmp_path / "APP.dat", app)
    inp = refio.OSBInput(sJOB=refio.JOB_RES1, sAP=True, sBJ=(20, 1e-4), sQMR=(1000, 1e-12),
                         sConv=(e0, 1e-11, 0, 5, 200, 4, 1), sOSBW=(e0, 0.0, 0.0, 0),
                         APPFile=str(tmp_path / "APP.dat"))
    inp = refio.write_problem_files(p, tmp_path, inp)
    refio.save_data(inp.H0File, np.ascontiguousarray(H0CX).view(np.float64))
    refio.save_data_dir(inp.DEPFile, np.ascontiguousarray(DEPCX).view(np.float64))
    inp = dataclasses.replace(inp, sCX=True)
    (tmp_path / "input.txt").write_text(refio.write_input(inp))
    o = osb.OSB.read((tmp_path / "input.txt").read_text())
    assert o.inp.sCX
    assert o.load_init_data()
    o.prog_diag(log=None)
    st, eig, res, _ = o.prog_pist_eig(log=None)
    o.close()
    want = ev[np.argsort(np.abs(ev.real - e0))[:4]]
    want = want[np.argsort(want.real)]
    assert st > 0
    np.testing.assert_allclose(eig, want, atol=1e-7)
