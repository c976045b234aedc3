"""The Fortran drop-in symbols, called exactly as gfortran would call them
(every argument by reference, caller-owned host arrays), against the oracle.
"""
import ctypes as C

import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

I = C.c_int
D = C.c_double
FOP = C.CFUNCTYPE(None, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double))
FLIN = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double),
                   C.POINTER(C.c_double))


def ref(x):
    return C.byref(x)


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("nin,nout,blk", [(1, 24, 640), (24, 32, 20), (768, 20, 1), (7, 5, 3)])
def test_h1x_xyz(lib, orc, nin, nout, blk):
    rng = np.random.default_rng(nin + nout)
    H = rng.standard_normal(nout * nout)
    X = rng.standard_normal(nin * nout * blk)
    Y = np.zeros_like(X)
    for name in ("h1x_xyz_", "h1x_xyz_seq_"):
        getattr(lib, name)(ref(I(nin)), ref(I(nout)), ref(I(blk)), dp(H), dp(X), dp(Y))
        assert rel(Y, orc.h1x_xyz(nin, nout, blk, H, X)) < 1e-14
    lib.h1tx_xyz_seq_(ref(I(nin)), ref(I(nout)), ref(I(blk)), dp(H), dp(X), dp(Y))
    assert rel(Y, orc.h1tx_xyz(nin, nout, blk, H, X)) < 1e-14


@pytest.mark.parametrize("nin,nout,blk", [(768, 20, 1), (24, 32, 20), (1, 6, 9)])
def test_h1x_dep(lib, orc, nin, nout, blk):
    rng = np.random.default_rng(3)
    H = rng.standard_normal(nout * nout)
    c = rng.uniform(0.5, 2.0, nin)
    X = rng.standard_normal(nin * nout * blk)
    Y = np.zeros_like(X)
    for name in ("h1x_dep_", "h2x_dep_seq_"):
        getattr(lib, name)(ref(I(nin)), ref(I(nout)), ref(I(blk)), dp(H), dp(c), dp(X), dp(Y))
        assert rel(Y, orc.h1x_dep(nin, nout, blk, H, c, X)) < 1e-14


def test_h3x_out_seq(lib, orc):
    rng = np.random.default_rng(4)
    nin, nout, blk = 30, 7, 2
    A = rng.standard_normal(nin * nout * nout)
    X = rng.standard_normal(nin * nout * blk)
    Y = np.zeros_like(X)
    lib.h3x_out_seq_(ref(I(nin)), ref(I(nout)), ref(I(blk)), dp(A), dp(X), dp(Y))
    for b in range(blk):
        sl = slice(b * nin * nout, (b + 1) * nin * nout)
        assert rel(Y[sl], orc.h3x(nin, nout, A, X[sl])) < 1e-14


@pytest.mark.parametrize("nin,nout,blk", [(1, 24, 50), (24, 32, 20), (768, 20, 1)])
def test_vx_vtx(lib, orc, nin, nout, blk):
    rng = np.random.default_rng(5)
    V = rng.standard_normal(nout * nout * blk)
    X = rng.standard_normal(nin * nout * blk)
    for name, fn in (("vx_", orc.vx), ("vtx_", orc.vtx), ("vx_seq_", orc.vx), ("vtx_seq_", orc.vtx)):
        Z = X.copy()
        getattr(lib, name)(ref(I(nin)), ref(I(nout)), ref(I(blk)), dp(V), dp(Z))
        assert rel(Z, fn(nin, nout, blk, V, X)) < 1e-14, name


def test_hosbdiag(lib, orc):
    """HosbDiag on a level-3-like stack (NDK > 1, joint Jacobi) and on 1x1 stacks."""
    p = hm.build_problem(hm.Grid3(6, 5, 4), hm.PES())
    for blk, mak, ndk in ((1, 4, 30), (30, 4, 1), (4, 5, 6)):
        rng = np.random.default_rng(blk * 100 + mak)
        H1 = rng.standard_normal((mak, mak))
        H1 = ((H1 + H1.T) / 2).ravel(order="F")
        res = rng.standard_normal(ndk * mak * blk)
        hosb = np.zeros(ndk * mak * mak * blk)
        orc.lib().orc_hosbinit_xyz(blk, mak, ndk, orc._p(H1), orc._p(res), orc._p(hosb))
        h_ref, v_ref, e_ref = hosb.copy(), np.zeros(mak * mak * blk), np.zeros(ndk * mak * blk)
        orc.lib().orc_hosbdiag(20, 1e-8, blk, mak, ndk, orc._p(h_ref), orc._p(v_ref), orc._p(e_ref),
                               None, None)
        h, v, e = hosb.copy(), np.zeros_like(v_ref), np.zeros_like(e_ref)
        lib.hosbdiag_(ref(I(20)), ref(D(1e-8)), ref(I(blk)), ref(I(mak)), ref(I(ndk)), dp(h), dp(v), dp(e))
        assert rel(e, e_ref) < 1e-12
        assert rel(v, v_ref) < 1e-10
        assert np.abs(h - h_ref).max() < 1e-10 * np.abs(h_ref).max() + 1e-14
    del p


def test_hosbdiag_mpi(lib, orc):
    """HOSBDIAG_MPI on one rank equals HosbDiag (hosbdiag_mpi.f90:5-96), IERR = 0."""
    blk, mak, ndk = 3, 5, 40
    rng = np.random.default_rng(21)
    H1 = rng.standard_normal((mak, mak))
    H1 = ((H1 + H1.T) / 2).ravel(order="F")
    res = rng.standard_normal(ndk * mak * blk)
    hosb = np.zeros(ndk * mak * mak * blk)
    orc.lib().orc_hosbinit_xyz(blk, mak, ndk, orc._p(H1), orc._p(res), orc._p(hosb))
    h_ref, v_ref, e_ref = hosb.copy(), np.zeros(mak * mak * blk), np.zeros(ndk * mak * blk)
    orc.lib().orc_hosbdiag(20, 1e-8, blk, mak, ndk, orc._p(h_ref), orc._p(v_ref), orc._p(e_ref), None, None)
    h, v, e = hosb.copy(), np.zeros_like(v_ref), np.zeros_like(e_ref)
    ierr = I(-5)
    lib.hosbdiag_mpi_(ref(I(0)), ref(I(20)), ref(D(1e-8)), ref(I(blk)), ref(I(mak)), ref(I(ndk)), dp(h), dp(v),
                      dp(e), ref(ierr), ref(I(0)))
    assert ierr.value == 0
    assert rel(e, e_ref) < 1e-12
    assert rel(v, v_ref) < 1e-10


@pytest.mark.parametrize("p,q,nout,nin", [(1, 2, 4, 1), (2, 5, 6, 300), (3, 1, 5, 7), (4, 4 + 3, 9, 25600)])
def test_mjacobi(lib, orc, p, q, nout, nin):
    """MJACOBI (jacobi.f90:2-83): the rotated stack and the returned angle equal the oracle's."""
    rng = np.random.default_rng(p * 10 + q)
    H = np.zeros((nin, nout, nout), order="F")
    for a in range(nin):
        m = rng.standard_normal((nout, nout))
        H[a] = (m + m.T) / 2
    flat = np.asfortranarray(H).ravel(order="F").copy()
    want = flat.copy()
    work = np.zeros(2 * nin)
    x_ref = orc.lib().orc_mjacobi(p, q, nout, nin, orc._p(want), orc._p(work))
    x = lib.mjacobi_(ref(I(p)), ref(I(q)), ref(I(nout)), ref(I(nin)), dp(flat))
    assert abs(x - x_ref) <= 1e-12 * max(1.0, abs(x_ref))
    assert np.abs(flat - want).max() <= 1e-12 * np.abs(want).max()


def _pisth0_case(n=400, m_max=12, seed=31):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n))
    H = (a + a.T) / 2 + np.diag(np.linspace(0.0, 3.0, n))
    E0 = 0.7
    x = rng.random(n)
    return H, E0, x


def _oracle_pisth0(H, E0, x, m_max, blocks):
    """pistH0 (pistHij.f90:70-125) on the oracle's MGS_ORTH, block after block."""
    n = x.size
    VJ = np.zeros((n, m_max), order="F")
    HM = np.zeros((m_max, m_max), order="F")
    out = []
    for m_low, m_high in blocks:
        if m_low == 1:
            VJ[:, 0] = x / np.sqrt(orc_dot(x, x))
        for J in range(1 if m_low == 1 else m_low - 1, m_high):
            w = np.linalg.solve(H - E0 * np.eye(n), VJ[:, J - 1])
            assert ORC.mgs_orth(w, J, VJ)
        for J in range(m_low, m_high + 1):
            w = H @ VJ[:, J - 1]
            for I_ in range(1, m_high + 1):
                HM[I_ - 1, J - 1] = orc_dot(np.ascontiguousarray(VJ[:, I_ - 1]), w)
                HM[J - 1, I_ - 1] = HM[I_ - 1, J - 1]
        out.append(m_high)
    return VJ, HM, out


ORC = None


def orc_dot(a, b):
    return ORC.lib().orc_dot(a.size, ORC._p(np.ascontiguousarray(a)), ORC._p(np.ascontiguousarray(b)))


@pytest.mark.parametrize("mpi", [False, True])
def test_pisth0(lib, orc, mpi):
    """pistH0 / pistH0_MPI with caller callbacks: the basis and HMAT of two
    successive blocks (1..6, then 7..10) equal the oracle's."""
    global ORC
    ORC = orc
    H, E0, x = _pisth0_case()
    n, m_max = x.size, 12
    nsolve = {"n": 0}

    @FOP
    def h0x(pn, px, py):
        k = pn[0]
        np.ctypeslib.as_array(py, shape=(k,))[:] = H @ np.ctypeslib.as_array(px, shape=(k,))

    @FLIN
    def linsolv(pn, pb, px, pres):
        k = pn[0]
        np.ctypeslib.as_array(px, shape=(k,))[:] = np.linalg.solve(H - E0 * np.eye(k),
                                                                   np.ctypeslib.as_array(pb, shape=(k,)))
        pres[0] = 0.0
        nsolve["n"] += 1
        return 3

    blocks = [(1, 6), (7, 10)]
    VJ_r, HM_r, out_r = _oracle_pisth0(H, E0, x, m_max, blocks)
    VJ = np.zeros(n * m_max)
    HM = np.zeros(m_max * m_max)
    for (m_low, m_high), want in zip(blocks, out_r):
        num2 = I(-1)
        if mpi:
            got = lib.pisth0_mpi_(ref(I(0)), ref(I(0)), ref(I(n)), dp(x), ref(I(m_max)), ref(I(m_low)),
                                  ref(I(m_high)), C.cast(h0x, C.c_void_p), C.cast(linsolv, C.c_void_p), dp(VJ),
                                  dp(HM), ref(num2))
            first = 1 if m_low == 1 else m_low - 1
            assert num2.value == 3 * (m_high - first)
        else:
            got = lib.pisth0_(ref(I(n)), dp(x), ref(I(m_max)), ref(I(m_low)), ref(I(m_high)),
                              C.cast(h0x, C.c_void_p), C.cast(linsolv, C.c_void_p), dp(VJ), dp(HM))
        assert got == want
    V = VJ.reshape((n, m_max), order="F")[:, :10]
    assert np.abs(V - VJ_r[:, :10]).max() < 1e-10
    Hm = HM.reshape((m_max, m_max), order="F")[:10, :10]
    assert np.abs(Hm - HM_r[:10, :10]).max() < 1e-10 * np.abs(HM_r).max()
    assert nsolve["n"] == 9
    # bad sizes return 0 without touching anything
    assert lib.pisth0_(ref(I(n)), dp(x), ref(I(m_max)), ref(I(5)), ref(I(5)),
                       C.cast(h0x, C.c_void_p), C.cast(linsolv, C.c_void_p), dp(VJ), dp(HM)) == 0


def test_norm_dot(lib):
    rng = np.random.default_rng(6)
    x, y = rng.standard_normal(10001), rng.standard_normal(10001)
    ierr = I(7)
    assert lib.norm_mpi_(ref(I(0)), ref(I(x.size)), dp(x), ref(ierr)) == pytest.approx(np.linalg.norm(x), rel=1e-14)
    assert ierr.value == 0
    assert lib.dotprod_mpi_(ref(I(0)), ref(I(x.size)), dp(x), dp(y), ref(ierr)) == pytest.approx(x @ y, rel=1e-12)


def test_mgs_orth(lib, orc):
    rng = np.random.default_rng(8)
    n, m = 5000, 6
    VJ = np.asfortranarray(np.linalg.qr(rng.standard_normal((n, m + 1)))[0])
    VJ[:, m] = 0.0
    w = rng.standard_normal(n)
    VR = VJ.copy(order="F")
    assert orc.mgs_orth(w, m, VR)
    flat = np.asfortranarray(VJ).ravel(order="F").copy()
    assert lib.mgs_orth_(ref(I(n)), dp(w), ref(I(m)), dp(flat)) == 1
    got = flat.reshape((n, m + 1), order="F")
    assert rel(got[:, m], VR[:, m]) < 1e-12
    flat2 = np.asfortranarray(VJ).ravel(order="F").copy()
    assert lib.mgs_orth_mpi_(ref(I(n)), dp(w), ref(I(m)), dp(flat2), ref(I(0))) == 1
    z = np.zeros(n)
    assert lib.mgs_orth_(ref(I(n)), dp(z), ref(I(m)), dp(flat)) == 0     # zero vector: .false.


def test_qmr_with_foreign_callbacks(lib, orc):
    """qmr_/qmr_mpi_ with caller callbacks (the reference's qmr.drv.f90 operators)."""
    rng = np.random.default_rng(9)
    n = 23
    a = rng.random((n, n))
    H = np.tril(a) + np.tril(a, -1).T + n * np.eye(n)
    x0 = np.arange(1, n + 1, dtype=np.float64)
    b = H @ x0
    calls = {"hx": 0, "px": 0}

    @FOP
    def hmult(pn, px, py):
        k = pn[0]
        xv = np.ctypeslib.as_array(px, shape=(k,))
        yv = np.ctypeslib.as_array(py, shape=(k,))
        yv[:] = H @ xv
        calls["hx"] += 1

    @FOP
    def pmult(pn, px, py):
        k = pn[0]
        np.ctypeslib.as_array(py, shape=(k,))[:] = np.ctypeslib.as_array(px, shape=(k,)) / np.diag(H)
        calls["px"] += 1

    x = np.zeros(n)
    res = D(0.0)
    code = lib.qmr_(ref(I(0)), ref(I(1000)), ref(D(1e-12)), ref(I(n)), dp(b),
                    C.cast(hmult, C.c_void_p), C.cast(pmult, C.c_void_p), dp(x), ref(res))
    code_r, x_r, res_r = orc.qmr_dense(H, b, 1000, 1e-12, ntype=0)
    assert code == code_r > 0
    assert np.max(np.abs((x0 - x) / x0)) < 1e-10
    assert calls["hx"] > 0 and calls["px"] > 0
    x2 = np.zeros(n)
    code2 = lib.qmr_mpi_(ref(I(0)), ref(I(1000)), ref(D(1e-12)), ref(I(n)), dp(b),
                         C.cast(hmult, C.c_void_p), C.cast(pmult, C.c_void_p), dp(x2), ref(res), ref(I(0)))
    assert code2 == code
    np.testing.assert_allclose(x2, x, rtol=1e-13)


def test_module_seam_qmr_and_pist(lib, orc):
    """scalit_fortran_init_/precond_ + qmr_mpi_/pist_conv_mpi_ with the library's callbacks
    run device-resident and agree with the oracle."""
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min())
    sn = (C.c_int * 3)(*p.sizes)
    sdep = (C.c_int * 3)(0, 0, 1)
    ierr = I(-1)
    lib.scalit_fortran_device_(ref(I(0)))
    lib.scalit_fortran_init_(ref(I(3)), sn, sdep, dp(p.H0), dp(p.RES), dp(p.DEP), ref(D(e0)), ref(ierr))
    assert ierr.value == 0
    lib.scalit_fortran_precond_(ref(I(1)), ref(D(0.0)), ref(D(0.0)), ref(I(20)), ref(D(1e-4)), ref(ierr))
    assert ierr.value == 0
    lib.scalit_fortran_qmr_param_(ref(I(-1)), ref(I(500)), ref(D(1e-4)), ref(I(0)))
    op = orc.Operator.from_problem(p, E0=e0)
    op.build_osb(20, 1e-4)
    try:
        ehx = C.cast(lib.scalit_ehx_, C.c_void_p)
        epx = C.cast(lib.scalit_epx_, C.c_void_p)
        hx0 = C.cast(lib.scalit_hx0_, C.c_void_p)
        linsolv = C.cast(lib.scalit_osb_qmr_, C.c_void_p)
        b = np.random.default_rng(10).random(p.N)
        x = np.zeros(p.N)
        res = D(0.0)
        code = lib.qmr_mpi_(ref(I(-1)), ref(I(300)), ref(D(1e-9)), ref(I(p.N)), dp(b), ehx, epx, dp(x),
                            ref(res), ref(I(0)))
        code_r, x_r, res_r, _ = op.qmr(b, 300, 1e-9)
        assert code == code_r
        assert rel(x, x_r) < 1e-8
        # the callbacks themselves, called like the module would
        y = np.zeros(p.N)
        lib.scalit_hx0_(ref(I(p.N)), dp(b), dp(y))
        assert rel(y, op.hx(b, 0)) < 1e-12
        lib.scalit_epx_(ref(I(p.N)), dp(b), dp(y))
        assert rel(y, op.px(b)) < 1e-9
        # PIST through the MPI library's symbol
        x0 = orc.start_vector(p.N, 0)
        eig = np.zeros(20)
        pres = D(0.0)
        st = lib.pist_conv_mpi_(ref(I(0)), ref(I(0)), ref(D(e0)), ref(D(1e-11)), ref(I(0)), ref(I(p.N)),
                                dp(x0), ref(I(40)), ref(I(5)), ref(I(1)), ref(I(20)), ref(I(400)),
                                hx0, linsolv, dp(eig), ref(pres))
        assert st > 0

        def lin(v):
            rc, X, _, _ = op.qmr(v, 500, 1e-4)
            return rc, X

        st_r, eig_r, _, _ = orc.pist_conv(e0, 1e-11, 0, x0, 40, 5, 1, 20, 400, lambda v: op.hx(v, 0), lin)
        assert np.abs(eig - eig_r).max() * hm.HARTREE_CM < 1e-4
    finally:
        lib.scalit_fortran_final_()


def test_pist_with_foreign_callbacks(lib):
    """pist_conv_ with caller callbacks on a dense 60x60 matrix (pist.drv.f90 pattern)."""
    rng = np.random.default_rng(11)
    n = 60
    a = rng.standard_normal((n, n))
    H = (a + a.T) / 2
    E0 = 0.0

    @FOP
    def h0x(pn, px, py):
        k = pn[0]
        np.ctypeslib.as_array(py, shape=(k,))[:] = H @ np.ctypeslib.as_array(px, shape=(k,))

    @FLIN
    def linsolv(pn, pb, px, pres):
        k = pn[0]
        np.ctypeslib.as_array(px, shape=(k,))[:] = np.linalg.solve(H - E0 * np.eye(k),
                                                                   np.ctypeslib.as_array(pb, shape=(k,)))
        pres[0] = 0.0
        return 1

    x0 = rng.random(n)
    eig = np.zeros(5)
    res = D(0.0)
    st = lib.pist_conv_(ref(D(E0)), ref(D(1e-12)), ref(I(0)), ref(I(n)), dp(x0), ref(I(10)), ref(I(5)),
                        ref(I(1)), ref(I(5)), ref(I(60)), C.cast(h0x, C.c_void_p), C.cast(linsolv, C.c_void_p),
                        dp(eig), ref(res))
    assert st > 0
    exact = np.linalg.eigvalsh(H)
    near = np.sort(exact[np.argsort(np.abs(exact - E0))[:5]])
    np.testing.assert_allclose(eig, near, atol=1e-10)
