"""OSBW window preconditioner on the GPU against the oracle (initOSBW,
src/iterate/module/osb.osbw.h:2-50; getVOSBH0, osb.hij.h:128-159; createWH,
osb.pij.h:6-45; MYPX with TOSBW, osb.px.h:191-206).

The context takes the oracle's VOSB / EIG0 (set_osb), so both sides select
the window from identical EIG0.  Tolerances: the window width and points are
the same host arithmetic (bit-exact); HW's off-diagonal entries are FP64
sums in another order (1e-12 of max |HW|) and its diagonal is EIG0 (exact);
P*X applies HWR^-1 (from the eigen-decomposition of HWR) where the oracle
solves with DSYTRF/DSYTRS (1e-9 norm-wise in FP64, 1e-4 in FP32).
"""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

COUNT = 40


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case(orc):
    p = hm.build_problem(hm.Grid3(12, 10, 8), hm.PES())
    ref = orc.Operator.from_problem(p, E0=0.0)
    ref.build_osb(20, 1e-4)
    e0 = float(np.sort(ref.EIG0)[15]) + 2e-4
    ref.set_e0(e0)
    return p, ref, e0


def context(p, ref, e0):
    ctx = capi.Context.from_problem(p, e0=e0)
    ctx.set_osb(ref.VOSB, ref.EIG0)
    return ctx


@pytest.mark.parametrize("de0", [1e-5, 0.05])
def test_window_and_hw_match_oracle(lib, orc, case, de0):
    p, ref, e0 = case
    win = orc.OSBW(ref, e0, COUNT, de0)
    with context(p, ref, e0) as ctx:
        m, de = ctx.build_osbw(e0, COUNT, de0)
        ind, HW = ctx.get_osbw()
    assert m == COUNT and de == win.de
    np.testing.assert_array_equal(ind, win.ind)
    np.testing.assert_array_equal(np.diag(HW), np.diag(win.HW))
    np.testing.assert_array_equal(HW, HW.T)
    assert np.abs(HW - win.HW).max() < 1e-12 * np.abs(win.HW).max()


@pytest.mark.parametrize("npc", [capi.TA1, capi.TA0])
def test_px_matches_oracle(lib, orc, case, npc):
    p, ref, e0 = case
    win = orc.OSBW(ref, e0, COUNT, 1e-4, npc=npc)
    X = np.random.default_rng(0).standard_normal((3, p.N))
    with context(p, ref, e0) as ctx:
        ctx.build_osbw(e0, COUNT, 1e-4, npc=npc)
        Z = ctx.px(X.ravel(), npc).reshape(3, p.N)
    for v in range(3):
        assert rel(Z[v], orc.osbw_px(ref, win, X[v], npc)) < 1e-9


def test_px_f32_matches_oracle(lib, orc, case):
    torch = pytest.importorskip("torch")
    p, ref, e0 = case
    win = orc.OSBW(ref, e0, COUNT, 1e-4)
    x = np.random.default_rng(1).standard_normal(p.N)
    with context(p, ref, e0) as ctx:
        ctx.build_osbw(e0, COUNT, 1e-4)
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dz = torch.empty_like(dx)
        ctx.px_f32_device(dx, dz)
        torch.cuda.synchronize()
        z = dz.double().cpu().numpy()
    assert rel(z, orc.osbw_px(ref, win, x, 1)) < 1e-4


def test_qmr_matches_oracle_and_beats_tosb(lib, orc, case):
    p, ref, e0 = case
    win = orc.OSBW(ref, e0, COUNT, 1e-4)
    b = np.random.default_rng(2).standard_normal(p.N)
    st_r, x_r, _, it_r = orc.osbw_qmr(ref, win, b, 2000, 1e-10)
    with context(p, ref, e0) as ctx:
        ctx.set_fp64_mode(capi.FP64_DFMA)
        ctx.build_osbw(e0, COUNT, 1e-4)
        st, x, res, it = ctx.qmr(b, 2000, 1e-10)
        ctx.set_precond(capi.TOSB)
        st1, _, _, it1 = ctx.qmr(b, 2000, 1e-10)
        ctx.set_precond(capi.TOSBW)
        st2, x2, _, it2 = ctx.qmr(b, 2000, 1e-10)
    assert st_r > 0 and st > 0 and st1 > 0
    assert abs(it - it_r) <= 1
    assert rel(x, x_r) < 1e-7
    assert it < it1
    assert it2 == it and rel(x2, x) < 1e-14


def test_set_osbw_from_saved_hw(lib, case):
    """saveHW / loadHW: HW taken back selects the same window and gives the same P*X."""
    p, ref, e0 = case
    x = np.random.default_rng(3).standard_normal(p.N)
    with context(p, ref, e0) as ctx:
        _, de = ctx.build_osbw(e0, COUNT, 1e-4)
        ind, HW = ctx.get_osbw()
        z = ctx.px(x)
    with context(p, ref, e0) as ctx2:
        de2 = ctx2.set_osbw(e0, COUNT, 1e-4, HW)
        ind2, HW2 = ctx2.get_osbw()
        z2 = ctx2.px(x)
    assert de2 == de
    np.testing.assert_array_equal(ind2, ind)
    np.testing.assert_array_equal(HW2, HW)
    assert rel(z2, z) < 1e-12           # the same HW factored again


def test_pist_with_window_preconditioner(lib, orc):
    """PIST's QMR solves through the window preconditioner reach the same levels."""
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min())
    x0 = orc.start_vector(p.N, 0)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        st1, eig1, _, info1 = ctx.pist(x0, 20, e0, 1e-11, m_max=400, qmr_max=500, qmr_tol=1e-4)
        ctx.build_osbw(e0, 60, 1e-4)
        st4, eig4, _, info4 = ctx.pist(x0, 20, e0, 1e-11, m_max=400, qmr_max=500, qmr_tol=1e-4)
    assert st1 > 0 and st4 > 0
    assert np.abs(eig4 - eig1).max() * hm.HARTREE_CM < 1e-4


def test_errors(lib, case):
    p, ref, e0 = case
    with capi.Context.from_problem(p, e0=e0) as ctx:
        with pytest.raises(capi.ScalitError) as e:
            ctx.build_osbw(e0, COUNT, 1e-4)                   # no preconditioner yet
        assert e.value.code == -104
        ctx.set_osb(ref.VOSB, ref.EIG0)
        with pytest.raises(capi.ScalitError) as e:
            ctx.set_precond(capi.TOSBW)                       # no window yet
        assert e.value.code == -104
        for count, de in ((0, 1e-4), (p.N + 1, 1e-4), (COUNT, 0.0), (COUNT, -1.0)):
            with pytest.raises(capi.ScalitError) as e:
                ctx.build_osbw(e0, count, de)
            assert e.value.code == -101
        e_on = float(np.sort(ref.EIG0)[15])
        with pytest.raises(capi.ScalitError) as e:
            ctx.build_osbw(e_on, 1, 1e-4)                     # HWR = 0: DSYTRF info > 0
        assert e.value.code == -101
        ctx.build_osbw(e0, COUNT, 1e-4)
        x = np.random.default_rng(4).standard_normal(p.N)
        ctx.px(x)
        ctx.set_osb(ref.VOSB, ref.EIG0)                      # the window is stale now
        with pytest.raises(capi.ScalitError) as e:
            ctx.px(x)
        assert e.value.code == -104


def test_module_seam_osbw(lib):
    """scalit_fortran_precond_ with sOSB = 4 then scalit_fortran_osbw_ (initOSBW):
    the module's EPX applies the same window preconditioner as a context that
    makes the same build and window (the device build is deterministic)."""
    import ctypes as C
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min()) + 1e-3
    I, D, ref = C.c_int, C.c_double, C.byref

    def dp(a):
        return a.ctypes.data_as(C.POINTER(C.c_double))

    sn = (C.c_int * 3)(*p.sizes)
    sdep = (C.c_int * 3)(*[int(d) for d in p.dep])
    ierr = I(-1)
    b = np.random.default_rng(5).standard_normal(p.N)
    y = np.zeros(p.N)
    lib.scalit_fortran_device_(ref(I(0)))
    lib.scalit_fortran_init_(ref(I(3)), sn, sdep, dp(p.H0), dp(p.RES), dp(p.DEP), ref(D(e0)), ref(ierr))
    assert ierr.value == 0
    try:
        lib.scalit_fortran_precond_(ref(I(4)), ref(D(0.0)), ref(D(0.0)), ref(I(20)), ref(D(1e-4)), ref(ierr))
        assert ierr.value == 0
        de = D(1e-4)
        lib.scalit_fortran_osbw_(ref(D(e0)), ref(I(50)), ref(de), ref(I(capi.TA1)), ref(ierr))
        assert ierr.value == 0
        lib.scalit_epx_(ref(I(p.N)), dp(b), dp(y))
    finally:
        lib.scalit_fortran_final_()
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        m, de_c = ctx.build_osbw(e0, 50, 1e-4)
        z = ctx.px(b)
    assert m == 50 and de.value == de_c
    assert rel(y, z) < 1e-12


def test_driver_flow_with_window(lib, tmp_path):
    """The driver with sOSB = 4: progDiag then initOSBW, HW written (sHW = 1) and
    read back (sHW = -1, loadHW) into the same P*X; PIST converges through it."""
    from scalit_gb300 import osb, refio
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min())
    inp = refio.OSBInput(sOSB=refio.TOSBW, sBJ=(20, 1e-4), sQMR=(500, 1e-4),
                         sConv=(e0, 1e-11, 0, 5, 400, 20, 1), sOSBW=(e0, 1e-4, 0.0, 60), sHW=1,
                         HWFile=str(tmp_path / "HW.dat"))
    inp = refio.write_problem_files(p, tmp_path, inp)
    text = (tmp_path / "input.txt").read_text()
    lines = []
    o = osb.OSB.read(text)
    assert o.load_init_data()
    o.prog_diag(log=lines.append)
    st, eig, res, info = o.prog_pist_eig(log=None)
    x = np.random.default_rng(6).standard_normal(p.N)
    z = o.ctx.px(x)
    _, HW = o.ctx.get_osbw()
    o.close()
    assert st > 0
    assert any("final window width" in s for s in lines)
    np.testing.assert_array_equal(refio.load_hw(inp.HWFile, 60), HW)
    inp2 = refio.read_input(text)
    inp2.sHW = -1
    o2 = osb.OSB(inp2)
    o2.load_init_data()
    o2.prog_diag(log=None)
    assert rel(o2.ctx.px(x), z) < 1e-12
    o2.close()
