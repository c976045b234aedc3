"""Shifted right-hand sides and batches of problems (QMR on many systems at once).

Each column of a shifted solve is the reference's QMR (qmr_mpi.f90) on
(H - E_v) x = b_v with the preconditioner's kernel at E_v, so it must equal a
single-system solve at that shift; a batch of problems must equal the problems
solved one by one."""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _problem(n_r, n_R, n_t, seed=0):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.9, 1.1, size=2)
    pes = hm.PES(de_R=hm.PES().de_R * f[0], amp2=hm.PES().amp2 * f[1])
    return hm.build_problem(hm.Grid3(n_r, n_R, n_t), pes)


def _shifts(p, nrhs):
    e = float(p.RES.min())
    return e + 0.02 * (np.arange(nrhs) + 0.5) / nrhs


def test_shifted_fp64_equals_single_solves(lib, orc):
    p = _problem(12, 10, 8)
    sh = _shifts(p, 3)
    B = np.random.default_rng(1).standard_normal((3, p.N))
    with capi.Context.from_problem(p, e0=0.0) as ctx:
        ctx.set_fp64_mode(capi.FP64_DFMA)
        ctx.set_precond(capi.TOSBD1, 0.002, 0.0)
        ctx.build_osb(20, 1e-6)
        dB = torch.tensor(B, device="cuda")
        dX = torch.zeros_like(dB)
        codes, res = ctx.qmr_shifts_device(dB, dX, sh, 400, 1e-9, ntype=-1)
        X = dX.cpu().numpy()
        for v, e in enumerate(sh):
            ctx.set_shift(e)
            code1, X1, res1, it1 = ctx.qmr(B[v], 400, 1e-9, ntype=-1)
            assert abs(int(codes[v]) - code1) <= 1, (v, codes[v], code1)
            assert code1 > 0
            np.testing.assert_allclose(X[v], X1, rtol=0, atol=1e-8 * np.abs(X1).max())
    # each column really solves its own shifted system (oracle H*X)
    ref = orc.Operator.from_problem(p, E0=0.0)
    for v, e in enumerate(sh):
        r = ref.hx(X[v], 0) - e * X[v] - B[v]
        assert np.linalg.norm(r) / np.linalg.norm(B[v]) < 1e-7


def test_shifted_fp32_residuals(lib, orc):
    p = _problem(16, 12, 10, seed=2)
    nrhs = 16
    sh = _shifts(p, nrhs)
    B = np.random.default_rng(3).standard_normal((nrhs, p.N))
    with capi.Context.from_problem(p, e0=0.0) as ctx:
        ctx.set_precond(capi.TOSBD1, 0.002, 0.0)
        ctx.build_osb(20, 1e-6)
        dB = torch.tensor(B, device="cuda")
        dX = torch.zeros_like(dB)
        codes, res = ctx.qmr_shifts_device(dB, dX, sh, 2000, 1e-4, ntype=-1, precision=capi.PREC_FP32)
        X = dX.cpu().numpy()
    # shifts inside the spectrum make some systems nearly singular; most converge
    assert (codes > 0).sum() >= 12, codes
    ref = orc.Operator.from_problem(p, E0=0.0)
    for v, e in enumerate(sh):
        if codes[v] <= 0:
            continue
        r = ref.hx(X[v], 0) - e * X[v] - B[v]
        # QMR's own test is |HX-B|/|HX| < 1e-4 in FP32 arithmetic
        assert np.linalg.norm(r) / np.linalg.norm(ref.hx(X[v], 0) - e * X[v]) < 5e-4


def test_batch_equals_one_by_one(lib):
    probs = [_problem(12, 10, 8, 0), _problem(9, 14, 6, 1), _problem(16, 8, 12, 2)]
    nrhs = 4
    shifts = np.stack([_shifts(p, nrhs) for p in probs])
    rng = np.random.default_rng(4)
    Bs = [rng.standard_normal((nrhs, p.N)) for p in probs]
    ctxs = [capi.Context.from_problem(p, e0=0.0) for p in probs]
    try:
        for c in ctxs:
            c.set_precond(capi.TOSBD1, 0.002, 0.0)
            c.build_osb(20, 1e-6)
        dBs = [torch.tensor(B, device="cuda") for B in Bs]
        dXs = [torch.zeros_like(b) for b in dBs]
        codes, res, sec = capi.qmr_shifts_batch(ctxs, shifts, dBs, dXs, 2000, 1e-4, precision=capi.PREC_FP32)
        assert sec > 0
        for k, c in enumerate(ctxs):
            dX1 = torch.zeros_like(dBs[k])
            codes1, res1 = c.qmr_shifts_device(dBs[k], dX1, shifts[k], 2000, 1e-4, precision=capi.PREC_FP32)
            np.testing.assert_array_equal(codes[k], codes1)
            assert torch.equal(dXs[k], dX1)          # same kernels, same order: bit for bit
    finally:
        for c in ctxs:
            c.close()


def test_shift_bad_arguments(lib):
    p = _problem(8, 6, 4)
    with capi.Context.from_problem(p, e0=0.0) as ctx:
        dB = torch.zeros((2, p.N), dtype=torch.float64, device="cuda")
        with pytest.raises(capi.ScalitError):      # no preconditioner yet
            ctx.qmr_shifts_device(dB, torch.zeros_like(dB), [0.0, 0.1], 10, 1e-4)
        ctx.build_osb(10, 1e-6)
        with pytest.raises(capi.ScalitError):
            ctx.qmr_shifts_device(dB, torch.zeros_like(dB), [0.0, 0.1], 10, 1e-4, precision=7)
