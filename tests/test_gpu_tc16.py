"""FP32 H*X on the persistent tensor-core level kernel (csrc/tc_fp32p.cu).

Grids whose inner blocks are multiples of 32 points (32x24x20, 64x20x12,
96x96x64) run every level on it, partial tiles included; the others run
their first level on it and the rest on the earlier engines.

Split-FP16 x3 with exponent scaling (SCALIT_FP32_TENSOR16) must carry the
accuracy of the FP32 CUDA-core GEMM: H*X within 2e-6 norm-wise of the FP64
oracle (MYHX, osb.hx.h:71-110), for vectors of any scale (the per-vector
exponent), with partial tiles, more tiles than SMs (the persistent walk over
many vectors) and per-vector shifts.  Split-BF16 x3 (SCALIT_FP32_TENSOR) runs
on the same kernel at its own 16-bit tolerance.  The mixed QMR converges with
the FP16 form as with the CUDA cores.
"""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

TOL_F16X3 = 2e-6    # split-FP16 x3: 22 significant bits per operand, FP32 sums
TOL_BF16X3 = 3e-5   # split-BF16 x3: 16 significant bits


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _hx32(ctx, X, ntype):
    import torch
    dx = torch.tensor(X, dtype=torch.float32, device="cuda")
    dy = torch.full_like(dx, float("nan"))
    ctx.hx_f32_device(dx, dy, X.shape[0], ntype)
    torch.cuda.synchronize()
    return dy.double().cpu().numpy()


@pytest.mark.parametrize("sizes", [(24, 32, 20), (20, 12, 8), (36, 44, 28), (32, 24, 20), (64, 20, 12),
                                   (160, 12, 8), (224, 12, 4), (96, 12, 8), (160, 12, 7)])
@pytest.mark.parametrize("mode,tol", [(capi.FP32_TENSOR16, TOL_F16X3), (capi.FP32_TENSOR, TOL_BF16X3)])
def test_hx_f32_persistent(lib, orc, sizes, mode, tol):
    """Both split forms against the FP64 oracle; vectors scaled by 1e-30 ..
    1e+30 exercise the FP16 form's per-vector exponent.  Blocks of 32, 64,
    96, 160 and 224 points put a tile's four 32-point groups in 1 to 4 runs
    of one to four groups, and short last blocks leave rows past the
    vector's end."""
    pytest.importorskip("torch")
    p = hm.build_problem(hm.Grid3(*sizes), hm.PES())
    e0 = float(p.RES.min())
    ref = orc.Operator.from_problem(p, E0=e0)
    rng = np.random.default_rng(7)
    X = rng.standard_normal((4, p.N))
    X[1] *= 1e-30
    X[2] *= 1e30
    X[3] = rng.random(p.N) * np.exp(-np.linspace(0.0, 20.0, p.N))   # 9 decades inside one vector
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.set_fp32_mode(mode)
        for ntype in (capi.TA0, capi.TA1):
            Y = _hx32(ctx, X, ntype)
            for v in range(4):
                assert rel(Y[v], ref.hx(X[v], ntype)) < tol, (ntype, v)


def test_hx_f32_persistent_many_tiles(lib, orc):
    """96x96x64 with 16 vectors: 768 level-1 tiles, so each CTA walks several
    tiles through both TMEM accumulators; the result equals one-vector calls
    and the oracle."""
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-96x96x64")
    e0 = float(p.RES.min())
    ref = orc.Operator.from_problem(p, E0=e0)
    X = np.random.default_rng(3).standard_normal((16, p.N))
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.set_fp32_mode(capi.FP32_TENSOR16)
        Y = _hx32(ctx, X, capi.TA1)
        Y1 = np.stack([_hx32(ctx, X[v:v + 1], capi.TA1)[0] for v in (0, 9, 15)])
    for v in (0, 5, 9, 15):
        assert rel(Y[v], ref.hx(X[v], 1)) < TOL_F16X3, v
    # one launch or sixteen: the same tiles, the same arithmetic
    np.testing.assert_array_equal(Y1, Y[[0, 9, 15]])
    del torch


def test_hx_f32_persistent_level_times(lib):
    """The per-level timing entry point runs the persistent kernel (every
    level of 96x96x64 fits one tile) and reports positive durations."""
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-96x96x64")
    with capi.Context.from_problem(p, e0=float(p.RES.min())) as ctx:
        ctx.set_fp32_mode(capi.FP32_TENSOR16)
        dx = torch.randn(4, p.N, dtype=torch.float32, device="cuda")
        dy = torch.empty_like(dx)
        ms = ctx.hx_level_times(dx, dy, 4, reps=3)
    assert len(ms) == 3 and all(t > 0 for t in ms)


def test_qmr_fp32_tensor16_converges(lib):
    """The FP32 QMR with H*X in split-FP16 x3 reaches the tolerance the
    CUDA-core engine reaches, within a few iterations of it."""
    c0 = hm.workload("tri-24x32x20")
    e0 = float(c0.RES.min()) - 1e-3
    b = np.random.default_rng(1).random(c0.N)
    out = {}
    for mode in (capi.FP32_SIMT, capi.FP32_TENSOR16):
        with capi.Context.from_problem(c0, e0=e0) as ctx:
            ctx.set_fp32_mode(mode)
            ctx.build_osb(20, 1e-4)
            code, X, res, it = ctx.qmr(b, 300, 1e-6, precision=capi.PREC_FP32)
            r = ctx.hx(X, capi.TA1) - b
        out[mode] = (code, np.linalg.norm(r) / np.linalg.norm(b))
    c_simt, r_simt = out[capi.FP32_SIMT]
    c_16, r_16 = out[capi.FP32_TENSOR16]
    assert c_simt > 0 and c_16 > 0
    assert abs(c_16 - c_simt) <= max(3, c_simt // 10), (c_16, c_simt)
    assert r_16 < 1e-5


def test_pist_mixed_tensor16(lib):
    """Mixed PIST with the FP16 tensor-core H*X in its inner solves: the
    levels equal the oracle's 24x32x20 fixture within 1e-4 cm^-1."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "pist_tri-24x32x20.json")) as f:
        fx = json.load(f)
    p = hm.workload(fx["workload"])
    x0 = np.random.default_rng(fx["seed"]).random(p.N)
    with capi.Context.from_problem(p, e0=fx["e0"]) as ctx:
        ctx.set_fp32_mode(capi.FP32_TENSOR16)
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, fx["levels"], fx["e0"], fx["etol"], startcnt=fx["startcnt"],
                                      stepcnt=fx["stepcnt"], m_max=fx["m_max"], qmr_max=fx["qmr_max"],
                                      qmr_tol=fx["qmr_tol"], precision=capi.PREC_FP32, orth=2)
    assert st > 0
    err = np.abs(eig - np.array(fx["eigenvalues_eh"])) * hm.HARTREE_CM
    assert err.max() < 1e-4
