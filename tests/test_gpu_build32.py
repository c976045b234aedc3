"""Preconditioner build with FP32 Jacobi sweeps
(scalit_set_build_precision(SCALIT_PREC_FP32)): the build the mixed PIST arm
uses, since its preconditioner only feeds FP32 inner solves.

* EIG0 equals the FP64 build's (the same rotation order, FP32 rounding), the
  first level's V blocks are orthogonal to FP32 accuracy; the grids put the
  outer levels on both the one-CTA stacks (FP64 in both builds) and the
  spread schedule (FP32 stacks);
* mixed PIST on the FP32-built preconditioner (QMR tolerance 1e-6, FP64
  residual refinement to 1e-8 Eh, as the bench's mixed arm runs) reproduces
  the oracle's committed 24x32x20 levels within 1e-4 cm^-1 and meets the
  residual target;
* the FP32 P*X with the first level's matrices stored in FP16
  (scalit_set_fp32_px_storage(16)) stays within the FP16 rounding of the
  FP32 P*X, and returns to it bit for bit when the storage goes back to 32;
  mixed PIST with both (the bench's mixed arm) still meets the fixture and
  the residual target;
* an unknown precision or storage is refused.
"""
import json
import os

import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu


def _build(p, e0, prec):
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.set_build_precision(prec)
        stats = ctx.build_osb(20, 1e-4)
        V, E = ctx.get_osb()
    return stats, V, E


@pytest.mark.parametrize("sizes", [(24, 32, 20), (40, 12, 10)])
def test_fp32_build_matches_fp64(lib, sizes):
    p = hm.build_problem(hm.Grid3(*sizes), hm.PES())
    e0 = float(p.RES.min())
    s64, V64, E64 = _build(p, e0, capi.PREC_FP64)
    s32, V32, E32 = _build(p, e0, capi.PREC_FP32)
    scale = np.abs(E64).max()
    assert np.abs(E32 - E64).max() < 2e-5 * scale
    n0, blk0 = sizes[0], sizes[1] * sizes[2]
    for b in (0, blk0 // 2, blk0 - 1):
        Vb = V32[b * n0 * n0:(b + 1) * n0 * n0].reshape(n0, n0)
        assert np.abs(Vb @ Vb.T - np.eye(n0)).max() < 1e-5, b
    # sweeps of the first level: the FP32 sweep test sees the same decay
    assert abs(s32[0, 4] - s64[0, 4]) <= 0.25 * s64[0, 4] + blk0


def test_fp16_px_storage(lib):
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-24x32x20")
    with capi.Context.from_problem(p, e0=float(p.RES.min()) - 1e-3) as ctx:
        ctx.build_osb(20, 1e-4)
        X = torch.randn(3, p.N, dtype=torch.float32, device="cuda")
        Y32, Y16, Yb = (torch.empty_like(X) for _ in range(3))
        ctx.px_f32_device(X, Y32, 3)
        ctx.set_fp32_px_storage(16)
        ctx.px_f32_device(X, Y16, 3)
        ctx.set_fp32_px_storage(32)
        ctx.px_f32_device(X, Yb, 3)
        torch.cuda.synchronize()
        with pytest.raises(capi.ScalitError):
            ctx.set_fp32_px_storage(8)
    a, b = Y32.double().cpu().numpy(), Y16.double().cpu().numpy()
    for v in range(3):
        r = np.linalg.norm(a[v] - b[v]) / np.linalg.norm(a[v])
        assert 1e-6 < r < 3e-3, (v, r)       # the FP16 copy is used, and only rounds
    assert torch.equal(Y32, Yb)


def test_fp16_px_storage_needs_blocks_of_eight(lib):
    """First levels of a length that is not a multiple of 8 keep the FP32
    matrices (the FP16 chunks would not be 16-byte aligned): storage 16 then
    gives the FP32 P*X bit for bit."""
    torch = pytest.importorskip("torch")
    p = hm.build_problem(hm.Grid3(20, 12, 8), hm.PES())
    with capi.Context.from_problem(p, e0=float(p.RES.min()) - 1e-3) as ctx:
        ctx.build_osb(20, 1e-4)
        X = torch.randn(2, p.N, dtype=torch.float32, device="cuda")
        Y32, Y16 = torch.empty_like(X), torch.empty_like(X)
        ctx.px_f32_device(X, Y32, 2)
        ctx.set_fp32_px_storage(16)
        ctx.px_f32_device(X, Y16, 2)
        torch.cuda.synchronize()
    assert torch.equal(Y32, Y16)


@pytest.mark.parametrize("bits", [32, 16])
def test_mixed_pist_on_fp32_build(lib, bits):
    with open(os.path.join(os.path.dirname(__file__), "golden", "pist_tri-24x32x20.json")) as f:
        fx = json.load(f)
    p = hm.workload(fx["workload"])
    x0 = np.random.default_rng(fx["seed"]).random(p.N)
    with capi.Context.from_problem(p, e0=fx["e0"]) as ctx:
        ctx.set_fp32_mode(capi.FP32_TENSOR16)
        ctx.set_build_precision(capi.PREC_FP32)
        ctx.set_fp32_px_storage(bits)
        ctx.build_osb(20, 1e-4)
        st, eig, res, info = ctx.pist(x0, fx["levels"], fx["e0"], fx["etol"], startcnt=fx["startcnt"],
                                      m_max=fx["m_max"], qmr_max=fx["qmr_max"], qmr_tol=1e-6,
                                      precision=capi.PREC_FP32_REFINED, orth=3, refine_tol=1e-8,
                                      refine_steps=20)
    assert st > 0
    err = np.abs(eig - np.array(fx["eigenvalues_eh"])) * hm.HARTREE_CM
    assert err.max() < 1e-4
    assert np.max(info["resid"]) <= 1e-8


def test_build_precision_rejects_unknown(lib):
    p = hm.workload("tri-24x32x20")
    with capi.Context.from_problem(p, e0=float(p.RES.min())) as ctx:
        with pytest.raises(capi.ScalitError):
            ctx.set_build_precision(capi.PREC_FP32_REFINED)
