"""OSB preconditioner build and P*X on the GPU against the oracle.

The device block-Jacobi keeps the reference's rotation order (hosbdiag.f90:
i = 1..MAK-1, j = 1..MAK-i), so EIG0, VOSB and P*X agree with the oracle to
rounding (norm-wise 1e-10), not only in effect.
"""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("sizes", [(6, 5, 4), (12, 10, 8), (24, 32, 20), (3, 70, 5)])
def test_build_and_px_match_oracle(lib, orc, sizes):
    p = hm.build_problem(hm.Grid3(*sizes), hm.PES())
    e0 = float(p.RES.min()) - 1e-3
    ref = orc.Operator.from_problem(p, E0=e0)
    st_ref = ref.build_osb(20, 1e-4)
    x = np.random.default_rng(0).standard_normal(p.N)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        st = ctx.build_osb(20, 1e-4)
        V, E = ctx.get_osb()
        z = ctx.px(x)
        z0 = ctx.px(x, capi.TA0)
    assert rel(E, ref.EIG0) < 1e-11
    assert rel(V, ref.VOSB) < 1e-9
    np.testing.assert_array_equal(st[:, 4], st_ref[:, 4])       # sweep counters
    assert rel(z, ref.px(x)) < 1e-9
    assert rel(z0, ref.px(x, npc=0)) < 1e-9


@pytest.mark.parametrize("kind,de,beta", [(2, 2e-3, 0.0), (3, 2e-3, 0.5)])
def test_windowed_kernels(lib, orc, kind, de, beta):
    """TOSBD1 / TOSBD2 windows (osb.px.h:160-189)."""
    p = hm.build_problem(hm.Grid3(12, 10, 8), hm.PES())
    e0 = 0.004
    ref = orc.Operator.from_problem(p, E0=e0)
    ref.build_osb(20, 1e-4)
    x = np.random.default_rng(1).standard_normal(p.N)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.set_precond(kind, de, beta)
        ctx.build_osb(20, 1e-4)
        z = ctx.px(x)
    assert rel(z, ref.px(x, nosb=kind, de=de, beta=beta)) < 1e-9


def test_px_is_inverse_for_one_level(lib):
    """With one level the block-Jacobi is an exact eigen-decomposition, so P = (H-E0)^-1."""
    rng = np.random.default_rng(3)
    n = 40
    a = rng.standard_normal((n, n))
    H = (a + a.T) / 2
    res = rng.standard_normal(n) + 10.0
    with capi.Context((n,), (False,)) as ctx:
        ctx.load(H.ravel(order="F"), res, None)
        ctx.set_shift(0.0)
        ctx.build_osb(50, 1e-14)
        x = rng.standard_normal(n)
        z = ctx.px(ctx.hx(x, capi.TA1))
    assert rel(z, x) < 1e-10


def test_set_osb_roundtrip(lib):
    p = hm.build_problem(hm.Grid3(6, 5, 4), hm.PES())
    x = np.random.default_rng(4).standard_normal(p.N)
    with capi.Context.from_problem(p, e0=0.0) as ctx:
        ctx.build_osb(20, 1e-4)
        V, E = ctx.get_osb()
        z = ctx.px(x)
    with capi.Context.from_problem(p, e0=0.0) as ctx2:
        with pytest.raises(capi.ScalitError):
            ctx2.px(x)
        ctx2.set_osb(V, E)
        np.testing.assert_array_equal(ctx2.px(x), z)


def test_px_f32(lib, orc):
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min()) - 1e-3
    ref = orc.Operator.from_problem(p, E0=e0)
    ref.build_osb(20, 1e-4)
    x = np.random.default_rng(5).standard_normal(p.N)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dz = torch.empty_like(dx)
        ctx.px_f32_device(dx, dz)
        torch.cuda.synchronize()
        z = dz.double().cpu().numpy()
    assert rel(z, ref.px(x)) < 1e-5


def test_px_f32_tensor_engine(lib, orc):
    """P*X in FP32 with the outer rotations on the tensor cores (split-BF16 x3)."""
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min()) - 1e-3
    ref = orc.Operator.from_problem(p, E0=e0)
    ref.build_osb(20, 1e-4)
    x = np.random.default_rng(5).standard_normal(p.N)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.set_fp32_mode(capi.FP32_TENSOR)
        ctx.build_osb(20, 1e-4)
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dz = torch.empty_like(dx)
        ctx.px_f32_device(dx, dz)
        torch.cuda.synchronize()
        z = dz.double().cpu().numpy()
    assert rel(z, ref.px(x)) < 1e-4


def test_fp32_tensor_px_mode(lib):
    """SCALIT_FP32_TENSOR_PX: the preconditioner's rotations take the tensor
    cores (the same results as SCALIT_FP32_TENSOR) while H*X stays on the CUDA
    cores (the same results as SCALIT_FP32_SIMT)."""
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-24x32x20")
    x = np.random.default_rng(6).standard_normal(p.N)
    out = {}
    with capi.Context.from_problem(p, e0=float(p.RES.min()) - 1e-3) as ctx:
        ctx.build_osb(20, 1e-4)
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        for mode in (capi.FP32_SIMT, capi.FP32_TENSOR, capi.FP32_TENSOR_PX, capi.FP32_TENSOR16):
            ctx.set_fp32_mode(mode)
            hy, pz = torch.empty_like(dx), torch.empty_like(dx)
            ctx.hx_f32_device(dx, hy)
            ctx.px_f32_device(dx, pz)
            torch.cuda.synchronize()
            out[mode] = (hy.cpu(), pz.cpu())
        with pytest.raises(capi.ScalitError):
            ctx.set_fp32_mode(4)
    assert torch.equal(out[capi.FP32_TENSOR_PX][0], out[capi.FP32_SIMT][0])
    # SCALIT_FP32_TENSOR16 rotates with the same split-BF16 x3 rotations
    assert torch.equal(out[capi.FP32_TENSOR16][1], out[capi.FP32_TENSOR][1])
    assert torch.equal(out[capi.FP32_TENSOR_PX][1], out[capi.FP32_TENSOR][1])
    assert not torch.equal(out[capi.FP32_TENSOR][1], out[capi.FP32_SIMT][1])
