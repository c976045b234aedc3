"""H*X on the GPU against the oracle (MYHX, src/iterate/module/osb.hx.h:71-110).

Tolerance: norm-wise relative error 1e-12 in FP64 (elementwise relative error
is ill-posed where the potential cancels the kinetic terms); 2e-6 in FP32.
"""
import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-6


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def c0():
    return hm.workload("tri-24x32x20")


ENGINES = [capi.FP64_TENSOR, capi.FP64_DFMA]


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("ntype", [0, 1])
def test_hx_c0_16_vectors(lib, orc, c0, ntype, engine):
    e0 = float(c0.RES.min())
    ref = orc.Operator.from_problem(c0, E0=e0)
    X = np.random.default_rng(0).standard_normal((16, c0.N))
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        ctx.set_fp64_mode(engine)
        Y = ctx.hx(X, ntype)
    for v in range(16):
        assert rel(Y[v], ref.hx(X[v], ntype)) < TOL64


@pytest.mark.parametrize("sizes", [(2, 3, 2), (5, 7, 3), (8, 8, 8), (13, 1, 9), (1, 6, 4),
                                   (67, 3, 5), (3, 130, 2)])
@pytest.mark.parametrize("engine", ENGINES)
def test_hx_odd_shapes(lib, orc, sizes, engine):
    grid = hm.Grid3(*sizes)
    p = hm.build_problem(grid, hm.PES())
    ref = orc.Operator.from_problem(p, E0=0.01)
    x = np.random.default_rng(1).standard_normal(p.N)
    with capi.Context.from_problem(p, e0=0.01) as ctx:
        ctx.set_fp64_mode(engine)
        y = ctx.hx(x, capi.TA1)
    assert rel(y, ref.hx(x, 1)) < TOL64


def test_hx_general_levels(lib, orc):
    """A 4-level grid with two dependent levels (the layout is general in sF)."""
    sizes = (4, 5, 3, 6)
    dep = (False, True, False, True)
    rng = np.random.default_rng(2)
    H0 = []
    for n in sizes:
        a = rng.standard_normal((n, n))
        H0.append(((a + a.T) / 2).ravel(order="F"))
    H0 = np.concatenate(H0)
    N = int(np.prod(sizes))
    RES = rng.standard_normal(N)
    dims = np.cumprod((1,) + sizes[:-1])
    DEP = np.concatenate([rng.uniform(0.5, 1.5, int(dims[l])) for l in range(4) if dep[l]])
    ref = orc.Operator(sizes, dep, H0, RES, DEP, E0=0.3)
    x = rng.standard_normal(N)
    with capi.Context(sizes, dep) as ctx:
        ctx.load(H0, RES, DEP)
        ctx.set_shift(0.3)
        for nt in (0, 1):
            assert rel(ctx.hx(x, nt), ref.hx(x, nt)) < TOL64


def test_hx_f32_device(lib, orc, c0):
    torch = pytest.importorskip("torch")
    e0 = float(c0.RES.min())
    ref = orc.Operator.from_problem(c0, E0=e0)
    x = np.random.default_rng(3).standard_normal(c0.N)
    with capi.Context.from_problem(c0, e0=e0) as ctx:
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dy = torch.empty_like(dx)
        ctx.hx_f32_device(dx, dy, 1, capi.TA1)
        torch.cuda.synchronize()
        y = dy.double().cpu().numpy()
    assert rel(y, ref.hx(x, 1)) < TOL32


def test_hx_device_many(lib, orc, c0):
    torch = pytest.importorskip("torch")
    X = np.random.default_rng(4).standard_normal((3, c0.N))
    ref = orc.Operator.from_problem(c0, E0=0.0)
    with capi.Context.from_problem(c0, e0=0.0) as ctx:
        dX = torch.tensor(X, device="cuda")
        dY = torch.empty_like(dX)
        ctx.hx_device(dX, dY, 3, capi.TA0)
        torch.cuda.synchronize()
        Y = dY.cpu().numpy()
    for v in range(3):
        assert rel(Y[v], ref.hx(X[v], 0)) < TOL64


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("name", ["tri-96x96x64", "tri-160x160x120"])
def test_hx_large(lib, orc, name, engine):
    p = hm.workload(name)
    e0 = float(p.RES.min())
    ref = orc.Operator.from_problem(p, E0=e0)
    x = np.random.default_rng(5).standard_normal(p.N)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.set_fp64_mode(engine)
        y = ctx.hx(x, capi.TA1)
    assert rel(y, ref.hx(x, 1)) < TOL64


def test_hx_tensor_matches_dfma_elementwise(lib, c0):
    """The digit-sliced tensor-core engine against the FP64 pipe, element by element
    relative to the row scale (|Y| can cancel to zero, the row scale cannot)."""
    x = np.random.default_rng(9).standard_normal(c0.N)
    with capi.Context.from_problem(c0, e0=0.0) as ctx:
        ctx.set_fp64_mode(capi.FP64_DFMA)
        y0 = ctx.hx(x, capi.TA1)
        ctx.set_fp64_mode(capi.FP64_TENSOR)
        y1 = ctx.hx(x, capi.TA1)
    scale = np.abs(y0).max()
    assert np.abs(y1 - y0).max() / scale < 1e-13


def test_hx_rejects_nonfinite(lib, c0):
    bad = c0.RES.copy()
    bad[7] = np.nan
    with capi.Context(c0.sizes, c0.dep) as ctx:
        with pytest.raises(capi.ScalitError) as e:
            ctx.load(c0.H0, bad, c0.DEP)
        assert e.value.code == -106


def test_hx_before_load_is_an_error(lib, c0):
    with capi.Context(c0.sizes, c0.dep) as ctx:
        with pytest.raises(capi.ScalitError) as e:
            ctx.hx(np.zeros(c0.N))
        assert e.value.code == -104


def test_tile_autotuner_picks(lib, c0):
    """The load-time autotuner picks a tile for every level GEMM it tuned."""
    with capi.Context.from_problem(c0, e0=0.0) as ctx:
        t = ctx.tile_picks()
    assert t.shape == (2, 3, 2)
    assert set(np.unique(t[1])) <= {0, 1}            # FP32: one vector and 16
    assert set(np.unique(t[0, :, 0])) <= {0, 1}      # FP64 CUDA-core engine: one vector
    assert (t[0, :, 1] == -1).all()


TOL_BF16X3 = 3e-5   # split-BF16 x3: 16 significant bits per operand, FP32 sums


@pytest.mark.parametrize("sizes", [(24, 32, 20), (13, 7, 5), (17, 33, 9)])
def test_hx_f32_tensor_engine(lib, orc, sizes):
    """FP32 H*X on the tensor cores (split-BF16 x3) against the FP64 oracle,
    several vectors with their own shifts, odd sizes (partial tiles)."""
    torch = pytest.importorskip("torch")
    p = hm.build_problem(hm.Grid3(*sizes), hm.PES())
    ref = orc.Operator.from_problem(p, E0=0.0)
    X = np.random.default_rng(11).standard_normal((3, p.N))
    shifts = float(p.RES.min()) + np.array([0.0, 0.004, 0.011])
    with capi.Context.from_problem(p, e0=0.0) as ctx:
        ctx.set_fp32_mode(capi.FP32_TENSOR)
        dx = torch.tensor(X, dtype=torch.float32, device="cuda")
        dy = torch.empty_like(dx)
        ctx.hx_f32_device(dx, dy, 3, capi.TA0)
        torch.cuda.synchronize()
        Y = dy.double().cpu().numpy()
    for v in range(3):
        assert rel(Y[v], ref.hx(X[v], 0)) < TOL_BF16X3
    # shifted systems through the multi-shift QMR use per-vector shifts; checked there
    del shifts
