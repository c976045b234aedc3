"""The oracle's OSBW window preconditioner against dense mathematics (CPU).

The reference (src/iterate/module/osb.osbw.h, osb.vi.h, osb.hij.h, osb.pij.h,
osb.px.h:191-206) ships no known answers for it, so the restatement is pinned
to its definition: the window basis vectors are columns of V = V_sF..V_1,
Hij is V^T H V on the window with EIG0 on the diagonal, and P*X equals
V M V^T X with M = 1/(EIG0 - E0) outside the window and (Hij - E0)^-1 on it.
"""
import numpy as np
import pytest

from scalit_gb300 import hamiltonian as hm


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def small(orc, sizes=(6, 7, 5)):
    p = hm.build_problem(hm.Grid3(*sizes), hm.PES())
    op = orc.Operator.from_problem(p, E0=0.0)
    op.build_osb(30, 1e-12)
    return p, op


def dense_v(orc, op):
    """V = V_sF .. V_1 column by column through the oracle's VX (hpx.f90:40-56)."""
    sizes = op.sizes
    vs = orc.vosb_starts(sizes)
    dims = np.cumprod((1,) + sizes[:-1])
    V = np.zeros((op.N, op.N))
    for j in range(op.N):
        y = np.zeros(op.N)
        y[j] = 1.0
        for l, n in enumerate(sizes):
            blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
            y = orc.vx(int(dims[l]), n, blk, op.VOSB[vs[l]:vs[l] + blk * n * n], y)
        V[:, j] = y
    return V


def test_osbw_window_width(orc):
    rng = np.random.default_rng(0)
    eig = rng.uniform(0.0, 1.0, 1000)
    for de0 in (1e-4, 0.3):                  # grows from too narrow, bisects from too wide
        de = orc.osbw_adjust(eig, 0.3, 37, de0)
        ind = orc.osbw_index(eig, 0.3, de)
        assert ind.size == 37 and np.all(np.diff(ind) > 0)
        nearest = np.sort(np.argsort(np.abs(eig - 0.3))[:37])
        np.testing.assert_array_equal(ind, nearest)
    with pytest.raises(ValueError):          # tied distances: no width holds exactly one state
        orc.osbw_adjust(np.array([0.1, -0.1, 0.5]), 0.0, 1, 0.01)


def test_osbw_vi_is_column_of_v(orc):
    p, op = small(orc)
    V = dense_v(orc, op)
    ind = np.array([0, 1, 17, 41, 100, op.N - 1])
    bk, col = orc.osbw_level_index(op.sizes, ind)
    for i, j in enumerate(ind):
        np.testing.assert_allclose(orc.osbw_vi(op.sizes, op.VOSB, bk[:, i], col[:, i]), V[:, j],
                                   rtol=0, atol=1e-15)


@pytest.mark.parametrize("count", [1, 12, 40])
def test_osbw_hij_is_projected_h(orc, count):
    p, op = small(orc)
    V = dense_v(orc, op)
    H = hm.dense_hamiltonian(p, shift=0.0)
    e0 = float(np.sort(op.EIG0)[8]) + 2e-4
    win = orc.OSBW(op, e0, count, 1e-4)
    ind = win.ind
    assert ind.size == count
    Hp = V[:, ind].T @ H @ V[:, ind]
    off = ~np.eye(count, dtype=bool)
    if count > 1:
        assert np.abs(win.HW[off] - Hp[off]).max() < 1e-12 * np.abs(H).max()
    np.testing.assert_array_equal(np.diag(win.HW), op.EIG0[ind])


def test_osbw_singular_window_is_an_error(orc):
    """E0 on an OSB eigenvalue with a one-state window: HWR = 0, DSYTRF
    reports info > 0 and createWH (osb.pij.h:40-42) fails."""
    p, op = small(orc)
    e0 = float(np.sort(op.EIG0)[8])
    with pytest.raises(ValueError):
        orc.OSBW(op, e0, 1, 1e-4)


@pytest.mark.parametrize("npc", [0, 1])
def test_osbw_px_equals_dense(orc, npc):
    p, op = small(orc)
    V = dense_v(orc, op)
    e0 = float(np.sort(op.EIG0)[10]) + 2e-4
    op.set_e0(e0)
    win = orc.OSBW(op, e0, 25, 1e-4, npc=npc)
    shift = e0 if npc else 0.0
    M = np.diag(1.0 / (op.EIG0 - shift))
    M[np.ix_(win.ind, win.ind)] = np.linalg.inv(win.HW - (e0 if npc else 0.0) * np.eye(win.ind.size))
    x = np.random.default_rng(1).standard_normal(op.N)
    assert rel(orc.osbw_px(op, win, x, npc), V @ M @ V.T @ x) < 1e-10


def test_osbw_qmr_needs_fewer_iterations(orc):
    """The exact window removes the near-singular OSB states around E0: QMR on
    (H - E0) x = b converges in fewer iterations than with TOSB and reaches
    the same solution."""
    p, op = small(orc, (10, 9, 8))
    e0 = float(np.sort(op.EIG0)[12]) + 3e-4
    op.set_e0(e0)
    win = orc.OSBW(op, e0, 40, 1e-4)
    b = np.random.default_rng(2).standard_normal(op.N)
    st1, x1, _, it1 = op.qmr(b, 2000, 1e-10, nosb=1)
    st4, x4, _, it4 = orc.osbw_qmr(op, win, b, 2000, 1e-10)
    assert st1 > 0 and st4 > 0
    assert it4 < it1
    H = hm.dense_hamiltonian(p, shift=e0)
    assert rel(H @ x4, b) < 1e-8
    assert rel(x4, x1) < 1e-7
