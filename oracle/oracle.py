"""Python side of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Thin ctypes wrappers over ``liborc.so`` (the C restatement in
``scalit_oracle.c``) plus the PIST outer loop, which is restated here in NumPy
because its dense eigen-step is LAPACK ``DSYEV`` in the reference
(``src/iterate/libiterate/pist/pist.f90:54,62``) and NumPy's ``eigvalsh`` is the
same LAPACK family.  Only tests, the package's smoke check and the benchmark's
CPU-baseline leg import this module.

Parity status: pinned against the reference's known-answer test patterns and
independent mathematics (see the header of ``scalit_oracle.c``); the reference
itself cannot be built here, so no output of the reference is compared.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

FMAX = 20
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class OrcOSB(C.Structure):
    _fields_ = [("sF", C.c_int), ("sN", C.c_int * FMAX), ("sDEP", C.c_int * FMAX),
                ("sNDVR", C.c_int), ("H0", _dp), ("RES", _dp), ("DEP", _dp),
                ("OUTH", _dp), ("E0", C.c_double)]


_OP = C.CFUNCTYPE(None, C.c_void_p, C.c_int, _dp, _dp)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_h1x_xyz.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_h1tx_xyz.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_h1x_dep.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_h3x.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_vx.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.orc_vtx.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.orc_myhx.argtypes = [C.POINTER(OrcOSB), C.c_int, _dp, _dp, _dp]
        L.orc_mypx.argtypes = [C.POINTER(OrcOSB), _dp, _dp, C.c_int, C.c_int, C.c_double,
                               C.c_double, _dp, _dp]
        L.orc_mypx.restype = C.c_int
        L.orc_hosbinit_xyz.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_hosbinit_dep.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_mjacobi.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.orc_mjacobi.restype = C.c_double
        L.orc_sumoffdiag.argtypes = [C.c_int, C.c_int, _dp]
        L.orc_sumoffdiag.restype = C.c_double
        L.orc_sumdiag.argtypes = [C.c_int, C.c_int, _dp]
        L.orc_sumdiag.restype = C.c_double
        L.orc_hosbdiag.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _dp, _dp,
                                   _dp, _dp, _ip]
        L.orc_mydiag.argtypes = [C.POINTER(OrcOSB), C.c_int, C.c_double, _dp, _dp, _dp]
        L.orc_mydiag.restype = C.c_int
        L.orc_qmr.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, _dp, _OP, C.c_void_p,
                              _OP, C.c_void_p, _dp, _dp, C.c_int, _ip]
        L.orc_qmr.restype = C.c_int
        L.orc_osb_qmr.argtypes = [C.POINTER(OrcOSB), _dp, _dp, C.c_int, C.c_double, C.c_double,
                                  C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, C.c_int, _ip]
        L.orc_osb_qmr.restype = C.c_int
        L.orc_mgs_orth.argtypes = [C.c_int, _dp, C.c_int, _dp]
        L.orc_mgs_orth.restype = C.c_int
        L.orc_dot.argtypes = [C.c_longlong, _dp, _dp]
        L.orc_dot.restype = C.c_double
        L.orc_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def num_threads() -> int:
    return lib().orc_num_threads()


# ----------------------------------------------------------------------------------
# per-level contractions
# ----------------------------------------------------------------------------------
def h1x_xyz(nin, nout, blk, H, X):
    H, X = _f64(H), _f64(X)
    Y = np.empty_like(X)
    lib().orc_h1x_xyz(nin, nout, blk, _p(H), _p(X), _p(Y))
    return Y


def h1tx_xyz(nin, nout, blk, H, X):
    H, X = _f64(H), _f64(X)
    Y = np.empty_like(X)
    lib().orc_h1tx_xyz(nin, nout, blk, _p(H), _p(X), _p(Y))
    return Y


def h1x_dep(nin, nout, blk, H, corx, X):
    H, corx, X = _f64(H), _f64(corx), _f64(X)
    Y = np.empty_like(X)
    lib().orc_h1x_dep(nin, nout, blk, _p(H), _p(corx), _p(X), _p(Y))
    return Y


def h3x(nin, nout, A, X):
    A, X = _f64(A), _f64(X)
    Y = np.empty_like(X)
    lib().orc_h3x(nin, nout, _p(A), _p(X), _p(Y))
    return Y


def vx(nin, nout, blk, V, X):
    V, X = _f64(V), _f64(X).copy()
    lib().orc_vx(nin, nout, blk, _p(V), _p(X))
    return X


def vtx(nin, nout, blk, V, X):
    V, X = _f64(V), _f64(X).copy()
    lib().orc_vtx(nin, nout, blk, _p(V), _p(X))
    return X


# ----------------------------------------------------------------------------------
# whole operator
# ----------------------------------------------------------------------------------
class Operator:
    """The OSB operator state (module globals H0/RES/DEP/VOSB/EIG0 of the reference)."""

    def __init__(self, sizes, dep, H0, RES, DEP, E0=0.0, ndvr=False, OUTH=None):
        self.sizes = tuple(int(n) for n in sizes)
        self.dep = tuple(bool(d) for d in dep)
        self.H0, self.RES = _f64(H0), _f64(RES)
        self.DEP = _f64(DEP if DEP is not None and len(DEP) else np.zeros(1))
        self.OUTH = _f64(OUTH) if OUTH is not None else np.zeros(1)
        self.E0 = float(E0)
        self.ndvr = bool(ndvr)
        self.N = int(np.prod(self.sizes))
        self.VOSB = None
        self.EIG0 = None
        self._tmp = np.empty(self.N)
        self._struct = OrcOSB()
        self._sync()

    @classmethod
    def from_problem(cls, problem, E0=0.0):
        return cls(problem.sizes, problem.dep, problem.H0, problem.RES, problem.DEP, E0)

    def _sync(self):
        s = self._struct
        s.sF = len(self.sizes)
        for i, n in enumerate(self.sizes):
            s.sN[i] = n
            s.sDEP[i] = int(self.dep[i])
        s.sNDVR = int(self.ndvr)
        s.H0, s.RES, s.DEP, s.OUTH = _p(self.H0), _p(self.RES), _p(self.DEP), _p(self.OUTH)
        s.E0 = self.E0

    def set_e0(self, e0):
        self.E0 = float(e0)
        self._sync()

    @property
    def vosb_len(self) -> int:
        blk = np.cumprod((self.sizes[1:] + (1,))[::-1])[::-1]
        return int(sum(int(b) * n * n for b, n in zip(blk, self.sizes)))

    def hx(self, X, ntype=1):
        X = _f64(X)
        Y = np.empty_like(X)
        lib().orc_myhx(C.byref(self._struct), int(ntype), _p(X), _p(Y), _p(self._tmp))
        return Y

    def build_osb(self, bjmax, bjtol):
        """myDiag: returns per-level stats (the reference's eff(1:5))."""
        self.VOSB = np.empty(self.vosb_len)
        self.EIG0 = self.RES.copy()
        stats = np.zeros(5 * len(self.sizes))
        rc = lib().orc_mydiag(C.byref(self._struct), int(bjmax), float(bjtol), _p(self.VOSB),
                              _p(self.EIG0), _p(stats))
        if rc != 0:
            raise MemoryError("oracle myDiag allocation failed")
        return stats.reshape(len(self.sizes), 5)

    def px(self, X, nosb=1, npc=1, de=0.0, beta=0.0):
        X = _f64(X)
        Y = np.empty_like(X)
        rc = lib().orc_mypx(C.byref(self._struct), _p(self.VOSB), _p(self.EIG0), int(nosb),
                            int(npc), float(de), float(beta), _p(X), _p(Y))
        if rc != 0:
            raise ValueError("unsupported preconditioner kind")
        return Y

    def qmr(self, B, qmrmax, qmrtol, nosb=1, de=0.0, beta=0.0, ntype=-1, mpi_codes=True):
        """OSB_QMR: returns (status, X, RES, iterations)."""
        B = _f64(B)
        X = np.zeros_like(B)
        res = C.c_double(0.0)
        it = C.c_int(0)
        rc = lib().orc_osb_qmr(C.byref(self._struct), _p(self.VOSB), _p(self.EIG0), int(nosb),
                               float(de), float(beta), int(ntype), int(qmrmax), float(qmrtol),
                               _p(B), _p(X), C.byref(res), int(bool(mpi_codes)), C.byref(it))
        return rc, X, res.value, it.value


def qmr_dense(H, B, qmrmax, qmrtol, ntype=0, mpi_codes=False):
    """QMR on an explicit symmetric matrix with the Jacobi preconditioner
    (the operators of src/iterate/libiterate/qmr/testing/qmr.drv.f90:56-119)."""

    class Dense(C.Structure):
        _fields_ = [("n", C.c_int), ("H", _dp)]

    H = np.asfortranarray(H, dtype=np.float64)
    Hc = np.ascontiguousarray(H.ravel(order="F"))
    n = H.shape[0]
    ctx = Dense(n, _p(Hc))
    L = lib()
    hx = _OP(("orc_dense_hx", L))
    px = _OP(("orc_dense_jacobi_px", L))
    B = _f64(B)
    X = np.zeros(n)
    res = C.c_double(0.0)
    it = C.c_int(0)
    rc = L.orc_qmr(int(ntype), int(qmrmax), float(qmrtol), n, _p(B), hx, C.byref(ctx), px,
                   C.byref(ctx), _p(X), C.byref(res), int(bool(mpi_codes)), C.byref(it))
    return rc, X, res.value


def mgs_orth(W, m, VJ):
    """MGS_ORTH in place on the Fortran-ordered (n, >=m+1) array ``VJ``."""
    assert VJ.flags.f_contiguous
    n = VJ.shape[0]
    W = _f64(W)
    flat = VJ.ravel(order="K")
    ok = lib().orc_mgs_orth(n, _p(W), int(m), flat.ctypes.data_as(_dp))
    return bool(ok)


# ----------------------------------------------------------------------------------
# PIST window / convergence helpers (src/libutil/serial/base/util.f90)
# ----------------------------------------------------------------------------------
def get_window(E0, vec, M):
    """getWindow0 (util.f90:669-716): the M entries closest to E0, picked one
    at a time; ties keep the lowest index."""
    vec = np.asarray(vec, dtype=np.float64)
    n = vec.size
    if n < M:
        out = np.empty(M)
        out[:n] = vec
        out[n:] = vec[n - 1]
        return out
    absv = np.abs(vec - E0)
    label = np.ones(n, dtype=bool)
    out = np.empty(M)
    for i in range(M):
        cand = np.where(label, absv, np.inf)
        idx = int(np.argmin(cand))    # first minimum, as the strict '>' comparison
        out[i] = vec[idx]
        label[idx] = False
    return out


def get_diff_max(v1, v2):
    """getDiffMax (util.f90:84-100)."""
    return float(np.max(np.abs(np.asarray(v1) - np.asarray(v2))))


def get_sep_max(v1, v2):
    """getSepMax (util.f90:124-149)."""
    v1, v2 = np.asarray(v1), np.asarray(v2)
    return float(np.max(np.min(np.abs(v1[:, None] - v2[None, :]), axis=1)))


def cgs2_orth(W, m, VJ):
    """Classical Gram-Schmidt applied twice (the re-orthogonalising variant of
    MGS_ORTH): W against VJ(:, 0:m) into VJ(:, m)."""
    v = _f64(W).copy()
    if np.sqrt(lib().orc_dot(v.size, _p(v), _p(v))) == 0.0:
        return False
    V = VJ[:, :m]
    for _ in range(2):
        v -= V @ (V.T @ v)
    nrm = np.sqrt(lib().orc_dot(v.size, _p(v), _p(v)))
    if nrm == 0.0:
        return False
    VJ[:, m] = v / nrm
    return True


def pist_conv(E0, etol, ntype, x, startcnt, stepcnt, stepeig, M, m_max, h0x, linsolv,
              log=None, orth=0):
    """PIST_CONV (src/iterate/libiterate/pist/pist.f90:7-98) with pistH0
    (pistHij.f90:70-125) and MGS_ORTH (gsorth.f90:42-72).

    ``h0x(v) -> H v`` and ``linsolv(v) -> (status, w)`` are the operator callbacks.
    ``orth=1`` replaces the single MGS pass by classical Gram-Schmidt twice.
    Returns ``(status, eig[M] ascending, RES, info)``.
    """
    x = _f64(x)
    N = x.size
    if stepeig >= m_max or startcnt > m_max or M > m_max:
        return 0, np.zeros(M), 0.0, {}
    VJ = np.zeros((N, m_max), order="F")
    HMAT = np.zeros((m_max, m_max))
    cnt_low, cnt_high = 1, max(startcnt, M, stepeig + 1)
    info = {"qmr_iters": [], "steps": []}
    status = 0
    res = 0.0
    eig = np.zeros(M)

    def pisth0(m_low, m_high):
        if m_low < 1 or m_low >= m_high or m_high > m_max:
            return 0
        if m_low == 1:
            m_start = 1
            t = np.sqrt(lib().orc_dot(N, _p(x), _p(x)))
            if t == 0.0:
                return 0
            VJ[:, 0] = x / t
        else:
            m_start = m_low - 1
        for J in range(m_start, m_high):
            num, W = linsolv(np.ascontiguousarray(VJ[:, J - 1]))
            info["qmr_iters"].append(num)
            if num <= 0:
                return num
            if not (cgs2_orth(W, J, VJ) if orth else mgs_orth(W, J, VJ)):
                return -J
        for J in range(m_low, m_high + 1):
            vj = np.ascontiguousarray(VJ[:, J - 1])
            W = _f64(h0x(vj))
            for I in range(1, m_high + 1):
                vi = np.ascontiguousarray(VJ[:, I - 1])
                HMAT[I - 1, J - 1] = lib().orc_dot(N, _p(vi), _p(W))
                HMAT[J - 1, I - 1] = HMAT[I - 1, J - 1]
        return m_high

    while cnt_high <= m_max:
        rc = pisth0(cnt_low, cnt_high)
        if rc < 0:
            return -cnt_high, eig, res, info
        num = cnt_high - stepeig
        tmp = np.linalg.eigvalsh(HMAT[:num, :num], UPLO="U")
        old = get_window(E0, tmp, M)
        num = cnt_high
        tmp = np.linalg.eigvalsh(HMAT[:num, :num], UPLO="U")
        eig = get_window(E0, tmp, M)
        res = get_diff_max(eig, old) if ntype <= 0 else get_sep_max(old, tmp[:cnt_high])
        info["steps"].append((cnt_high, res))
        if log:
            log(f"Cnt1={cnt_high} Cnt2={cnt_high - stepeig} RES={res}")
        if res <= etol:
            status = cnt_high
            break
        status = -cnt_high
        cnt_low = cnt_high + 1
        if cnt_low >= m_max:
            status = -m_max
            break
        cnt_high = min(cnt_high + stepcnt, m_max)
    info["hmat"] = HMAT[:cnt_high, :cnt_high].copy()
    return status, np.sort(eig), res, info


def pist_params(M0, conv):
    """setPISTConvParam (src/iterate/module/osbw.pistconv.h:303-333).

    ``conv`` = (mE0, mTol, mStart, mStep, mMax, mNum, mGap)."""
    mE0, mTol, mStart, mStep, mMax, _mNum, mGap = conv
    start = 2 * M0 if mStart < M0 else mStart
    step = 5 if mStep < 1 else mStep
    eigstep = 1 if mGap < 1 else mGap
    nmax = start + M0 if mMax < start else mMax
    return dict(E0=mE0, etol=mTol, startcnt=start, stepcnt=step, stepeig=eigstep, m_max=nmax)


def start_vector(N, seed=0):
    """Seeded uniform(0,1) start vector standing in for ``random_number(X)``
    (osbw.pistconv.h:35)."""
    return np.random.default_rng(seed).random(N)


# ----------------------------------------------------------------------------------
# OSBW window preconditioner (sOSB = TOSBW = 4), bound-state (real) form
# ----------------------------------------------------------------------------------
TOSBW = 4


def osbw_size(EIG0, E0, DE):
    """getOSBWSize (src/iterate/module/osb.osbw.h:62-73): states with |EIG0 - E0| <= DE."""
    return int(np.count_nonzero(np.abs(np.asarray(EIG0) - E0) <= DE))


def osbw_adjust(EIG0, E0, count, de, max_iter=2000):
    """adjustWinSize (osb.osbw.h:118-145): doubles DE while the window holds
    fewer than ``count`` states and bisects between the last two widths while
    it holds more, until it holds exactly ``count``.  The reference loops
    without a bound (forever when no width gives exactly ``count`` states,
    e.g. tied EIG0 values, or when DE starts at 0); this restatement raises
    ValueError after ``max_iter`` steps instead."""
    EIG0 = np.asarray(EIG0, dtype=np.float64)
    de1 = 0.0
    cnt0 = osbw_size(EIG0, E0, de)
    it = 0
    while cnt0 != count:
        if cnt0 < count:
            de1 = de
            de = 2.0 * de
        else:
            de = 0.5 * (de1 + de)
        cnt0 = osbw_size(EIG0, E0, de)
        it += 1
        if it > max_iter:
            raise ValueError(f"no window width holds exactly {count} states")
    return de


def osbw_index(EIG0, E0, DE):
    """getOSBWIndex (osb.osbw.h:76-92): the window's grid indices in ascending
    order (0-based here; the reference's are 1-based)."""
    return np.nonzero(np.abs(np.asarray(EIG0) - E0) <= DE)[0]


def osbw_level_index(sizes, ind):
    """getLevelIndex (src/iterate/module/osb.vi.h:11-27): per level l the block
    bk (the combined coordinates of the slower levels) and the column col
    (the level-l coordinate) of each window state, both 0-based, shape
    (len(sizes), len(ind))."""
    sizes = np.asarray(sizes, dtype=np.int64)
    dim = np.cumprod(np.concatenate(([1], sizes[:-1])))
    clen = dim * sizes
    ind = np.asarray(ind, dtype=np.int64)
    bk = ind[None, :] // clen[:, None]
    col = (ind[None, :] - bk * clen[:, None]) // dim[:, None]
    return bk, col


def vosb_starts(sizes):
    """myVOSB%mStart (src/iterate/module/osb.init.h:37): level l's blocks of
    sN(l) x sN(l) start after the lower levels' myBlk(l) sN(l)^2 entries."""
    sizes = list(sizes)
    vs, v = [], 0
    for l, n in enumerate(sizes):
        vs.append(v)
        v += int(np.prod(sizes[l + 1:], dtype=np.int64)) * n * n
    return vs


def osbw_vi(sizes, VOSB, bk, col):
    """getLevelVi / getVi (osb.vi.h:38-80): the preconditioner's basis vector of
    one state, V_sF..V_1 applied to the unit vector -- a Kronecker product of
    one column per level, v_sF x ... x v_1 (level 1 fastest), built in the
    reference's order (level 1 first, each level multiplying the previous)."""
    vs = vosb_starts(sizes)
    Vi = np.ones(1)
    for l, n in enumerate(sizes):
        off = vs[l] + int(bk[l]) * n * n + int(col[l]) * n
        Vi = np.kron(VOSB[off:off + n], Vi)
    return Vi


def osbw_hij(op, ind):
    """getVOSBH0 (src/iterate/module/osb.hij.h:128-159): Hij(I, J) = Vi . (H Vj)
    for I < J with H = MYHX(TA0) (HijX, osb.hx.h:29-36), mirrored, and
    Hij(I, I) = EIG0(ind(I)).  H Vj is formed once per J (the reference forms
    it again for every I; the values are the same)."""
    m = len(ind)
    bk, col = osbw_level_index(op.sizes, ind)
    vec = [osbw_vi(op.sizes, op.VOSB, bk[:, i], col[:, i]) for i in range(m)]
    H = np.zeros((m, m))
    for J in range(m):
        hv = op.hx(vec[J], 0)
        for I in range(J):
            H[I, J] = lib().orc_dot(op.N, _p(vec[I]), _p(hv))
            H[J, I] = H[I, J]
    for I in range(m):
        H[I, I] = op.EIG0[ind[I]]
    return H


class OSBW:
    """initOSBW for the bound-state job (osb.osbw.h:2-50 with getOSBWH through
    getVOSBH0, and createWH, src/iterate/module/osb.pij.h:6-45): the window
    of ``count`` states around E0, its matrix HW, and HWR = HW - shift I
    (shift = E0 for TA1, 0 for TA0) factored by LAPACK DSYTRF('U')."""

    def __init__(self, op, E0, count, de, npc=1, HW=None):
        from scipy.linalg import lapack
        if de <= 0.0:
            raise ValueError("window width must be positive")
        self.E0 = float(E0)
        self.de = osbw_adjust(op.EIG0, E0, int(count), float(de))
        self.ind = osbw_index(op.EIG0, E0, self.de)
        if self.ind.size == 0:
            raise ValueError("empty window")
        self.HW = osbw_hij(op, self.ind) if HW is None else np.array(HW, dtype=np.float64)
        HWR = self.HW.copy()
        if npc != 0:
            HWR[np.diag_indices_from(HWR)] -= self.E0
        m = self.ind.size
        self.ldu, self.ipiv, info = lapack.dsytrf(HWR, lower=0, lwork=6 * m)
        if info != 0:
            raise ValueError(f"DSYTRF info={info}")
        self.HWR = HWR

    def solve(self, wy):
        """DSYTRS('U', hwLen, 1, HWR, WIPIV, WY) (osb.px.h:196-199)."""
        from scipy.linalg import lapack
        x, info = lapack.dsytrs(self.ldu, self.ipiv, np.asarray(wy, dtype=np.float64), lower=0)
        if info != 0:
            raise ValueError(f"DSYTRS info={info}")
        return x


def osbw_px(op, win, X, npc=1):
    """MYPX with the TOSBW kernel (src/iterate/module/osb.px.h:125-148,191-206,
    213-219): V^T of levels sF..1, the window entries WY = Y(WIND) solved
    with the factored HWR, every other entry divided by EIG0 - E0, then V of
    levels 1..sF."""
    sizes = op.sizes
    vs = vosb_starts(sizes)
    dims = np.cumprod((1,) + sizes[:-1])
    Y = _f64(X).copy()
    nlev = len(sizes)
    for l in range(nlev - 1, -1, -1):
        blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
        lib().orc_vtx(int(dims[l]), sizes[l], blk, _p(op.VOSB[vs[l]:]), _p(Y))
    E0 = 0.0 if npc == 0 else op.E0
    wy = win.solve(Y[win.ind])
    Y = Y / (op.EIG0 - E0)
    Y[win.ind] = wy
    for l in range(nlev):
        blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
        lib().orc_vx(int(dims[l]), sizes[l], blk, _p(op.VOSB[vs[l]:]), _p(Y))
    return Y


def osbw_qmr(op, win, B, qmrmax, qmrtol, ntype=-1, mpi_codes=True):
    """OSB_QMR with HX = MYHX(TA1) and PX = MYPX(TOSBW, TA1): returns
    (status, X, RES, iterations)."""
    N = op.N

    def hx(_ctx, n, x, y):
        xv = np.ctypeslib.as_array(x, shape=(N,))
        np.ctypeslib.as_array(y, shape=(N,))[:] = op.hx(xv.copy(), 1)

    def px(_ctx, n, x, y):
        xv = np.ctypeslib.as_array(x, shape=(N,))
        np.ctypeslib.as_array(y, shape=(N,))[:] = osbw_px(op, win, xv.copy(), 1)

    fh, fp = _OP(hx), _OP(px)
    B = _f64(B)
    X = np.zeros_like(B)
    res = C.c_double(0.0)
    it = C.c_int(0)
    rc = lib().orc_qmr(int(ntype), int(qmrmax), float(qmrtol), N, _p(B), fh, None, fp, None, _p(X),
                       C.byref(res), int(bool(mpi_codes)), C.byref(it))
    return rc, X, res.value, it.value


# ----------------------------------------------------------------------------------
# Complex forms with absorbing potentials (resonances JOB_RES1/2, CRP)
# ----------------------------------------------------------------------------------
# nType codes (src/iterate/module/osb.data.h:18-22)
TA0, TA1, TAAP0, TMAP0 = 0, 1, 2, 3
TAAP, TAAPP, TAAPR = 100, 101, 102
TMAP, TMAPP, TMAPR = 200, 201, 202

_CX_DIAG = {TA0: (False, 0, None), TA1: (True, 0, None),
            TAAP0: (False, 1, "AP"), TMAP0: (False, -1, "AP"),
            TAAP: (True, 1, "AP"), TAAPP: (True, 1, "APP"), TAAPR: (True, 1, "APR"),
            TMAP: (True, -1, "AP"), TMAPP: (True, -1, "APP"), TMAPR: (True, -1, "APR")}


def cx_terms(ntype):
    """(E0 used?, sign of i, absorbing array) of the nType: MYHX_DX's diagonal
    (src/iterate/module/osb.hxdx.h:178-215); unknown codes are (H - E0) X."""
    return _CX_DIAG.get(int(ntype), (True, 0, None))


def cx_levels(sizes, dep, ndvr, H0CX, DEPCX, OUTHCX, X):
    """The level sum of MYHX_CX (osb.hxcx.h:244-260) with complex level
    matrices: H1X_XYZ_CX / H1X_DEP_CX (hpx_cx.f90:6-34) through H1X_CX /
    H2X_CX (matrix_cx.f90:97-112, 144-159), and H3X_CX (matrix_cx.f90:194-208)
    for the outer per-point layer when sNDVR; in the reference's loop order
    (j = 1..NOUT accumulated per output column i)."""
    sizes = tuple(int(n) for n in sizes)
    nlev = len(sizes)
    N = int(np.prod(sizes))
    X = np.asarray(X, dtype=np.complex128)
    Y = np.zeros(N, dtype=np.complex128)
    h0 = 0
    dp = 0
    for l, nout in enumerate(sizes):
        nin = int(np.prod(sizes[:l], dtype=np.int64))
        blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
        Xl = X.reshape((nin, nout, blk), order="F")
        T = np.zeros((nin, nout, blk), dtype=np.complex128)
        if ndvr and l == nlev - 1:
            A = np.asarray(OUTHCX, dtype=np.complex128).reshape((nin, nout, nout), order="F")
            for i in range(nout):
                acc = A[:, i, 0] * Xl[:, 0, 0]
                for j in range(1, nout):
                    acc = acc + A[:, i, j] * Xl[:, j, 0]
                T[:, i, 0] = acc
        else:
            H = np.asarray(H0CX[h0:h0 + nout * nout], dtype=np.complex128).reshape((nout, nout), order="F")
            h0 += nout * nout
            if dep[l]:
                cor = np.asarray(DEPCX[dp:dp + nin], dtype=np.complex128)
                dp += nin
            for b in range(blk):
                for i in range(nout):
                    if dep[l]:
                        acc = H[i, 0] * cor * Xl[:, 0, b]
                        for j in range(1, nout):
                            acc = acc + H[i, j] * cor * Xl[:, j, b]
                    else:
                        acc = H[i, 0] * Xl[:, 0, b]
                        for j in range(1, nout):
                            acc = acc + H[i, j] * Xl[:, j, b]
                    T[:, i, b] = acc
        Y = Y + T.reshape(N, order="F")
    return Y


class CxOperator:
    """The real operator with absorbing potentials: AP = APP (JOB_RES1/2,
    APR = 0) or APP + APR (JOB_CRP) (loadInitData, osb.io.h:18-30,92-112).
    With set_complex_h0 the level matrices (and DEP, OUTH) are complex: the
    complex-Hamiltonian job (sCX)."""

    def __init__(self, op, APP, APR=None):
        self.op = op
        self.APP = _f64(APP)
        self.APR = np.zeros_like(self.APP) if APR is None else _f64(APR)
        self.AP = self.APP + self.APR if APR is not None else self.APP.copy()
        self.cxh = None

    def set_complex_h0(self, H0CX, DEPCX=None, OUTHCX=None):
        self.cxh = (np.asarray(H0CX, dtype=np.complex128),
                    None if DEPCX is None else np.asarray(DEPCX, dtype=np.complex128),
                    None if OUTHCX is None else np.asarray(OUTHCX, dtype=np.complex128))

    def _absorb(self, which):
        return {"AP": self.AP, "APP": self.APP, "APR": self.APR}[which]

    def hx(self, X, ntype):
        """MYHX_DX (osb.hxdx.h:178-240): Y = (RES - E0 [+-] i A) X + sum_level H_level X
        with the real level matrices applied to the real and imaginary parts."""
        use_e0, sign, which = cx_terms(ntype)
        X = np.asarray(X, dtype=np.complex128)
        nt = 1 if use_e0 else 0
        if self.cxh is not None:
            # MYHX_CX (osb.hxcx.h:191-261): the real diagonal, then the complex levels
            op = self.op
            Y = (op.RES - (op.E0 if use_e0 else 0.0)) * X
            Y = Y + cx_levels(op.sizes, op.dep, op.ndvr, self.cxh[0], self.cxh[1], self.cxh[2], X)
        else:
            Y = self.op.hx(X.real.copy(), nt) + 1j * self.op.hx(X.imag.copy(), nt)
        if sign:
            Y = Y + 1j * sign * self._absorb(which) * X
        return Y

    def _kernel(self, ntype, E0):
        use_e0, sign, which = cx_terms(ntype)
        e0 = E0 if ntype not in (TA0, TAAP0, TMAP0) else 0.0
        return e0, sign, (self._absorb(which) if sign else None)

    def px(self, X, nosb=1, ntype=TA1, de=0.0, beta=0.0, win=None):
        """MYPX_DX (src/iterate/module/osb.mypxdx.h): V^T of levels sF..1 on the
        real and imaginary parts, the complex kernel, V of levels 1..sF.
        TOSB divides by EIG0 - E0 [+-] i A; TOSBD1 clamps |EIG0 - E0| <= DE to
        +-DE first; TOSBD2 maps it to alpha + beta (EIG0 - E0) on both sides of
        E0 (the complex form has the same expression in both branches, unlike
        the real TOSBD2 of osb.px.h:174-189)."""
        op = self.op
        sizes = op.sizes
        vs = vosb_starts(sizes)
        dims = np.cumprod((1,) + sizes[:-1])
        nlev = len(sizes)

        def rot(y, transpose):
            yr, yi = _f64(y.real).copy(), _f64(y.imag).copy()
            order = range(nlev - 1, -1, -1) if transpose else range(nlev)
            for l in order:
                blk = int(np.prod(sizes[l + 1:], dtype=np.int64))
                f = lib().orc_vtx if transpose else lib().orc_vx
                f(int(dims[l]), sizes[l], blk, _p(op.VOSB[vs[l]:]), _p(yr))
                f(int(dims[l]), sizes[l], blk, _p(op.VOSB[vs[l]:]), _p(yi))
            return yr + 1j * yi

        Y = rot(np.asarray(X, dtype=np.complex128), True)
        e0, sign, A = self._kernel(ntype, op.E0)
        ade = op.EIG0 - e0
        DE = abs(de)
        if nosb == 2:                                   # TOSBD1
            inside = np.abs(ade) <= DE
            ade = np.where(inside, np.where(ade < 0.0, -DE, DE), ade)
        elif nosb == 3:                                 # TOSBD2
            b1 = beta + 1.0
            alpha = -beta * DE
            inside = np.abs(ade) <= DE
            ade = np.where(inside, alpha + b1 * ade, ade)
        elif nosb == TOSBW and win is None:
            raise ValueError("TOSBW needs the window (an OSBW object)")
        den = ade + 1j * sign * A if sign else ade
        if nosb == TOSBW:
            wy = np.linalg.solve(self.window_matrix(win, ntype, e0), Y[win.ind])
            Y = Y / den
            Y[win.ind] = wy
        else:
            Y = Y / den
        return rot(Y, False)

    def window_matrix(self, win, ntype, e0):
        """HWRCX of createWH_DXCX (src/iterate/module/osb.pij.h:63-135): the
        window matrix HW with -E0 (nTypes that use E0) and +-i A(WIND) added
        on the diagonal; MYPX_DX (osb.mypxdx.h) solves with it by ZGETRF /
        ZGETRS (ZHETRF / ZHETRS for TA0, TA1).  For TA1 the reference reads the
        diagonal from HWCX, the complex job's array, which the real job does
        not fill; this uses HW, the evident intent."""
        use_e0, sign, which = cx_terms(ntype)
        A = np.array(win.HW, dtype=np.complex128)
        d = np.diag_indices_from(A)
        if ntype not in (TA0, TAAP0, TMAP0):
            A[d] -= e0
        if sign:
            A[d] += 1j * sign * self._absorb(which)[win.ind]
        return A


def qmr_cx(hx, px, B, qmrmax, qmrtol, ntype=0, X0=None):
    """QMR_CX (src/iterate/libiterate/qmr/qmrcx.f90:4-175): QMR for complex
    symmetric systems, bilinear products DOT_CX = X^T Y (vector_cx.f90:227-234),
    norms from the conjugated dot_product.  Returns (code, X, RES)."""
    B = np.asarray(B, dtype=np.complex128)
    n = B.size
    X = np.zeros(n, np.complex128) if (ntype <= 0 or X0 is None) else np.asarray(X0, np.complex128).copy()
    nrm = lambda v: np.sqrt(abs(np.vdot(v, v)))
    zvrat = 1.0
    R = B.copy()
    V = B.copy()
    bnrm = nrm(B)
    vnrm = bnrm
    Z = px(B)
    znrm = nrm(Z)
    gamamo, eta = 1.0, -1.0
    code, res = 0, 0.0
    Q = S = UX = UR = None
    qsdot = 0.0
    thetamo = 0.0
    for i in range(1, qmrmax + 1):
        if vnrm == 0.0 or znrm == 0.0:
            break
        zvrat = zvrat * znrm / vnrm
        V = V / vnrm
        Z = Z / znrm
        vzdot = np.sum(V * Z)
        if abs(vzdot) == 0.0:
            break
        Q = Z.copy() if i == 1 else Z - (vnrm * vzdot) / qsdot * Q
        S = zvrat * hx(Q)
        qsdot = np.sum(Q * S)
        beta = qsdot / vzdot
        if abs(qsdot) == 0.0 or abs(beta) == 0.0:
            break
        V = S - beta * V
        vnrmpo = nrm(V)
        Z = px(V) / zvrat
        znrm = nrm(Z)
        theta = vnrmpo / (gamamo * abs(beta))
        gama = 1.0 / np.sqrt(1.0 + theta * theta)
        eta = -eta * vnrm * gama * gama / (beta * gamamo * gamamo)
        if gama == 0.0:
            break
        if i == 1:
            UX = eta * zvrat * Q
            UR = eta * S
        else:
            UX = (eta * zvrat) * Q + ((thetamo * gama) ** 2) * UX
            UR = eta * S + ((thetamo * gama) ** 2) * UR
        X = X + UX
        R = R - UR
        if abs(ntype) == 1:
            HX0 = hx(X)
            res = nrm(HX0 - B) / nrm(HX0)
        elif abs(ntype) == 2:
            res = max(nrm(R) / bnrm, np.sqrt(abs(np.vdot(UX, UX) / np.vdot(X, X))),
                      np.sqrt(abs(np.vdot(UR, UR) / np.vdot(R, R))))
        else:
            res = nrm(R) / bnrm
        if abs(res) < qmrtol:
            code = i
            break
        code = -i
        vnrm, gamamo, thetamo = vnrmpo, gama, theta
    return code, X, res


# ----------------------------------------------------------------------------------
# Complex symmetric PIST (PIST_CONV_SX) and its helpers
# ----------------------------------------------------------------------------------
def get_op_cx(ntype, vec):
    """getOpCX (src/libutil/serial/base/util_cx.f90:375-420): the real value a
    complex number is compared by."""
    v = np.asarray(vec, dtype=np.complex128)
    re, im = v.real, v.imag
    ops = {1: re, 2: np.abs(re), 3: im, 4: np.abs(im), 5: np.abs(re) + np.abs(im),
           6: re ** 2 + im ** 2, 7: re + im, 8: np.abs(re + im), 9: re - im, 10: im - re,
           11: np.abs(im - re), 12: np.abs(re) - np.abs(im), 13: np.abs(im) - np.abs(re),
           14: np.abs(np.abs(im) - np.abs(re)), 15: np.abs(re) ** 2 - np.abs(im) ** 2}
    return np.array(ops[int(ntype)], dtype=np.float64)


def get_window_index(E0, vec, M):
    """getWindow0 (util.f90:669-716) returning the picked indices."""
    vec = np.asarray(vec, dtype=np.float64)
    n = vec.size
    if n < M:
        return np.concatenate([np.arange(n), np.full(M - n, n - 1)])
    absv = np.abs(vec - E0)
    label = np.ones(n, dtype=bool)
    out = np.empty(M, dtype=np.int64)
    for i in range(M):
        out[i] = int(np.argmin(np.where(label, absv, np.inf)))
        label[out[i]] = False
    return out


def get_window_cx(E0, ntype, vec, M):
    """getWindow_CX (util_cx.f90:301-325): the window of getWindow0 on getOpCX."""
    vec = np.asarray(vec, dtype=np.complex128)
    return vec[get_window_index(E0, get_op_cx(ntype, vec), M)]


def get_diff_max_cx(ntype, v1, v2):
    """getDiffMax_CX (util_cx.f90:33-43)."""
    return get_diff_max(get_op_cx(ntype, v1), get_op_cx(ntype, v2))


def reorder_cx(ntype, vec):
    """ReOrder_CX('A', ...) (util_cx.f90:187-214): ascending by getOpCX."""
    vec = np.asarray(vec, dtype=np.complex128)
    return vec[np.argsort(get_op_cx(ntype, vec), kind="stable")]


def dot_cx(x, y):
    """DOT_CX (vector_cx.f90:227-234): the bilinear X^T Y."""
    return complex(np.sum(np.asarray(x) * np.asarray(y)))


def mgs_orth_cx(W, m, VJ):
    """MGS_ORTH_CX (src/iterate/libiterate/orth/gsorth_cx.f90:51-79): the same
    in the conjugated product, normalised by the real norm."""
    v = np.asarray(W, dtype=np.complex128).copy()
    for i in range(m):
        v = v - np.vdot(VJ[:, i], v) * VJ[:, i]
    nrm = np.sqrt(np.real(np.vdot(v, v)))
    if nrm == 0.0:
        return False
    VJ[:, m] = v / nrm
    return True


def mgs_orth_sx(W, m, VJ):
    """MGS_ORTH_SX (src/iterate/libiterate/orth/gsorth_sx.f90:47-72): modified
    Gram-Schmidt in the bilinear product, column m of VJ (0-based) from W,
    normalised by the principal square root of W^T W."""
    v = np.asarray(W, dtype=np.complex128).copy()
    for i in range(m):
        v = v - dot_cx(VJ[:, i], v) * VJ[:, i]
    nrm = np.sqrt(dot_cx(v, v))
    if nrm == 0.0:
        return False
    VJ[:, m] = v / nrm
    return True


def pisth0_sx(X, m_max, m_low, m_high, h0x, linsolv, VJ, HMAT, conj=False):
    """pistH0_SX (src/iterate/libiterate/pist/pistHij_sx.f90:62-118); with conj,
    pistH0_CX (pistHij_cx.f90) in the conjugated product."""
    dot = (lambda a, b: complex(np.vdot(a, b))) if conj else dot_cx
    orth = mgs_orth_cx if conj else mgs_orth_sx
    if m_low < 1 or m_low >= m_high or m_high > m_max:
        return 0
    if m_low == 1:
        m_start = 1
        t = np.sqrt(np.real(np.vdot(X, X))) if conj else np.sqrt(dot_cx(X, X))
        if t == 0.0:
            return 0
        VJ[:, 0] = np.asarray(X, dtype=np.complex128) / t
    else:
        m_start = m_low - 1
    for J in range(m_start, m_high):
        num, WJ = linsolv(VJ[:, J - 1])
        if num <= 0:
            return num
        if not orth(WJ, J, VJ):
            return -J
    for J in range(m_low, m_high + 1):
        WJ = h0x(VJ[:, J - 1])
        for I in range(1, m_high + 1):
            HMAT[I - 1, J - 1] = dot(VJ[:, I - 1], WJ)
    for J in range(1, m_low):
        WJ = h0x(VJ[:, J - 1])
        for I in range(m_low, m_high + 1):
            HMAT[I - 1, J - 1] = dot(VJ[:, I - 1], WJ)
    return m_high


def pist_conv_sx(E0, etol, ntype, x, startcnt, stepcnt, stepeig, M, m_max, h0x, linsolv, conj=False):
    """PIST_CONV_SX (src/iterate/libiterate/pist/pist_sx.f90:4-96): PIST for a
    complex symmetric operator.  The eigenvalues of HMAT come from ZGEEV
    (numpy's eigvals is LAPACK's ZGEEV), the window and the final order use
    the real part, the convergence test |lambda|^2 (getOpCX types 1 and 6).
    ntype > 0 is not restated: the reference calls getSepMax_CX with five
    arguments (an integer where a complex array is expected), which has no
    defined result.  With conj this is PIST_CONV_CX (pist/pist_cx.f90): the
    same steps in the conjugated product.  Returns (status, eig[M], RES)."""
    if ntype > 0:
        raise ValueError("PIST_CONV_SX with ntype > 0 has no defined result in the reference")
    n_diff, n_conv = 1, 6
    if stepeig >= m_max or startcnt > m_max or M > m_max:
        return 0, np.zeros(M, np.complex128), 0.0
    N = len(x)
    VJ = np.zeros((N, m_max), np.complex128)
    HMAT = np.zeros((m_max, m_max), np.complex128)
    cnt_low, cnt_high = 1, max(startcnt, M, stepeig + 1)
    status, res, eig = 0, 0.0, np.zeros(M, np.complex128)
    while cnt_high <= m_max:
        num = pisth0_sx(x, m_max, cnt_low, cnt_high, h0x, linsolv, VJ, HMAT, conj)
        if num <= 0:
            return -cnt_high, eig, res
        n1 = cnt_high - stepeig
        old = get_window_cx(E0, n_diff, np.linalg.eigvals(HMAT[:n1, :n1]), M)
        eig = get_window_cx(E0, n_diff, np.linalg.eigvals(HMAT[:cnt_high, :cnt_high]), M)
        res = get_diff_max_cx(n_conv, eig, old)
        if res <= etol:
            status = cnt_high
            break
        status = -cnt_high
        cnt_low = cnt_high + 1
        if cnt_low >= m_max:
            status = -m_max
            break
        cnt_high = min(cnt_high + stepcnt, m_max)
    return status, reorder_cx(n_diff, eig), res


# ----------------------------------------------------------------------------------
# Cumulative reaction probability (osbCRP, src/iterate/module/osbw.crp.h)
# ----------------------------------------------------------------------------------
def lan_dx(x, M, hx):
    """LAN_DX (src/iterate/libiterate/lanczos/lan_dx.f90:299-325) with lanHij_dx
    (lanHij_dx.f90:59-97) and LAN_MGS_ORTH_CX (orth/gsorth_cx.f90:132-160):
    Lanczos for a Hermitian operator on complex vectors with full
    re-orthogonalisation in the conjugated product, then DSTEV on the
    tridiagonal.  Returns (status, eig)."""
    from scipy.linalg import lapack
    x = np.asarray(x, dtype=np.complex128)
    n = x.size
    t = np.sqrt(np.real(np.vdot(x, x)))
    if t == 0.0:
        return 0, None
    VJ = np.zeros((n, M + 1), np.complex128)
    VJ[:, 0] = x / t
    alpha = np.zeros(M)
    beta = np.zeros(M)
    for J in range(1, M + 1):
        w = hx(VJ[:, J - 1])
        if J != 1:
            w = w - beta[J - 2] * VJ[:, J - 2]
        alpha[J - 1] = np.real(np.vdot(w, VJ[:, J - 1]))
        v = w.copy()
        for I in range(1, J + 1):
            v = v - np.vdot(VJ[:, I - 1], v) * VJ[:, I - 1]
        nrm = np.sqrt(np.real(np.vdot(v, v)))
        beta[J - 1] = nrm
        if nrm == 0.0:
            return -J, None
        VJ[:, J] = v / nrm
    d, _, info = lapack.dstev(alpha, beta[:M - 1], compute_v=0)
    if info != 0:
        return -M, None
    return M, d


def crp_operator(cx, E, qmrmax, qmrtol, sap=True, conv=0):
    """CRP_HXDX (osbw.crp.h:71-101) at energy E: y = sqrt(APR) x, solved with
    (H - E - i AP), times APP, solved with (H - E + i AP), times sqrt(APR).
    The preconditioner carries the absorbing potential when sAP is set
    (sPC = TMAP / TAAP), the real kernel otherwise (sPC = TA1)."""
    op = cx.op
    op.set_e0(E)
    sq = np.sqrt(cx.APR)
    pm, pp = (TMAP, TAAP) if sap else (TA1, TA1)

    def apply(x):
        y = sq * x
        _, t, _ = qmr_cx(lambda u: cx.hx(u, TMAP), lambda u: cx.px(u, 1, pm), y, qmrmax, qmrtol, conv)
        y = cx.APP * t
        _, t, _ = qmr_cx(lambda u: cx.hx(u, TAAP), lambda u: cx.px(u, 1, pp), y, qmrmax, qmrtol, conv)
        return sq * t
    return apply


def osb_crp(cx, energies, NM, x0s, qmrmax, qmrtol, sap=True, conv=0):
    """osbCRP / calOSBCRP (osbw.crp.h:6-68): N(E) = 4 sum of the NM Lanczos
    eigenvalues of the CRP operator from the start vector x0s[i] (the
    reference draws it with randMat_CX); 0 when the Lanczos fails."""
    out = np.zeros(len(energies))
    for i, E in enumerate(energies):
        st, eig = lan_dx(x0s[i], NM, crp_operator(cx, float(E), qmrmax, qmrtol, sap, conv))
        out[i] = 4.0 * float(np.sum(eig)) if st > 0 else 0.0
    return out
