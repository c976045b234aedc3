"""Synthetic triatomic Jacobi-DVR Hamiltonians in the layout the iterate stage reads.

The reference's stage 2 (``src/ham/ja3``) writes the per-level 1-D kinetic
matrices (the ``H0`` file), the diagonal potential (``RES``) and the
coordinate-dependent factor of the angular term (``DEP``).  The iterate stage
then applies

    H = V(r,R,theta) + K_r (x) 1 + 1 (x) K_R (x) 1 + c(r,R) * K_theta

on the direct-product grid.  This module produces those arrays for the
workloads this package is measured on:

* level 1 = r, level 2 = R, level 3 = theta (``src/ham/ja3/module/ja3.data:10-11``:
  the outermost layer is the angle; the linear index is
  ``p = i_r + n_r*i_R + n_r*n_R*i_theta``, column-major as in Fortran);
* radial kinetic matrices: particle-in-a-box sine DVR on ``[a, b]`` with ``n``
  interior points (Colbert & Miller, JCP 96, 1982 (1992), appendix A; the
  reference cites the same paper for its sinc DVR, ``src/ham/libham/dvr/sinc.f90:4``);
* angular kinetic matrix: Gauss-Legendre DVR, ``K_theta = T diag(j(j+1)) T^T``
  with ``T[a, j] = sqrt(w_a) * Pbar_j(x_a)`` and ``Pbar_j`` the normalised Legendre
  polynomial (nodes and normalisation as ``src/ham/libham/poly/gauLege.f90:54-100``
  and ``src/ham/libham/poly/yjm.f90:16-48``);
* ``c(r,R) = 1/(2 mu_R R^2) + 1/(2 mu_r r^2)`` (cf. ``mR0 = 0.5/(ma R^2)``,
  ``src/ham/ja3/module/ja3.h0dvr:63``), the DEP array of level 3;
* potential: Morse(R) + Morse(r) + sum_l A_l P_l(cos theta) exp(-((R-Rc)/w_l)^2),
  capped at ``vcap`` Hartree.

Everything is float64 and deterministic; no random numbers are involved.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# Hartree -> cm^-1, the constant the reference uses (src/ham/libham/dvr/sinc.f90:27).
HARTREE_CM = 8.06554477e3 * 27.2114


@dataclasses.dataclass(frozen=True)
class PES:
    """Analytic triatomic potential with 12 parameters (Hartree, bohr).

    V = De_R (1 - exp(-a_R (R - Re)))^2 + De_r (1 - exp(-a_r (r - re)))^2
        + sum_{l=1..3} A_l P_l(cos theta) exp(-((R - rc) / w_l)^2),
    then capped at ``vcap``.
    """

    de_R: float = 0.01
    a_R: float = 1.0
    re_R: float = 4.0
    de_r: float = 0.2
    a_r: float = 1.2
    re_r: float = 2.2
    amp1: float = 0.0
    amp2: float = 0.002
    amp3: float = 0.0
    width1: float = 1.0
    width2: float = 1.0
    width3: float = 1.0
    rc: float = 4.0
    vcap: float = 0.5

    PARAM_NAMES = ("de_R", "a_R", "re_R", "de_r", "a_r", "re_r",
                   "amp1", "amp2", "amp3", "width1", "width2", "width3")

    def params(self) -> np.ndarray:
        return np.array([getattr(self, k) for k in self.PARAM_NAMES], dtype=np.float64)

    def with_params(self, vec) -> "PES":
        kw = {k: float(v) for k, v in zip(self.PARAM_NAMES, vec)}
        return dataclasses.replace(self, **kw)


@dataclasses.dataclass(frozen=True)
class Grid3:
    """A triatomic direct-product grid: sizes, ranges and reduced masses."""

    n_r: int
    n_R: int
    n_th: int
    r_range: tuple = (1.5, 4.0)
    R_range: tuple = (2.0, 8.0)
    mu_r: float = 14582.6
    mu_R: float = 14582.6

    @property
    def sizes(self):
        return (self.n_r, self.n_R, self.n_th)

    @property
    def npoints(self) -> int:
        return self.n_r * self.n_R * self.n_th


# Workloads (sizes, ranges, masses and potential) the package is exercised on.
WORKLOADS = {
    # 15,360 points, 20 lowest levels: the CPU-runnable plain FP64 case.
    "tri-24x32x20": (Grid3(24, 32, 20), PES()),
    # 589,824 points, 100 levels: plain FP64 on the GPU.
    "tri-96x96x64": (Grid3(96, 96, 64), PES()),
    # 3,072,000 points, P2 amplitude 0.005 Eh: the precision form, 200 levels.
    "tri-160x160x120": (Grid3(160, 160, 120), PES(amp2=0.005)),
    # 1,572,864 points: the differentiation form (all three anisotropy terms on,
    # so every one of the 12 parameters moves the levels).
    "tri-128x128x96": (Grid3(128, 128, 96), PES(amp1=0.001, amp3=0.0005, width1=1.2, width3=0.8)),
}


def sine_dvr(n: int, a: float, b: float, mass: float):
    """Particle-in-a-box sine DVR on ``[a, b]`` with ``n`` interior points.

    Returns ``(x, T)``: grid points ``x_i = a + i (b-a)/(n+1)`` and the kinetic
    matrix ``T = U diag(k^2 pi^2 / (2 m L^2)) U^T`` with the orthogonal DVR
    transform ``U[i, k] = sqrt(2/(n+1)) sin(i k pi/(n+1))``.
    """
    L = b - a
    i = np.arange(1, n + 1, dtype=np.float64)
    x = a + i * L / (n + 1)
    U = math.sqrt(2.0 / (n + 1)) * np.sin(np.outer(i, i) * math.pi / (n + 1))
    eps = (i * math.pi / L) ** 2 / (2.0 * mass)
    T = (U * eps) @ U.T
    T = 0.5 * (T + T.T)
    return x, T


def sine_dvr_closed_form(n: int, a: float, b: float, mass: float):
    """Closed-form sine-DVR kinetic matrix (Colbert & Miller appendix A).

    Used only to cross-check :func:`sine_dvr`.
    """
    L = b - a
    m1 = n + 1
    pre = (1.0 / (2.0 * mass)) * (math.pi / L) ** 2 / 2.0
    T = np.empty((n, n))
    for i in range(1, n + 1):
        for j in range(1, n + 1):
            if i == j:
                T[i - 1, j - 1] = pre * ((2.0 * m1 * m1 + 1.0) / 3.0
                                         - 1.0 / math.sin(math.pi * i / m1) ** 2)
            else:
                T[i - 1, j - 1] = pre * (-1.0) ** (i - j) * (
                    1.0 / math.sin(math.pi * (i - j) / (2 * m1)) ** 2
                    - 1.0 / math.sin(math.pi * (i + j) / (2 * m1)) ** 2)
    return T


def legendre_dvr(n: int):
    """Gauss-Legendre DVR for the Jacobi angle (J = 0).

    Returns ``(x, w, T, K)``: nodes ``x = cos(theta)`` (ascending), weights,
    the orthogonal transform ``T[a, j] = sqrt(w_a) Pbar_j(x_a)`` (j = 0..n-1)
    and ``K = T diag(j (j+1)) T^T`` (the j^2 operator in the DVR).
    """
    x, w = np.polynomial.legendre.leggauss(n)
    P = np.empty((n, n))
    P[:, 0] = 1.0
    if n > 1:
        P[:, 1] = x
    for j in range(2, n):
        P[:, j] = ((2 * j - 1) * x * P[:, j - 1] - (j - 1) * P[:, j - 2]) / j
    jj = np.arange(n, dtype=np.float64)
    Pbar = P * np.sqrt((2.0 * jj + 1.0) / 2.0)
    T = np.sqrt(w)[:, None] * Pbar
    K = (T * (jj * (jj + 1.0))) @ T.T
    K = 0.5 * (K + K.T)
    return x, w, T, K


def legendre_p(l: int, x):
    if l == 0:
        return np.ones_like(x)
    if l == 1:
        return x
    if l == 2:
        return 0.5 * (3.0 * x * x - 1.0)
    if l == 3:
        return 0.5 * (5.0 * x ** 3 - 3.0 * x)
    raise ValueError(l)


def potential(r, R, c, pes: PES):
    """V(r, R, cos theta) on broadcastable arrays (Hartree)."""
    v = pes.de_R * (1.0 - np.exp(-pes.a_R * (R - pes.re_R))) ** 2
    v = v + pes.de_r * (1.0 - np.exp(-pes.a_r * (r - pes.re_r))) ** 2
    for l, (amp, wid) in enumerate(((pes.amp1, pes.width1), (pes.amp2, pes.width2),
                                    (pes.amp3, pes.width3)), start=1):
        if amp != 0.0:
            v = v + amp * legendre_p(l, c) * np.exp(-((R - pes.rc) / wid) ** 2)
    return np.minimum(v, pes.vcap)


def potential_grad(r, R, c, pes: PES):
    """dV/dp for the 12 PES parameters (same order as ``PES.PARAM_NAMES``).

    Points where the cap is active have zero gradient.
    """
    eR = np.exp(-pes.a_R * (R - pes.re_R))
    er = np.exp(-pes.a_r * (r - pes.re_r))
    g = []
    g.append((1.0 - eR) ** 2)
    g.append(2.0 * pes.de_R * (1.0 - eR) * eR * (R - pes.re_R))
    g.append(-2.0 * pes.de_R * (1.0 - eR) * eR * pes.a_R)
    g.append((1.0 - er) ** 2)
    g.append(2.0 * pes.de_r * (1.0 - er) * er * (r - pes.re_r))
    g.append(-2.0 * pes.de_r * (1.0 - er) * er * pes.a_r)
    amps = (pes.amp1, pes.amp2, pes.amp3)
    wids = (pes.width1, pes.width2, pes.width3)
    gauss = [np.exp(-((R - pes.rc) / w) ** 2) for w in wids]
    for l in range(3):
        g.append(legendre_p(l + 1, c) * gauss[l])
    for l in range(3):
        g.append(amps[l] * legendre_p(l + 1, c) * gauss[l]
                 * 2.0 * (R - pes.rc) ** 2 / wids[l] ** 3)
    vraw = potential(r, R, c, dataclasses.replace(pes, vcap=np.inf))
    mask = vraw < pes.vcap
    return [np.broadcast_to(gi * mask, np.broadcast(r, R, c).shape) for gi in g]


@dataclasses.dataclass
class Problem:
    """Arrays of one problem in the reference's layout (all float64)."""

    sizes: tuple            # sN = (n_r, n_R, n_theta)
    dep: tuple              # sDEP per level
    H0: np.ndarray          # concatenation of the sN(l)^2 column-major level matrices
    RES: np.ndarray         # diagonal potential, length N
    DEP: np.ndarray         # concatenation of myDim(l) factors for dependent levels
    grids: dict             # r, R, cos(theta), weights (for reference only)
    pes: PES
    grid: Grid3

    @property
    def N(self) -> int:
        return int(np.prod(self.sizes))

    def level_matrix(self, level: int) -> np.ndarray:
        """The 1-based ``level``'s kinetic matrix as an (n, n) array."""
        off = 0
        for l in range(level - 1):
            off += self.sizes[l] ** 2
        n = self.sizes[level - 1]
        return self.H0[off:off + n * n].reshape(n, n, order="F")


def build_problem(grid: Grid3, pes: PES = PES()) -> Problem:
    r, Kr = sine_dvr(grid.n_r, *grid.r_range, grid.mu_r)
    R, KR = sine_dvr(grid.n_R, *grid.R_range, grid.mu_R)
    c, w, _, Kt = legendre_dvr(grid.n_th)
    H0 = np.concatenate([Kr.ravel(order="F"), KR.ravel(order="F"), Kt.ravel(order="F")])
    # DEP for level 3: length myDim(3) = n_r * n_R, r fastest.
    cdep = (1.0 / (2.0 * grid.mu_R * R[None, :] ** 2)
            + 1.0 / (2.0 * grid.mu_r * r[:, None] ** 2))
    DEP = cdep.ravel(order="F")
    V = potential(r[:, None, None], R[None, :, None], c[None, None, :], pes)
    RES = np.ascontiguousarray(V.ravel(order="F"))
    return Problem(sizes=grid.sizes, dep=(False, False, True), H0=H0, RES=RES,
                   DEP=DEP, grids={"r": r, "R": R, "cos_theta": c, "w": w},
                   pes=pes, grid=grid)


def workload(name: str) -> Problem:
    grid, pes = WORKLOADS[name]
    return build_problem(grid, pes)


def batched_problems(count: int = 48, seed: int = 0):
    """Uneven-size problems: n_R, n_r in [24, 96], n_theta in [16, 64], PES
    parameters of the 24x32x20 problem perturbed uniformly by +-10%."""
    rng = np.random.default_rng(seed)
    out = []
    base = PES()
    for _ in range(count):
        n_R = int(rng.integers(24, 97))
        n_r = int(rng.integers(24, 97))
        n_th = int(rng.integers(16, 65))
        f = rng.uniform(0.9, 1.1, size=7)
        pes = dataclasses.replace(base, de_R=base.de_R * f[0], a_R=base.a_R * f[1],
                                  re_R=base.re_R * f[2], de_r=base.de_r * f[3],
                                  a_r=base.a_r * f[4], re_r=base.re_r * f[5],
                                  amp2=base.amp2 * f[6])
        out.append(build_problem(Grid3(n_r, n_R, n_th), pes))
    return out


def dense_hamiltonian(p: Problem, shift: float = 0.0) -> np.ndarray:
    """Explicit N x N matrix of H - shift (Kronecker sum); small problems only."""
    n_r, n_R, n_t = p.sizes
    Kr, KR, Kt = (p.level_matrix(l) for l in (1, 2, 3))
    Ir, IR, It = np.eye(n_r), np.eye(n_R), np.eye(n_t)
    # Column-major index p = i_r + n_r i_R + n_r n_R i_t  <=>  kron(t, R, r).
    H = np.kron(It, np.kron(IR, Kr)) + np.kron(It, np.kron(KR, Ir))
    H += np.diag(np.tile(p.DEP, n_t)) @ np.kron(Kt, np.eye(n_r * n_R))
    H += np.diag(p.RES - shift)
    return H


@dataclasses.dataclass
class NdvrProblem:
    """A problem in the sNDVR form: the outermost (theta) layer is given as
    per-point matrices OUTH(n_r n_R, n_theta, n_theta) instead of a level
    matrix, as the JA3 H0GM output (src/ham/ja3/module/ja3.hgmij:6-62) feeds
    H3X (src/libutil/serial/base/matrix.f90:188-203)."""

    sizes: tuple
    dep: tuple
    H0: np.ndarray      # K_r, K_R only (the outer level has no H0 block)
    RES: np.ndarray     # the diagonal kept outside OUTH
    DEP: np.ndarray     # empty: no dependent level
    OUTH: np.ndarray    # (n_r n_R) x n_theta x n_theta, column-major, point index fastest

    @property
    def N(self) -> int:
        return int(np.prod(self.sizes))


def ndvr_problem(p: Problem, coupling: float = 1e-4, seed: int = 0) -> NdvrProblem:
    """The same Hamiltonian with its angular layer moved into per-point
    matrices: OUTH(a, :, :) = c(a) K_theta + diag(V(a, :)) + coupling * S_a,
    S_a a seeded symmetric matrix per (r, R) point (a per-point angular term
    no level matrix can express).  RES is zero, since V sits inside OUTH: the
    outer level's block-Jacobi blocks are then OUTH itself, as myDiagInit
    copies it (osb.diag.h:19-30)."""
    n_r, n_R, n_t = p.sizes
    nin = n_r * n_R
    Kt = p.level_matrix(3)
    c = p.DEP[:nin]
    V = p.RES.reshape(nin, n_t, order="F")
    rng = np.random.default_rng(seed)
    S = rng.standard_normal((nin, n_t, n_t))
    S = 0.5 * (S + S.transpose(0, 2, 1))
    A = c[:, None, None] * Kt[None, :, :] + coupling * S
    A[:, np.arange(n_t), np.arange(n_t)] += V
    OUTH = np.ascontiguousarray(A.transpose(2, 1, 0)).ravel()   # a fastest, then i, then j
    H0 = np.concatenate([p.level_matrix(1).ravel(order="F"), p.level_matrix(2).ravel(order="F")])
    return NdvrProblem(sizes=p.sizes, dep=(False, False, False), H0=H0, RES=np.zeros(p.N),
                       DEP=np.zeros(0), OUTH=OUTH)


def dense_ndvr(q: NdvrProblem) -> np.ndarray:
    """Explicit N x N matrix of an sNDVR problem (small problems only)."""
    n_r, n_R, n_t = q.sizes
    nin = n_r * n_R
    Kr = q.H0[:n_r * n_r].reshape(n_r, n_r, order="F")
    KR = q.H0[n_r * n_r:].reshape(n_R, n_R, order="F")
    H = np.kron(np.eye(n_t), np.kron(np.eye(n_R), Kr)) + np.kron(np.eye(n_t), np.kron(KR, np.eye(n_r)))
    A = q.OUTH.reshape(n_t, n_t, nin).transpose(2, 1, 0)      # A[a, i, j]
    for i in range(n_t):
        for j in range(n_t):
            H[i * nin:(i + 1) * nin, j * nin:(j + 1) * nin] += np.diag(A[:, i, j])
    H += np.diag(q.RES)
    return H
