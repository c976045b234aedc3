"""ctypes bindings of libscalit_gb300.so (the C ABI in include/scalit_gb300.h).

The library must have been built (``scalit_gb300.build.build()``); loading
fails loudly otherwise -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

TA0, TA1 = 0, 1
TOSB, TOSBD1, TOSBD2, TOSBW = 1, 2, 3, 4
# nType codes of the complex forms (osb.data.h:18-22)
TAAP0, TMAP0, TAAP, TAAPP, TAAPR, TMAP, TMAPP, TMAPR = 2, 3, 100, 101, 102, 200, 201, 202
FP32_SIMT, FP32_TENSOR, FP32_TENSOR_PX, FP32_TENSOR16 = 0, 1, 2, 3
PREC_FP64, PREC_FP32, PREC_FP32_REFINED = 0, 1, 2
FP64_DFMA, FP64_TENSOR = 0, 1
FMAX = 20

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

# Every function the header declares: name -> (restype, argtypes).
SIGNATURES = {
    "scalit_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, _ip, _ip, C.c_int, C.c_int]),
    "scalit_destroy": (None, [_vp]),
    "scalit_last_error": (C.c_char_p, []),
    "scalit_npoints": (C.c_longlong, [_vp]),
    "scalit_h0_len": (C.c_longlong, [_vp]),
    "scalit_dep_len": (C.c_longlong, [_vp]),
    "scalit_vosb_len": (C.c_longlong, [_vp]),
    "scalit_load": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "scalit_get_stream": (C.c_void_p, [_vp]),
    "scalit_set_stream": (C.c_int, [_vp, _vp]),
    "scalit_set_fp64_mode": (C.c_int, [_vp, C.c_int]),
    "scalit_set_shift": (C.c_int, [_vp, C.c_double]),
    "scalit_set_precond": (C.c_int, [_vp, C.c_int, C.c_double, C.c_double]),
    "scalit_hx": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp]),
    "scalit_hx_device": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "scalit_hx_f32_device": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "scalit_level_device": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "scalit_pist_refined": (C.c_int, [_vp, _vp, _dp, _dp, _dp, _vp, C.c_double, C.c_int, _dp, _dp, _ip]),
    "scalit_hx_level_times": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, C.c_int,
                                        C.POINTER(C.c_float)]),
    "scalit_build_osb": (C.c_int, [_vp, C.c_int, C.c_double, _dp]),
    "scalit_build_times": (C.c_int, [_vp, _dp]),
    "scalit_selftest_wait": (C.c_int, [_vp, C.c_double]),
    "scalit_set_fp32_mode": (C.c_int, [_vp, C.c_int]),
    "scalit_set_build_precision": (C.c_int, [_vp, C.c_int]),
    "scalit_set_fp32_px_storage": (C.c_int, [_vp, C.c_int]),
    "scalit_tile_picks": (C.c_int, [_vp, _ip]),
    "scalit_get_osb": (C.c_int, [_vp, _dp, _dp]),
    "scalit_set_osb": (C.c_int, [_vp, _dp, _dp]),
    "scalit_build_osbw": (C.c_int, [_vp, C.c_double, C.c_int, _dp, C.c_int, _ip]),
    "scalit_set_absorbing": (C.c_int, [_vp, _dp, _dp]),
    "scalit_hx_cx": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp]),
    "scalit_load_cx": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "scalit_hx_cx_device": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "scalit_px_cx": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp]),
    "scalit_px_cx_device": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "scalit_qmr_cx": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp, _ip, _dp]),
    "scalit_crp": (C.c_int, [_vp, C.c_int, _dp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, _dp, _dp]),
    "scalit_pist_cx": (C.c_int, [_vp, C.c_double, C.c_double, C.c_int, C.c_int, _dp, C.c_int, C.c_int, C.c_int,
                                 C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                 _dp, _dp, _ip]),
    "scalit_set_osbw": (C.c_int, [_vp, C.c_double, C.c_int, _dp, C.c_int, _dp]),
    "scalit_get_osbw": (C.c_int, [_vp, _ip, _ip, _dp]),
    "scalit_px": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp]),
    "scalit_px_device": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "scalit_px_f32_device": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "scalit_px_noalloc_device": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "scalit_qmr": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp, _dp, _ip]),
    "scalit_qmr_device": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp, _dp, _ip]),
    "scalit_qmr_ex": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp, _ip, _dp, _ip]),
    "scalit_qmr_device_ex": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp, _ip, _dp, _ip]),
    "scalit_pist_default_params": (None, [_vp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                          C.c_int, C.c_int, C.c_int, C.c_double]),
    "scalit_pist": (C.c_int, [_vp, _vp, _dp, _dp, _dp, _vp]),
    "scalit_hx_adjoint": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp, _dp, _dp]),
    "scalit_hx_adjoint_device": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    "scalit_hx_adjoint_f32_device": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    "scalit_hf_gradients": (C.c_int, [_vp, C.c_int, _dp, C.c_int, _dp, _dp]),
    "scalit_pist_vectors": (C.c_int, [_vp, _vp, _dp, _dp, _dp, _vp, _dp]),
    "scalit_pist_residuals": (C.c_int, [_vp, _vp, _dp, _dp, _dp, _vp, _dp]),
    "scalit_qmr_shifts_device": (C.c_int, [_vp, C.c_int, _dp, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp,
                                           _ip, _dp]),
    "scalit_qmr_shifts_batch": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, _dp, C.c_int, C.c_int,
                                          C.c_double, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                          _ip, _dp, _dp]),
    "scalit_pist_basis": (C.c_int, [_vp, _vp, _dp, _dp, _dp, _vp, _ip, _dp, _dp, _dp]),
    # Fortran drop-ins (all arguments by reference)
    "h1x_xyz_": (None, [_ip, _ip, _ip, _dp, _dp, _dp]),
    "h1x_xyz_seq_": (None, [_ip, _ip, _ip, _dp, _dp, _dp]),
    "h1tx_xyz_seq_": (None, [_ip, _ip, _ip, _dp, _dp, _dp]),
    "h1x_dep_": (None, [_ip, _ip, _ip, _dp, _dp, _dp, _dp]),
    "h2x_dep_seq_": (None, [_ip, _ip, _ip, _dp, _dp, _dp, _dp]),
    "h3x_out_seq_": (None, [_ip, _ip, _ip, _dp, _dp, _dp]),
    "vx_": (None, [_ip, _ip, _ip, _dp, _dp]),
    "vtx_": (None, [_ip, _ip, _ip, _dp, _dp]),
    "vx_seq_": (None, [_ip, _ip, _ip, _dp, _dp]),
    "vtx_seq_": (None, [_ip, _ip, _ip, _dp, _dp]),
    "hosbdiag_": (None, [_ip, _dp, _ip, _ip, _ip, _dp, _dp, _dp]),
    "hosbdiag_seq_": (None, [_ip, _dp, _ip, _ip, _ip, _dp, _dp, _dp, _ip]),
    "hosbdiag_mpi_": (None, [_ip, _ip, _dp, _ip, _ip, _ip, _dp, _dp, _dp, _ip, _ip]),
    "mjacobi_": (C.c_double, [_ip, _ip, _ip, _ip, _dp]),
    "norm_mpi_": (C.c_double, [_ip, _ip, _dp, _ip]),
    "dotprod_mpi_": (C.c_double, [_ip, _ip, _dp, _dp, _ip]),
    "mgs_orth_": (C.c_int, [_ip, _dp, _ip, _dp]),
    "mgs_orth_mpi_": (C.c_int, [_ip, _dp, _ip, _dp, _ip]),
    "qmr_": (C.c_int, [_ip, _ip, _dp, _ip, _dp, _vp, _vp, _dp, _dp]),
    "qmr_cx_": (C.c_int, [_ip, _ip, _dp, _ip, _dp, _vp, _vp, _dp, _dp]),
    "pist_conv_sx_": (C.c_int, [_dp, _dp, _ip, _ip, _dp, _ip, _ip, _ip, _ip, _ip, _vp, _vp, _dp, _dp]),
    "pist_conv_cx_": (C.c_int, [_dp, _dp, _ip, _ip, _dp, _ip, _ip, _ip, _ip, _ip, _vp, _vp, _dp, _dp]),
    "qmr_mpi_": (C.c_int, [_ip, _ip, _dp, _ip, _dp, _vp, _vp, _dp, _dp, _ip]),
    "pist_conv_": (C.c_int, [_dp, _dp, _ip, _ip, _dp, _ip, _ip, _ip, _ip, _ip, _vp, _vp, _dp, _dp]),
    "pisth0_": (C.c_int, [_ip, _dp, _ip, _ip, _ip, _vp, _vp, _dp, _dp]),
    "pisth0_mpi_": (C.c_int, [_ip, _ip, _ip, _dp, _ip, _ip, _ip, _vp, _vp, _dp, _dp, _ip]),
    "pist_conv_mpi_": (C.c_int, [_ip, _ip, _dp, _dp, _ip, _ip, _dp, _ip, _ip, _ip, _ip, _ip, _vp, _vp,
                                 _dp, _dp]),
    "scalit_fortran_device_": (None, [_ip]),
    "scalit_fortran_init_": (None, [_ip, _ip, _ip, _dp, _dp, _dp, _dp, _ip]),
    "scalit_fortran_precond_": (None, [_ip, _dp, _dp, _ip, _dp, _ip]),
    "scalit_fortran_osbw_": (None, [_dp, _ip, _dp, _ip, _ip]),
    "scalit_fortran_qmr_param_": (None, [_ip, _ip, _dp, _ip]),
    "scalit_fortran_final_": (None, []),
    "scalit_hx0_": (None, [_ip, _dp, _dp]),
    "scalit_ehx_": (None, [_ip, _dp, _dp]),
    "scalit_epx_": (None, [_ip, _dp, _dp]),
    "scalit_osb_qmr_": (C.c_int, [_ip, _dp, _dp, _dp]),
}


class PistParams(C.Structure):
    _fields_ = [("e0", C.c_double), ("etol", C.c_double), ("ntype", C.c_int),
                ("startcnt", C.c_int), ("stepcnt", C.c_int), ("stepeig", C.c_int),
                ("m", C.c_int), ("m_max", C.c_int), ("qmr_ntype", C.c_int),
                ("qmr_max", C.c_int), ("qmr_tol", C.c_double), ("precision", C.c_int),
                ("verbose", C.c_int), ("orth", C.c_int)]


class PistInfo(C.Structure):
    _fields_ = [("krylov", C.c_int), ("qmr_total", C.c_int), ("qmr_solves", C.c_int),
                ("checks", C.c_int), ("t_qmr", C.c_double), ("t_orth", C.c_double),
                ("t_hmat", C.c_double), ("t_ritz", C.c_double), ("t_resid", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the shared library (build it first when asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run scalit_gb300.build.build() (nvcc, sm_103a)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class ScalitError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"scalit error {code}: {msg}")
        self.code = code


def _check(rc):
    if rc < -100:
        raise ScalitError(rc, load().scalit_last_error().decode())
    return rc


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(t):
    """Raw device pointer of a torch tensor or an int."""
    if isinstance(t, int):
        return C.c_void_p(t)
    return C.c_void_p(t.data_ptr())


class Context:
    """One OSB operator on one GPU (the reference's module state)."""

    def __init__(self, sizes, dep=None, ndvr=False, device=0):
        self.lib = load()
        sizes = [int(n) for n in sizes]
        dep = [int(bool(d)) for d in (dep or [0] * len(sizes))]
        n = (C.c_int * len(sizes))(*sizes)
        d = (C.c_int * len(dep))(*dep)
        h = C.c_void_p()
        _check(self.lib.scalit_create(C.byref(h), len(sizes), n, d, int(bool(ndvr)), int(device)))
        self.h = h
        self.sizes = tuple(sizes)
        self.N = int(self.lib.scalit_npoints(h))
        self.vosb_len = int(self.lib.scalit_vosb_len(h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.scalit_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @classmethod
    def from_problem(cls, problem, e0=0.0, device=0):
        ctx = cls(problem.sizes, problem.dep, device=device)
        ctx.load(problem.H0, problem.RES, problem.DEP)
        ctx.set_shift(e0)
        return ctx

    def load(self, H0, RES, DEP=None, OUTH=None):
        self._keep = [_f64(H0), _f64(RES), _f64(DEP) if DEP is not None else None,
                      _f64(OUTH) if OUTH is not None else None]
        H0, RES, DEP, OUTH = self._keep
        _check(self.lib.scalit_load(self.h, _p(H0), _p(RES), _p(DEP) if DEP is not None else None,
                                    _p(OUTH) if OUTH is not None else None))

    @property
    def stream(self) -> int:
        return int(self.lib.scalit_get_stream(self.h) or 0)

    def set_stream(self, stream_ptr):
        _check(self.lib.scalit_set_stream(self.h, C.c_void_p(int(stream_ptr) if stream_ptr else 0)))

    def set_fp64_mode(self, mode):
        _check(self.lib.scalit_set_fp64_mode(self.h, int(mode)))

    def set_fp32_mode(self, mode):
        _check(self.lib.scalit_set_fp32_mode(self.h, int(mode)))

    def set_fp32_px_storage(self, bits):
        """32 (default) or 16: storage of the first level's preconditioner
        matrices for the FP32 P*X."""
        _check(self.lib.scalit_set_fp32_px_storage(self.h, int(bits)))

    def set_build_precision(self, precision):
        """PREC_FP64 (default) or PREC_FP32: precision of the next builds'
        Jacobi sweeps on one-matrix blocks."""
        _check(self.lib.scalit_set_build_precision(self.h, int(precision)))

    def set_shift(self, e0):
        _check(self.lib.scalit_set_shift(self.h, float(e0)))

    def set_precond(self, kind=TOSB, de=0.0, beta=0.0):
        _check(self.lib.scalit_set_precond(self.h, int(kind), float(de), float(beta)))

    def hx(self, X, ntype=TA1, out=None):
        X = _f64(X)
        nvec = X.size // self.N
        Y = np.empty_like(X) if out is None else out
        assert Y.dtype == np.float64 and Y.flags.c_contiguous and Y.size == X.size
        _check(self.lib.scalit_hx(self.h, int(ntype), nvec, _p(X), _p(Y)))
        return Y

    def hx_device(self, dX, dY, nvec=1, ntype=TA1):
        _check(self.lib.scalit_hx_device(self.h, int(ntype), int(nvec), _ptr(dX), _ptr(dY)))

    def level_device(self, level, dX, dY, accumulate=False):
        _check(self.lib.scalit_level_device(self.h, int(level), int(bool(accumulate)), _ptr(dX), _ptr(dY)))

    def hx_level_times(self, dX, dY, nvec, reps=10, ntype=TA1):
        """Average duration (ms) of each level's launch over reps H*X
        applications to nvec device vectors (float64 or float32 tensors)."""
        import torch
        prec = PREC_FP64 if dX.dtype == torch.float64 else PREC_FP32
        ms = (C.c_float * 20)()
        _check(self.lib.scalit_hx_level_times(self.h, prec, ntype, nvec, _ptr(dX), _ptr(dY), reps, ms))
        return [float(ms[i]) for i in range(len(self.sizes))]

    def hx_f32_device(self, dX, dY, nvec=1, ntype=TA1):
        _check(self.lib.scalit_hx_f32_device(self.h, int(ntype), int(nvec), _ptr(dX), _ptr(dY)))

    def build_osb(self, bjmax, bjtol):
        stats = np.zeros(5 * len(self.sizes))
        _check(self.lib.scalit_build_osb(self.h, int(bjmax), float(bjtol), _p(stats)))
        return stats.reshape(len(self.sizes), 5)

    def tile_picks(self):
        """Autotuned GEMM tiles, shape (precision [FP64, FP32], level, [one vector, many])."""
        t = np.zeros(2 * len(self.sizes) * 2, dtype=np.int32)
        _check(self.lib.scalit_tile_picks(self.h, t.ctypes.data_as(C.POINTER(C.c_int))))
        return t.reshape(2, len(self.sizes), 2)

    def selftest_wait(self, seconds):
        """Run the bounded-wait self-test; returns the C call's status code."""
        return int(self.lib.scalit_selftest_wait(self.h, float(seconds)))

    def build_times(self):
        t = np.zeros(len(self.sizes))
        _check(self.lib.scalit_build_times(self.h, _p(t)))
        return t

    def get_osb(self):
        V = np.empty(self.vosb_len)
        E = np.empty(self.N)
        _check(self.lib.scalit_get_osb(self.h, _p(V), _p(E)))
        return V, E

    def set_osb(self, VOSB, EIG0):
        V, E = _f64(VOSB), _f64(EIG0)
        _check(self.lib.scalit_set_osb(self.h, _p(V), _p(E)))

    def build_osbw(self, e0, count, de, npc=TA1):
        """initOSBW: the window of ``count`` states around ``e0`` (starting width
        ``de``), its matrix HW and factor; selects TOSBW.  Returns (hwlen, de)."""
        d = C.c_double(float(de))
        m = C.c_int(0)
        _check(self.lib.scalit_build_osbw(self.h, float(e0), int(count), C.byref(d), int(npc), C.byref(m)))
        return m.value, d.value

    def set_osbw(self, e0, count, de, HW, npc=TA1):
        """loadHW + createWH: the window selected as build_osbw selects it, HW
        (count x count) given.  Returns the final width."""
        d = C.c_double(float(de))
        hw = np.ascontiguousarray(np.asarray(HW, dtype=np.float64).ravel(order="F"))
        _check(self.lib.scalit_set_osbw(self.h, float(e0), int(count), C.byref(d), int(npc), _p(hw)))
        return d.value

    def set_absorbing(self, APP, APR=None):
        """The absorbing potentials: AP = APP (APR None) or APP + APR."""
        self._ap = [_f64(APP), None if APR is None else _f64(APR)]
        _check(self.lib.scalit_set_absorbing(self.h, _p(self._ap[0]),
                                             None if self._ap[1] is None else _p(self._ap[1])))

    def _cx_apply(self, fn, X, ntype):
        Z = np.ascontiguousarray(X, dtype=np.complex128)
        nvec = Z.size // self.N
        out = np.empty_like(Z)
        zf, of = Z.view(np.float64), out.view(np.float64)
        _check(fn(self.h, int(ntype), nvec, _p(zf), _p(of)))
        return out

    def load_cx(self, H0CX, RES, DEPCX=None, OUTHCX=None):
        """The complex-Hamiltonian job (sCX): complex level matrices, DEP
        factors and outer per-point matrices, real RES."""
        def cx(a):
            return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.complex128)).view(np.float64)
        h, d, o = cx(H0CX), cx(DEPCX), cx(OUTHCX)
        res = _f64(RES)
        _check(self.lib.scalit_load_cx(self.h, _p(h), _p(res), _p(d) if d is not None else None,
                                       _p(o) if o is not None else None))

    def hx_cx(self, X, ntype=TAAP):
        """MYHX_DX on complex vectors (N or nvec x N)."""
        return self._cx_apply(self.lib.scalit_hx_cx, X, ntype)

    def px_cx(self, X, ntype=TAAP):
        """MYPX_DX on complex vectors."""
        return self._cx_apply(self.lib.scalit_px_cx, X, ntype)

    def qmr_cx(self, B, qmrmax, qmrtol, ntype=TAAP, conv=0, X0=None):
        """QMR_CX: returns (code, X, RES)."""
        Bc = np.ascontiguousarray(B, dtype=np.complex128)
        X = np.zeros_like(Bc) if X0 is None else np.ascontiguousarray(X0, dtype=np.complex128).copy()
        code = C.c_int(0)
        res = C.c_double(0.0)
        _check(self.lib.scalit_qmr_cx(self.h, int(conv), int(qmrmax), float(qmrtol), int(ntype),
                                      _p(Bc.view(np.float64)), _p(X.view(np.float64)), C.byref(code),
                                      C.byref(res)))
        return code.value, X, res.value

    def crp(self, energies, nm, qmrmax=2000, qmrtol=1e-4, conv=0, sap=True, X0=None, seed=0):
        """osbCRP: N(E) at each energy.  X0 (len(energies) x N complex) defaults
        to seeded uniform real and imaginary parts, as randMat_CX draws them."""
        E = _f64(np.atleast_1d(energies))
        if X0 is None:
            rng = np.random.default_rng(seed)
            X0 = rng.random((E.size, self.N)) + 1j * rng.random((E.size, self.N))
        Z = np.ascontiguousarray(X0, dtype=np.complex128)
        out = np.zeros(E.size)
        _check(self.lib.scalit_crp(self.h, E.size, _p(E), int(nm), int(qmrmax), float(qmrtol), int(conv),
                                   int(bool(sap)), _p(Z.view(np.float64).ravel()), _p(out)))
        return out

    def pist_cx(self, x0, m, e0, etol, m_max, startcnt=0, stepcnt=5, stepeig=1, h0_ntype=TMAP0,
                ls_ntype=TMAP, ls_px_ntype=TMAP, conv=0, qmrmax=2000, qmrtol=1e-4, ntype=0, conjugate=False):
        """PIST_CONV_SX (PIST_CONV_CX with conjugate): returns (status, eig[m] complex, RES)."""
        Z = np.ascontiguousarray(x0, dtype=np.complex128)
        eig = np.zeros(int(m), dtype=np.complex128)
        res = C.c_double(0.0)
        st = C.c_int(0)
        _check(self.lib.scalit_pist_cx(self.h, float(e0), float(etol), int(ntype), int(bool(conjugate)),
                                       _p(Z.view(np.float64)),
                                       int(startcnt), int(stepcnt), int(stepeig), int(m), int(m_max),
                                       int(h0_ntype), int(ls_ntype), int(ls_px_ntype), int(conv), int(qmrmax),
                                       float(qmrtol), _p(eig.view(np.float64)), C.byref(res), C.byref(st)))
        return st.value, eig, res.value

    def get_osbw(self):
        """(ind, HW): the window's grid points (0-based) and its matrix."""
        m = C.c_int(0)
        _check(self.lib.scalit_get_osbw(self.h, C.byref(m), None, None))
        ind = np.zeros(m.value, dtype=np.int32)
        hw = np.zeros(m.value * m.value)
        _check(self.lib.scalit_get_osbw(self.h, None, ind.ctypes.data_as(_ip), _p(hw)))
        return ind.astype(np.int64), hw.reshape(m.value, m.value, order="F")

    def px(self, X, npc=TA1):
        X = _f64(X)
        nvec = X.size // self.N
        Y = np.empty_like(X)
        _check(self.lib.scalit_px(self.h, int(npc), nvec, _p(X), _p(Y)))
        return Y

    def px_device(self, dX, dY, nvec=1, npc=TA1):
        _check(self.lib.scalit_px_device(self.h, int(npc), int(nvec), _ptr(dX), _ptr(dY)))

    def px_noalloc_device(self, dX, dY, npc=TA1):
        """P*X of one device vector with the library's static scratch (no allocation)."""
        _check(self.lib.scalit_px_noalloc_device(self.h, int(npc), _ptr(dX), _ptr(dY)))

    def px_f32_device(self, dX, dY, nvec=1, npc=TA1):
        _check(self.lib.scalit_px_f32_device(self.h, int(npc), int(nvec), _ptr(dX), _ptr(dY)))

    def qmr_shifts_device(self, dB, dX, shifts, qmrmax, qmrtol, ntype=-1, precision=PREC_FP64):
        """QMR on len(shifts) right-hand sides at once (device arrays nrhs x N, FP64):
        column v solves (H - shifts[v]) x = b_v.  Returns (codes, res)."""
        shifts = _f64(shifts)
        nrhs = shifts.size
        codes = np.zeros(nrhs, dtype=np.int32)
        res = np.zeros(nrhs)
        _check(self.lib.scalit_qmr_shifts_device(self.h, nrhs, _p(shifts), int(ntype), int(qmrmax), float(qmrtol),
                                                 int(precision), _ptr(dB), _ptr(dX),
                                                 codes.ctypes.data_as(C.POINTER(C.c_int)), _p(res)))
        return codes, res

    def qmr(self, B, qmrmax, qmrtol, ntype=-1, precision=PREC_FP64, X0=None):
        """OSB_QMR: returns (code, X, RES, iterations)."""
        B = _f64(B)
        X = np.zeros_like(B) if X0 is None else _f64(X0).copy()
        res = C.c_double(0.0)
        it = C.c_int(0)
        code = C.c_int(0)
        _check(self.lib.scalit_qmr_ex(self.h, int(ntype), int(qmrmax), float(qmrtol), int(precision),
                                      _p(B), _p(X), C.byref(code), C.byref(res), C.byref(it)))
        return code.value, X, res.value, it.value

    def hx_adjoint(self, X, Ybar, ntype=TA1, want=("x", "v", "h")):
        """Adjoint of H*X: returns (Xbar, Vbar, H0bar) (None for what is not wanted)."""
        X, Ybar = _f64(X), _f64(Ybar)
        Xb = np.empty(self.N) if "x" in want else None
        Vb = np.empty(self.N) if "v" in want else None
        Hb = np.empty(int(self.lib.scalit_h0_len(self.h))) if "h" in want else None
        _check(self.lib.scalit_hx_adjoint(self.h, int(ntype), _p(X), _p(Ybar),
                                          _p(Xb) if Xb is not None else None,
                                          _p(Vb) if Vb is not None else None,
                                          _p(Hb) if Hb is not None else None))
        return Xb, Vb, Hb

    def hx_adjoint_device(self, dX, dYbar, dXbar=None, dVbar=None, dHbar=None, ntype=TA1, f32=False):
        f = self.lib.scalit_hx_adjoint_f32_device if f32 else self.lib.scalit_hx_adjoint_device
        nul = C.c_void_p(0)
        _check(f(self.h, int(ntype), _ptr(dX), _ptr(dYbar), _ptr(dXbar) if dXbar is not None else nul,
                 _ptr(dVbar) if dVbar is not None else nul, _ptr(dHbar) if dHbar is not None else nul))

    def hf_gradients(self, psi, dvdp):
        """dE_k/dp_j = <psi_k| dV/dp_j |psi_k> for psi (m x N) and dvdp (np x N)."""
        psi, dvdp = _f64(psi), _f64(dvdp)
        m, npar = psi.size // self.N, dvdp.size // self.N
        g = np.empty((m, npar))
        _check(self.lib.scalit_hf_gradients(self.h, m, _p(psi), npar, _p(dvdp), _p(g)))
        return g

    def pist(self, x0, m, e0, etol, startcnt=0, stepcnt=5, m_max=0, gap=1, qmr_max=2000,
             qmr_tol=1e-4, qmr_ntype=-1, precision=PREC_FP64, ntype=0, verbose=False, orth=1,
             vectors=False, basis=False, residuals=False, refine_tol=0.0, refine_steps=4):
        """OSB_PISTCONV: returns (status, eig[m], RES, info dict); with vectors=True the
        info dict also holds the m Ritz vectors ("vectors", m x N); with residuals=True
        it holds the FP64 residual norms |H psi - E psi| of the levels ("resid", m)."""
        p = PistParams()
        self.lib.scalit_pist_default_params(C.byref(p), int(m), float(e0), float(etol),
                                            int(startcnt), int(stepcnt), int(m_max), int(gap),
                                            int(qmr_max), float(qmr_tol))
        p.qmr_ntype = int(qmr_ntype)
        p.precision = int(precision)
        p.ntype = int(ntype)
        p.verbose = int(bool(verbose))
        p.orth = int(orth)
        x0 = _f64(x0)
        eig = np.zeros(int(m))
        res = C.c_double(0.0)
        info = PistInfo()
        if basis:
            mm = int(p.m_max)
            cnt = C.c_int(0)
            ritz = np.zeros(mm)
            hmat = np.zeros(mm * mm)
            vj = np.zeros(mm * self.N)
            st = _check(self.lib.scalit_pist_basis(self.h, C.byref(p), _p(x0), _p(eig), C.byref(res),
                                                   C.byref(info), C.byref(cnt), _p(ritz), _p(hmat), _p(vj)))
            k = cnt.value
            return st, eig, res.value, dict(info.as_dict(), m_max=p.m_max, startcnt=p.startcnt, cnt=k,
                                            ritz=ritz[:k], hmat=hmat[:k * k].reshape(k, k, order="F"),
                                            vj=vj[:k * self.N].reshape(self.N, k, order="F"))
        if refine_tol != 0.0:
            resid = np.zeros(int(m))
            vec = np.zeros((int(m), self.N)) if vectors else None
            steps = C.c_int(0)
            st = _check(self.lib.scalit_pist_refined(self.h, C.byref(p), _p(x0), _p(eig), C.byref(res),
                                                     C.byref(info), float(refine_tol), int(refine_steps),
                                                     _p(resid), _p(vec) if vec is not None else None,
                                                     C.byref(steps)))
            out = dict(info.as_dict(), m_max=p.m_max, startcnt=p.startcnt, resid=resid, refine_steps=steps.value)
            if st > 0:
                out["krylov"] = st
            if vec is not None:
                out["vectors"] = vec
            return st, eig, res.value, out
        if residuals:
            resid = np.zeros(int(m))
            st = _check(self.lib.scalit_pist_residuals(self.h, C.byref(p), _p(x0), _p(eig), C.byref(res),
                                                       C.byref(info), _p(resid)))
            return st, eig, res.value, dict(info.as_dict(), m_max=p.m_max, startcnt=p.startcnt, resid=resid)
        if vectors:
            vec = np.zeros((int(m), self.N))
            st = _check(self.lib.scalit_pist_vectors(self.h, C.byref(p), _p(x0), _p(eig), C.byref(res),
                                                     C.byref(info), _p(vec)))
            return st, eig, res.value, dict(info.as_dict(), m_max=p.m_max, startcnt=p.startcnt, vectors=vec)
        st = _check(self.lib.scalit_pist(self.h, C.byref(p), _p(x0), _p(eig), C.byref(res),
                                         C.byref(info)))
        return st, eig, res.value, dict(info.as_dict(), m_max=p.m_max, startcnt=p.startcnt)


def qmr_shifts_batch(contexts, shifts, dBs, dXs, qmrmax, qmrtol, ntype=-1, precision=PREC_FP32):
    """Shifted QMR of several problems advanced together by one CUDA graph.
    shifts: nprob x nrhs; dBs / dXs: per problem device arrays nrhs x N (FP64).
    Returns (codes, res, device_seconds)."""
    lib = load()
    shifts = np.ascontiguousarray(np.asarray(shifts, dtype=np.float64))
    nprob, nrhs = shifts.shape
    ctxs = (C.c_void_p * nprob)(*[c.h for c in contexts])
    bs = (C.c_void_p * nprob)(*[_ptr(b) for b in dBs])
    xs = (C.c_void_p * nprob)(*[_ptr(x) for x in dXs])
    codes = np.zeros((nprob, nrhs), dtype=np.int32)
    res = np.zeros((nprob, nrhs))
    sec = C.c_double(0.0)
    _check(lib.scalit_qmr_shifts_batch(ctxs, nprob, nrhs, _p(shifts), int(ntype), int(qmrmax), float(qmrtol),
                                       int(precision), bs, xs, codes.ctypes.data_as(C.POINTER(C.c_int)), _p(res),
                                       C.byref(sec)))
    return codes, res, sec.value
