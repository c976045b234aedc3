"""P*X through the entry point that allocates nothing (scalit_px_noalloc_device).

The variant exists for callers that cannot allocate device memory at call
time (their device memory is owned by another allocator, or they must avoid
the implicit synchronisation of cudaMalloc/cudaFree); it keeps its scratch in
a file-scope device array of 2^20 doubles.  It must give the same result as
scalit_px_device on two calls in a row, and reject grids larger than its
scratch.  This file is collected last on purpose; it also passes alone in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu

TOL = 1e-9   # the P*X tolerance of the other GPU tests


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_px_matches_px_device_twice(lib):
    torch = pytest.importorskip("torch")
    p = hm.workload("tri-24x32x20")
    e0 = float(p.RES.min()) - 1e-3
    rng = np.random.default_rng(7)
    with capi.Context.from_problem(p, e0=e0) as ctx:
        ctx.build_osb(20, 1e-4)
        for call in range(2):
            x = torch.tensor(rng.standard_normal(p.N), device="cuda")
            y_ref = torch.empty_like(x)
            y_new = torch.full_like(x, float("nan"))
            torch.cuda.synchronize()
            ctx.px_device(x, y_ref, 1, capi.TA1)
            rc = lib.scalit_px_noalloc_device(ctx.h, capi.TA1, C.c_void_p(x.data_ptr()),
                                              C.c_void_p(y_new.data_ptr()))
            assert rc == 0, lib.scalit_last_error()
            torch.cuda.ExternalStream(ctx.stream).synchronize()
            a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
            assert np.isfinite(a).all(), f"call {call}"
            assert rel(a, b) < TOL, f"call {call}: {rel(a, b)}"


def test_noalloc_px_rejects_large_grid(lib):
    with capi.Context((128, 128, 97), (False, False, True)) as ctx:
        rc = lib.scalit_px_noalloc_device(ctx.h, capi.TA1, C.c_void_p(0), C.c_void_p(0))
        assert rc == -101
        assert b"exceeds" in lib.scalit_last_error()
