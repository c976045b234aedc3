"""Bounded waits on the GPU: a wait that nothing completes runs out, the kernel
records the expiry and returns, the call reports SCALIT_ECUDA with a message,
and the context keeps working (no GPU fault, no hang: the expiry is the
designed path of every streaming and tensor-core kernel's mbarrier waits)."""
import time

import numpy as np
import pytest

from scalit_gb300 import capi, hamiltonian as hm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c0():
    return hm.workload("tri-24x32x20")


def test_bounded_wait_expires_and_context_survives(lib, c0):
    x = np.random.default_rng(11).standard_normal(c0.N)
    with capi.Context.from_problem(c0, e0=0.0) as ctx:
        y0 = ctx.hx(x)
        t0 = time.perf_counter()
        rc = ctx.selftest_wait(0.05)
        dt = time.perf_counter() - t0
        assert rc == -102                                   # SCALIT_ECUDA
        assert "wait ran out" in capi.load().scalit_last_error().decode()
        assert 0.04 < dt < 5.0
        # the flag was cleared and the context still computes
        np.testing.assert_array_equal(ctx.hx(x), y0)
        assert ctx.selftest_wait(0.0) == -101               # SCALIT_EINVAL
        assert ctx.selftest_wait(11.0) == -101
