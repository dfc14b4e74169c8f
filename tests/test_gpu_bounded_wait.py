"""The bounded waits of the tensor-core kernels run out as designed.

Every wait of the BF16 network kernels on an mbarrier phase gives up after a
configurable number of SM cycles and records an error status instead of
spinning forever.  The self-test arms a barrier for bytes that nothing
delivers (no copy is issued), waits with a short limit through the same
wait helper, and must come back with status 4; the device stays usable, and
the network kernels still run afterwards with a configured limit."""
import ctypes as C
import time

import numpy as np
import pytest

import orc
import xmd_x
from gpu_common import random_state

pytestmark = pytest.mark.gpu

TIMED_OUT = 4


@pytest.fixture(scope="module")
def lib():
    return xmd_x.load(3, 4)


@pytest.mark.parametrize("limit", [1 << 12, 1 << 18, 1 << 22])
def test_wait_runs_out_and_reports_status(lib, limit):
    status, waited = C.c_int(-1), C.c_longlong(0)
    t0 = time.perf_counter()
    lib.check(lib.md_gb300_wait_selftest_x(limit, C.byref(status), C.byref(waited)), "wait self-test")
    dt = time.perf_counter() - t0
    assert status.value == TIMED_OUT
    # the block waits twice (the wait, then the drain of its own copies),
    # each until `limit` cycles have passed
    assert 2 * limit <= waited.value <= 2 * limit + (1 << 25), waited.value
    assert dt < 5.0


def test_network_kernels_run_with_a_configured_limit(lib):
    default = lib.md_gb300_get_wait_limit_x()
    assert default == 1 << 32
    err = (C.c_double * 5)()
    try:
        lib.check(lib.md_gb300_set_wait_limit_x(1 << 30))
        assert lib.md_gb300_get_wait_limit_x() == 1 << 30
        lib.check(lib.md_gb300_tc_selftest_x(err), "self-test")
        assert err[0] < 1e-3, list(err)
        box, N, P = 6.0, 16, 4
        xmd_x.set_potentials(lib, coul_s=1.0, alpha=5.6 / box, nsum=4)
        s = xmd_x.PimdSystem(lib, N, P, 0.5, 1.0, box=box)
        s.set_state(**random_state(3, 4, N, P, 1.0, box, True, seed=3))
        m = xmd_x.EwaldModel(lib, s, nsum_cheap=2, capacity=1, seed=1)
        X = np.random.default_rng(2).standard_normal((256, 64)).astype(np.float32)
        Y = m.forward(X)
        Yo = orc.mlp_forward(X.astype(np.float64), m.params().astype(np.float64), bf=1)
        assert np.abs(Y - Yo).max() <= 5e-3 * max(1.0, np.abs(Yo).max())
        m.free()
        s.free()
    finally:
        lib.md_gb300_set_wait_limit_x(default)
    assert lib.md_gb300_set_wait_limit_x(0) != 0  # refused
