"""Host-side accumulator arithmetic of the C ABI against the reference: the
scalar (es) and function-valued (fxs, the _f forms, md_pimd_x.c:4566-4650)
helpers, on the sequence tests/golden/make_golden.c ran through MD-Lab's own
build.  No GPU: the accumulators live on the host until a device call."""
import numpy as np
import pytest

import fixtures
import xmd_x


@pytest.fixture(scope="module")
def lib():
    return xmd_x.load(3, 4)


def fxs(st):
    s = st.contents
    return np.array([s.fxs[s.N - 1][i] for i in range(s.points)])


@pytest.mark.parametrize("name", ["d3l4_obs_ueg", "d2l4_obs_trap"])
def test_function_valued_accumulators_match_reference(lib, name):
    fx = fixtures.load(name)
    a, b, q = lib.md_alloc_stats_x(5), lib.md_alloc_stats_x(5), lib.md_alloc_stats_x(4)
    for i in range(5):
        b.contents.fxs[0][i] = i + 0.5
    b.contents.es[0] = 1.5
    assert lib.md_reset_stats_f_x(a, 2.0) == 0
    assert np.array_equal(fxs(a), fx["acc/reset"])
    assert lib.md_stats_add_to_f_x(a, b) == 0
    assert np.array_equal(fxs(a), fx["acc/add"])
    assert lib.md_stats_mult_to_f_x(a, b) == 0
    assert np.array_equal(fxs(a), fx["acc/mult"])
    assert lib.md_stats_add_to_f_x(a, q) == fx["acc/add_mismatch_rc"][0]
    assert lib.md_stats_copy_to_f_x(a, q) == fx["acc/copy_mismatch_rc"][0]
    assert np.array_equal(fxs(a), fx["acc/mult"])  # a refused call changes nothing
    assert lib.md_stats_copy_to_f_x(a, b) == 0
    assert np.array_equal(fxs(a), fx["acc/copy"])
    for s in (a, b, q):
        lib.md_gb300_free_stats_x(s)
