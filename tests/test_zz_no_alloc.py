"""fv3d_global_residual_noalloc: the residual reduction with its scratch in
a static device array (no device allocation), called through the C ABI and
compared with fv3d_global_residual on two calls in a row.  Collected last so
that it also runs after every other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

from fv3d_gb300 import api, cases

pytestmark = pytest.mark.gpu

_f8p = C.POINTER(C.c_double)


def noalloc(s, dt):
    out = np.full(5, np.nan)
    st = s.lib.fv3d_global_residual_noalloc(s.h, dt, out.ctypes.data_as(_f8p))
    assert st == 0, s.lib.fv3d_last_error(s.h).decode()
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_residual_equals_allocating_entry_point(precision):
    c = cases.tgv_tet(6)
    with api.from_case(c, precision) as s:
        results = []
        for call in range(2):
            if call == 1:
                s.step_explicit("rk33", 2, 0.5)   # a different state for the second call
            s.time_derivative(0.0)
            ref = s.global_residual(0.01)
            got = noalloc(s, 0.01)
            assert np.all(np.isfinite(got))
            assert np.array_equal(got, ref), (call, got, ref)
            results.append(got)
        assert not np.array_equal(results[0], results[1])


def test_noalloc_residual_two_contexts_one_after_the_other():
    """Two contexts of different sizes share the one static array in turn."""
    outs = []
    for n in (5, 4):
        c = cases.tgv_tet(n)
        with api.from_case(c, "fp64") as s:
            s.time_derivative(0.0)
            outs.append((s.global_residual(1.0), noalloc(s, 1.0)))
    for ref, got in outs:
        assert np.array_equal(got, ref)
