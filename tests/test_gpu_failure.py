"""Failure detection on the GPU without a GPU fault: the bounded device
waits (the staged gradient pass's mbarrier waits) give up after their limit
and report it, and the context stays usable afterwards.  The wait is made to
run out on a barrier phase that no copy completes; nothing faults, traps or
hangs."""
import numpy as np
import pytest

from fv3d_gb300 import api, cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("limit_us", [1000, 20000])
def test_bounded_wait_gives_up_and_context_survives(limit_us):
    c = cases.tgv_tet(3)
    with api.from_case(c, "mixed") as s:
        r0 = s.time_derivative(0.0)
        timed_out, ms = s.selftest_bounded_wait(limit_us)
        assert timed_out == 1
        assert limit_us / 1000.0 <= ms < limit_us / 1000.0 + 100.0
        assert np.array_equal(s.time_derivative(0.0), r0)
        st = s.step_explicit("rk33", 3, cfl=0.5)
        assert np.isfinite(st["t"])


def test_bounded_wait_limit_checked():
    c = cases.tgv_tet(3)
    with api.from_case(c, "mixed") as s:
        for bad in (0, -5, 2000000):
            with pytest.raises(api.FV3DError) as e:
                s.selftest_bounded_wait(bad)
            assert e.value.status == 1
