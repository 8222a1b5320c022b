"""State upload / download through the C ABI from pageable and from
page-locked host memory (the latter read and written by kernels directly
over the host link): bitwise the same state, in the reference's AoS order."""
import numpy as np
import pytest

from fv3d_gb300 import api, cases

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def pinned(shape):
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pinned_and_pageable_round_trips_agree(precision):
    c = cases.tgv_tet(5)
    rng = np.random.default_rng(1)
    u = c.u0 * (1.0 + 0.01 * rng.uniform(-1, 1, c.u0.shape))
    with api.from_case(c, precision) as s:
        s.set_state(u)                       # pageable
        a = s.get_conserved()
        hp = pinned(u.shape)
        hp[:] = u
        s.set_state(hp)                      # page-locked
        out = pinned(u.shape)
        s.get_conserved(out=out)
        assert np.array_equal(a, u) and np.array_equal(out, u)
        # a step from each upload path gives the same state
        s.step_explicit("rk33", 3, cfl=0.5)
        r1 = s.get_conserved()
        s.set_state(u)
        s.step_explicit("rk33", 3, cfl=0.5)
        r2 = pinned(u.shape)
        s.get_conserved(out=r2)
    assert np.array_equal(r1, r2)


def test_exact_function_initial_state():
    """set_exact_function + set_solution: a host function of the cell centre
    gives the same state as uploading it."""
    c = cases.tgv_tet(4)

    def tgv(_id, _t, x):
        u, _ = cases.taylor_green(x[None, :], 0.8)
        return list(u[0]) + [0.0] * 5

    with api.from_case(c, "fp64") as s:
        s.set_exact_function(tgv)
        a = s.get_conserved()
    assert np.allclose(a, c.u0, rtol=1e-15, atol=0.0)


@pytest.mark.parametrize("pinned", [True, False])
def test_step_explicit_io_matches_separate_calls(pinned):
    """fv3d_step_explicit_io (host state in, steps, host state out, one
    synchronisation) gives bitwise what set_state + step_explicit +
    get_conserved give, with page-locked and pageable host rows; with no
    input it continues from the device state."""
    c = cases.tgv_tet(4)
    with api.from_case(c, "mixed") as s:
        s.set_state(c.u0)
        st_ref = s.step_explicit("rk33", 3, cfl=0.5)
        u3 = s.get_conserved()
        s.step_explicit("rk33", 2, cfl=0.5)
        u5 = s.get_conserved()
    with api.from_case(c, "mixed") as s:
        hb = torch.empty((c.mesh.n_cells, 5), dtype=torch.float64, pin_memory=True).numpy() if pinned \
            else np.empty((c.mesh.n_cells, 5))
        hb[:] = c.u0
        st = s.step_explicit_io("rk33", 3, cfl=0.5, u_in=hb, u_out=hb)
        assert np.array_equal(hb, u3)
        assert st["t"] == st_ref["t"] and st["steps"] == st_ref["steps"]
        out = np.empty_like(hb)
        s.step_explicit_io("rk33", 2, cfl=0.5, u_in=None, u_out=out)   # state kept on the device
        assert np.array_equal(out, u5)
