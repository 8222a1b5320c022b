"""fv3d_timedisc against the reference's time loop (timedisc.c:134-222)
driven on the oracle: the same dt per iteration (clipped to t_end), the same
calc_global_residual rows, the same stop iteration for each criterion
(t_end, abort_residual, max_iter), for explicit and implicit steps."""
import numpy as np
import pytest

from fv3d_gb300 import api, cases
from oracle import oracle as orc
from parity import rel_l2

pytestmark = pytest.mark.gpu

SCHEME_ID = {"euler": 0, "rk33": 1, "rk45": 2}


def oracle_timedisc(c, scheme, t_end, max_iter, is_transient, abort, cfl, implicit=False, u0=None):
    """timedisc.c:134-222 on the oracle (steady: t_end = infinity)."""
    o = orc.Oracle("restated")
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0 if u0 is None else u0)
    t_end = t_end if is_transient else np.inf
    t, it, rows = 0.0, 0, []
    o.time_derivative(t)
    while True:
        # cfl <= 0: calc_ns_timestep as written (on the oracle's phi_total,
        # whose primitives after a low-storage step are the last stage's input)
        dt = o.timestep_convective(cfl) if cfl > 0 else o.calc_ns_timestep()
        fin = False
        if t + dt > t_end:
            dt, fin = t_end - t, True
        if implicit:
            ni, _ = o.step_newton(it, t, dt, scheme={"euler": 0, "bdf2": 1}[scheme], solver=1, max_iter_inner=20,
                                  tolerance_lsoe=1e-12, max_iter_lsoe=200, krylov_dims=30, krylov_restarts=10,
                                  is_transient=is_transient)
        elif scheme == "ssprk3":
            o.step_ssprk3(t, dt)
        else:
            o.step_lserkw2(SCHEME_ID[scheme], it, t, dt)
        res = o.global_residual(dt)
        t += dt
        it += 1
        rows.append((it, t, dt, list(res)))
        if not is_transient and max(res) < abort:
            fin = True
        if it >= max_iter:
            fin = True
        if fin:
            break
    return rows, o.conserved()


def compare(rows_gpu, rows_ref, tol):
    assert len(rows_gpu) == len(rows_ref)
    for g, r in zip(rows_gpu, rows_ref):
        assert g[0] == r[0]
        assert abs(g[1] - r[1]) <= max(1e-12, tol) * abs(r[1])
        assert abs(g[2] - r[2]) <= tol * r[2]
        assert np.allclose(g[3], r[3], rtol=tol, atol=0.0)


def test_explicit_transient_stops_at_t_end_fp64():
    c = cases.tgv_hex(4)
    probe, _ = oracle_timedisc(c, "rk33", 1e9, 6, True, 0.0, 0.5)
    t_end = 0.5 * (probe[4][1] + probe[5][1])   # inside the sixth step: the last dt is clipped
    rows_ref, u_ref = oracle_timedisc(c, "rk33", t_end, 1000, True, 0.0, 0.5)
    with api.from_case(c, "fp64") as s:
        st, rows = s.timedisc("rk33", max_iter=1000, is_transient=True, t_end=t_end, cfl=0.5)
        u = s.get_conserved()
    assert st["stop_reason"] == 0 and st["iter"] == 6 and abs(st["t"] - t_end) < 1e-14
    compare(rows, rows_ref, 1e-10)
    assert rel_l2(u, u_ref).max() < 1e-10


def test_explicit_steady_abort_and_max_iter():
    c = cases.channel(6, 4, 4)
    probe, _ = oracle_timedisc(c, "rk33", 0.0, 12, False, 0.0, 0.5)
    # an abort threshold crossed for the first time at some iteration k
    maxes = [max(r[3]) for r in probe]
    k = next(i for i in range(3, len(maxes)) if maxes[i] < min(maxes[:i]))
    abort = 0.5 * (maxes[k] + min(maxes[:k]))
    rows_ref, u_ref = oracle_timedisc(c, "rk33", 0.0, 1000, False, abort, 0.5)
    with api.from_case(c, "fp64") as s:
        st, rows = s.timedisc("rk33", max_iter=1000, is_transient=False, abort_residual=abort, cfl=0.5)
        u = s.get_conserved()
        assert st["stop_reason"] == 1 and st["iter"] == k + 1
        compare(rows, rows_ref, 1e-10)
        assert rel_l2(u, u_ref).max() < 1e-10
        s.set_state(c.u0)
        st, rows = s.timedisc("rk33", max_iter=4, is_transient=False, abort_residual=0.0, cfl=0.5)
    assert st["stop_reason"] == 2 and st["iter"] == 4 and len(rows) == 4


def test_explicit_mixed_follows_reference_loop():
    c = cases.tgv_tet(4)
    rows_ref, u_ref = oracle_timedisc(c, "rk33", 1e9, 8, True, 0.0, 0.5)
    with api.from_case(c, "mixed") as s:
        st, rows = s.timedisc("rk33", max_iter=8, is_transient=True, t_end=1e9, cfl=0.5)
        u = s.get_conserved()
    assert st["stop_reason"] == 2 and len(rows) == 8
    compare(rows, rows_ref, 1e-4)
    assert rel_l2(u, u_ref).max() < 1e-5


@pytest.mark.parametrize("scheme", ["euler", "bdf2"])
def test_implicit_transient(scheme):
    c = cases.channel(6, 4, 4)
    rows_ref, u_ref = oracle_timedisc(c, scheme, 1e9, 4, True, 0.0, 2.0, implicit=True)
    with api.from_case(c, "fp64") as s:
        st, rows = s.timedisc(scheme, implicit=True, max_iter=4, is_transient=True, t_end=1e9, cfl=2.0,
                              max_iter_inner=20)
        u = s.get_conserved()
    assert st["stop_reason"] == 2 and len(rows) == 4
    compare(rows, rows_ref, 1e-9)
    assert rel_l2(u, u_ref).max() < 1e-10


@pytest.mark.parametrize("case,scheme", [("hex4", "rk33"), ("hex4", "rk45"), ("channel", "rk33"), ("hex4", "ssprk3")])
def test_calc_ns_timestep_as_written(case, scheme):
    """cfl <= 0: each iteration's dt is calc_ns_timestep on the reference's
    phi_total.  On the hexes the convective bound decides (after a low-storage
    step it sees the new density with the last stage's input u, v, w, p); on
    the channel the viscous bound (new density only)."""
    c = cases.tgv_hex(4) if case == "hex4" else cases.channel(6, 4, 4)
    rows_ref, u_ref = oracle_timedisc(c, scheme, 1e9, 6, True, 0.0, 0.0)
    with api.from_case(c, "fp64") as s:
        st, rows = s.timedisc(scheme, max_iter=6, is_transient=True, t_end=1e9, cfl=0.0)
        u = s.get_conserved()
    assert st["stop_reason"] == 2 and len(rows) == 6
    compare(rows, rows_ref, 1e-10)
    assert rel_l2(u, u_ref).max() < 1e-10


def test_output_cadence():
    """on_output where timedisc calls write_output: iteration 0 (after the
    initial time derivative), every i_output_data-th, the last; none on a
    restart; the datasets readable from the callback."""
    c = cases.tgv_hex(4)
    o = orc.Oracle("restated")
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0)
    r0 = o.time_derivative(0.0)
    with api.from_case(c, "fp64") as s:
        for every, expect in ((2, [0, 2, 4, 5]), (-1, [0, 5]), (0, [])):
            s.set_state(c.u0)
            seen = []

            def out(it, t):
                seen.append((it, t, s.get_state(), s.get_time_derivative()))

            st, rows = s.timedisc("rk33", max_iter=5, is_transient=True, t_end=1e9, cfl=0.5,
                                  i_output_data=every, on_output=out)
            assert [x[0] for x in seen] == expect
            if seen:
                assert seen[0][1] == 0.0 and rel_l2(seen[0][3], r0).max() < 1e-12
                assert abs(seen[-1][1] - st["t"]) == 0.0
                assert np.array_equal(seen[-1][2][:, :5], s.get_conserved())
        seen = []
        s.timedisc("rk33", max_iter=3, is_transient=True, t_end=1e9, cfl=0.5, iter_start=5,
                   i_output_data=2, on_output=lambda it, t: seen.append(it))
        assert seen == [6, 8]


def test_implicit_bdf2_restart_is_exact():
    """Four BDF2 iterations in one run, or two, an output, and two more
    continued from the output's state and history (read_restart_data):
    bitwise the same state."""
    c = cases.channel(6, 4, 4)
    kw = dict(implicit=True, is_transient=True, t_end=1e9, cfl=2.0, max_iter_inner=20)
    with api.from_case(c, "fp64") as s:
        s.timedisc("bdf2", max_iter=4, **kw)
        u_full = s.get_conserved()
    saved = {}
    with api.from_case(c, "fp64") as s:
        def out(it, t):
            saved.update(iter=it, t=t, phi=s.get_state(), hist=s.bdf_history())

        s.timedisc("bdf2", max_iter=2, i_output_data=-1, on_output=out, **kw)
    assert saved["iter"] == 2 and len(saved["hist"]) == 2
    with api.from_case(c, "fp64") as s:
        s.set_state(saved["phi"][:, :5])
        s.set_bdf_history("bdf2", saved["hist"])
        st, rows = s.timedisc("bdf2", max_iter=2, iter_start=2, t_start=saved["t"], **kw)
        assert st["iter"] == 4 and [r[0] for r in rows] == [3, 4]
        assert np.array_equal(s.get_conserved(), u_full)
    with api.from_case(c, "fp64") as s:     # BDF2 past its start needs the history
        st = s.step_newton(3, 0.0, 1e-3, scheme="bdf2", check=False)
        assert st["status"] != 0
