"""A simulation parameter file run through the reference's program flow
(set_solution + timedisc with calc_ns_timestep as written) gives the same
state as the same run set up by hand through the API."""
import os

import numpy as np
import pytest

from fv3d_gb300 import api, cases, meshgen as mg, params

pytestmark = pytest.mark.gpu
SIM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "channel_simulation.json")


def test_parameter_file_run_matches_manual_setup():
    sim = params.load_simulation(SIM)
    c = cases.channel(6, 4, 4)
    u, st, rows = params.run(sim, c.mesh)
    assert st["iter"] == 5 and len(rows) == 5
    rt = np.array([mg.BC_FLOW, mg.BC_INFLOW, mg.BC_OUTFLOW, mg.BC_WALL_ADIABATIC])
    p = dict(c.params, limiter=cases.NO_LIMITER)
    with api.Solver(c.mesh, p, rt, c.region_prim, "fp64") as s:
        s.set_state(c.u0)
        st2, rows2 = s.timedisc("rk33", max_iter=5, is_transient=True, t_end=1.0, cfl=0.0)
        u2 = s.get_conserved()
    assert np.array_equal(u, u2)
    assert [r[3] for r in rows] == [r[3] for r in rows2]
