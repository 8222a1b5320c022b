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
    u, st, rows, _ = params.run(sim, c.mesh)
    assert st["iter"] == 5 and len(rows) == 5
    rt = np.array([mg.BC_FLOW, mg.BC_INFLOW, mg.BC_OUTFLOW, mg.BC_WALL_ADIABATIC])
    p = dict(c.params, limiter=cases.NO_LIMITER)
    with api.Solver(c.mesh, p, rt, c.region_prim, "fp64") as s:
        s.set_state(c.u0)
        st2, rows2 = s.timedisc("rk33", max_iter=5, is_transient=True, t_end=1.0, cfl=0.0)
        u2 = s.get_conserved()
    assert np.array_equal(u, u2)
    assert [r[3] for r in rows] == [r[3] for r in rows2]


def test_output_files_and_restart(tmp_path):
    """Output/i_output_data files (the write_output datasets, .npz) and a
    restart from the last one continue the run exactly: the channel's time
    step is viscous-bound (new density only), so the restarted dt equals the
    continuous run's."""
    from fv3d_gb300 import output
    sim = params.load_simulation(SIM)
    c = cases.channel(6, 4, 4)
    u5, st, rows, files = params.run(sim, c.mesh, output_dir=str(tmp_path))
    assert [os.path.basename(f) for f in files] == ["channel.000000000.npz", "channel.000000005.npz"]
    r = output.read_restart(files[-1])
    assert r["iter"] == 5 and r["t"] == st["t"] and np.array_equal(r["phi_total"][:, :5], u5)
    assert r["phi_dt"].shape == (c.mesh.n_cells, 5) and r["phi_old"] == []
    sim10 = params.load_simulation(SIM)
    sim10.max_iter = 10
    u10, st10, rows10, _ = params.run(sim10, c.mesh)
    simr = params.load_simulation(SIM)
    simr.use_restart, simr.restart_file = True, files[-1]
    ur, str_, rowsr, _ = params.run(simr, c.mesh)
    assert str_["iter"] == 10 and [x[0] for x in rowsr] == list(range(6, 11))
    assert np.array_equal(ur, u10)
    assert [x[3] for x in rowsr] == [x[3] for x in rows10[5:]]
