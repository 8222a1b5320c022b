"""FV3D simulation parameter files: the JSON layout of the reference's
parameter module mapped onto the solver configuration (no GPU)."""
import json
import os

import numpy as np
import pytest

from fv3d_gb300 import cases, meshgen as mg, params

HERE = os.path.dirname(os.path.abspath(__file__))
SIM = os.path.join(HERE, "golden", "channel_simulation.json")


def test_channel_parameters_map_to_the_channel_case():
    sim = params.load_simulation(SIM)
    c = cases.channel(6, 4, 4)
    for k in ("kappa", "R_mix", "Pr", "cfl_scale", "dfl_scale", "flux_scheme", "reconstruction", "gradient"):
        assert sim.params[k] == c.params[k], k
    assert abs(sim.params["mu_mix"] - c.params["mu_mix"]) < 1e-18
    assert sim.params["limiter"] == cases.NO_LIMITER
    rt, rp = sim.regions(c.mesh)
    # the outlet is an outflow here (the generated channel uses the new pressure outlet)
    assert list(rt) == [mg.BC_FLOW, mg.BC_INFLOW, mg.BC_OUTFLOW, mg.BC_WALL_ADIABATIC]
    assert np.allclose(rp[:2], c.region_prim[:2])
    assert np.allclose(sim.initial_state(c.mesh), c.u0, rtol=1e-15, atol=1e-15)
    assert (sim.implicit, sim.scheme, sim.max_iter, sim.transient, sim.t_end) == (False, "rk33", 5, True, 1.0)
    assert sim.max_iter_inner == 20 and sim.i_output_data == 10


def test_rejections():
    tree = json.load(open(SIM))
    tree["Restart"]["use_restart"]["value"] = True
    tree["Restart"]["restart_file"] = {"value": "channel.000000100.h5"}
    with pytest.raises(ValueError, match="restart"):
        params.load_simulation(tree)
    tree["Restart"]["restart_file"] = {"value": "channel.000000100.npz"}
    sim = params.load_simulation(tree)
    assert sim.use_restart and sim.restart_file.endswith(".npz")
    tree = json.load(open(SIM))
    tree["Equation"]["Navier-Stokes"]["Flux"]["flux_scheme"]["value"] = "Roe"
    with pytest.raises(ValueError, match="flux"):
        params.load_simulation(tree)
    tree = json.load(open(SIM))
    del tree["Equation"]["Navier-Stokes"]["Boundary"]["wall"]
    sim = params.load_simulation(tree)
    with pytest.raises(KeyError, match="wall"):
        sim.regions(cases.channel(6, 4, 4).mesh)
