"""FV3D simulation parameter files: the JSON layout of the reference's
parameter module mapped onto the solver configuration (no GPU)."""
import json
import os

import numpy as np
import pytest

from conftest import REFERENCE
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


def test_gpu_subtree():
    """Settings the reference has no keys for live under GPU/: absent, the
    run is FP64, Morton-renumbered, with calc_ns_timestep's dt."""
    tree = json.load(open(SIM))
    sim = params.load_simulation(tree)
    assert (sim.precision, sim.renumbering, sim.cfl) == ("fp64", "morton", 0.0)
    tree["GPU"] = {"precision": {"value": "Mixed"}, "renumbering": {"value": "RCM"}, "cfl": {"value": 0.5}}
    sim = params.load_simulation(tree)
    assert (sim.precision, sim.renumbering, sim.cfl) == ("mixed", "rcm", 0.5)
    tree["GPU"]["precision"]["value"] = "FP16"
    with pytest.raises(ValueError, match="precision"):
        params.load_simulation(tree)


NACA = os.path.join(REFERENCE, "misc", "gmsh", "naca0012", "naca0012_simulation.json")


@pytest.mark.skipif(not os.path.exists(NACA), reason="reference tree absent")
def test_reference_example_simulation_file_loads():
    """The parameter file the reference ships with its NACA 0012 example:
    every key the reference's modules read maps to its value."""
    tree = json.load(open(NACA))
    sim = params.load_simulation(NACA)
    ns = tree["Equation"]["Navier-Stokes"]
    for k in ("kappa", "R_mix", "mu_mix", "Pr", "cfl_scale", "dfl_scale"):
        assert sim.params[k] == ns[k]["value"], k
    assert sim.params["flux_scheme"] == cases.AUSM
    assert (sim.params["reconstruction"], sim.params["limiter"]) == (cases.LINEAR, cases.BARTH_JESPERSEN)
    td = tree["TimeDisc"]
    assert (sim.implicit, sim.scheme) == (False, "rk33")
    assert (sim.max_iter, sim.transient, sim.abort_residual, sim.t_start, sim.t_end) == (
        td["max_iter"]["value"], td["transient"]["value"], td["abort_residual"]["value"],
        td["t_start"]["value"], td["t_end"]["value"])
    assert sim.i_output_data == tree["Output"]["i_output_data"]["value"]
    assert sim.use_restart is False and sim.mesh_file == "naca0012.mesh.h5"
    bnd = {name: b["type"] for name, b in ns["Boundary"].items()}      # plain objects
    assert {name: t for name, (t, _) in sim.boundaries.items()} == {
        name: params.BOUNDARY_TYPES[t] for name, t in bnd.items()}
    # the isothermal profile keeps its wall temperature
    assert sim.boundaries["profile"][1][4] == ns["Boundary"]["profile"]["T"]
