"""Generates the golden fixtures in this directory by running the reference's
own C sources (oracle/_ref/libfv3d_ref.so, built by oracle/Makefile.ref from
the reference tree) on small synthetic meshes.

Run where the reference tree exists:  python tests/golden/make_golden.py [name ...]
(no names: every fixture).
Each .npz holds the mesh arrays, physics settings, the input state and the
reference outputs, so the fixtures are self-contained on machines without the
reference tree.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fv3d_gb300 import cases, meshgen as mg  # noqa: E402
from oracle import oracle as orc  # noqa: E402

SEED = 20240601


def perturbed(c, amp=0.01):
    rng = np.random.default_rng(SEED)
    u = c.u0.copy()
    u[:, 0] *= 1.0 + amp * rng.uniform(-1, 1, u.shape[0])
    u[:, 1:4] += amp * rng.uniform(-1, 1, (u.shape[0], 3)) * u[:, :1]
    u[:, 4] *= 1.0 + amp * rng.uniform(-1, 1, u.shape[0])
    return u


def golden_cases():
    c = cases.euler16(4)
    yield "euler_hex4", c, dict(rk=[(1, 5)], newton=0)
    c = cases.tgv_tet(3)
    yield "tgv_tet3", c, dict(rk=[(1, 3), (2, 1), (0, 2)], newton=0)
    c = cases.tgv_hex(4, seed=SEED)
    c.params["gradient"] = cases.GREEN_GAUSS     # LSQ has no reference counterpart
    yield "tgv_hex4_gg", c, dict(rk=[(1, 3)], newton=0)
    c = cases.channel(6, 4, 4)
    c.region_type[2] = mg.BC_OUTFLOW             # the reference's own outlet type
    c.params["mu_mix"] = 0.01
    yield "channel_6x4x4", c, dict(rk=[(1, 2)], newton=3)
    # the other boundary types of boundary.c:252-307 on the outlet (and, for
    # the isothermal wall, the walls), viscous; slip wall and symmetry share
    # one treatment there (boundary.c:280-281, 377-378), so their fixtures
    # differ only in the type code
    for label, btype in (("isothermal", mg.BC_WALL_ISOTHERMAL), ("slip", mg.BC_WALL_SLIP),
                         ("symmetry", mg.BC_SYMMETRY), ("state", mg.BC_STATE)):
        yield f"channel_4x4x3_{label}", boundary_case(btype), dict(rk=[(1, 2)], newton=0)
    # hexahedra, prisms and pyramids (cells of 5 and 6 faces)
    yield "tgv_mixed3", cases.tgv_mixed(3), dict(rk=[(1, 3)], newton=0)


def boundary_case(btype):
    c = cases.channel(4, 4, 3)
    c.params["mu_mix"] = 0.01
    c.region_type[2] = btype
    c.region_prim[2] = [0.2, 0.01, 0.0, 1 / 1.4, 0.9 / 1.4]
    if btype == mg.BC_WALL_ISOTHERMAL:
        c.region_type[3] = btype
        c.region_prim[3] = [0.0, 0.0, 0.0, 1 / 1.4, 0.8 / 1.4]
    return c


def main(only=()):
    ref = orc.Oracle("reference")
    for name, c, what in golden_cases():
        if only and name not in only:
            continue
        ref.init(c.mesh, c.params, c.region_type, c.region_prim)
        u_in = perturbed(c)
        ref.set_conserved(u_in)
        out = {}
        out["total"] = ref.total()
        out["dphi"] = ref.time_derivative(0.0)
        out["gx"], out["gy"], out["gz"] = ref.gradients()
        out["left"], out["right"] = ref.face_states()
        out["flux"] = ref.flux()
        out["dt_conv"] = np.array(ref.timestep_convective(0.5))
        out["dt_ns"] = np.array(ref.calc_ns_timestep())
        k = 0
        for scheme, nsteps in what["rk"]:
            for s in range(nsteps):
                dt = ref.timestep_convective(0.5)
                ref.step_lserkw2(scheme, s, 0.0, dt)
                ref.time_derivative(0.0)
                out[f"rk{k}_s{scheme}_n{s}"] = ref.conserved()
                out[f"rk{k}_s{scheme}_n{s}_res"] = ref.global_residual(dt)
            k += 1
        if what["newton"]:
            ref.set_conserved(u_in)
            for it in range(what["newton"]):
                dt = ref.timestep_convective(1.0)
                ni, nl = ref.step_newton(it, 0.0, dt, scheme=1, solver=1, krylov_dims=15,
                                         krylov_restarts=2)
                out[f"newton{it}"] = ref.conserved()
                out[f"newton{it}_iters"] = np.array([ni, nl])
            out["jacobian"] = ref.jacobian()
        arrays = {f"mesh_{k}": v for k, v in c.mesh.arrays().items()}
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"), **arrays, **out, u_in=u_in,
            region_type=np.asarray(c.region_type, dtype=np.int32),
            region_prim=np.asarray(c.region_prim, dtype=np.float64),
            params=np.array([c.params[k] for k in PARAM_KEYS], dtype=np.float64),
            rk_plan=np.array(what["rk"], dtype=np.int64).reshape(-1, 2),
            newton=np.array(what["newton"]))
        print(name, c.mesh.n_cells, "cells")


PARAM_KEYS = ["kappa", "R_mix", "mu_mix", "Pr", "cfl_scale", "dfl_scale", "flux_scheme",
              "reconstruction", "limiter", "gradient"]

if __name__ == "__main__":
    main(sys.argv[1:])
