"""FV3D simulation parameter files (the JSON layout the reference's parameter
module reads: every parameter an object whose "value" holds the setting;
boundary regions as plain objects) mapped onto this library's configuration.

Keys follow the reference's parameter paths:
  Equation/Navier-Stokes/{kappa, R_mix, mu_mix, Pr, cfl_scale, dfl_scale}
      (navier_stokes.c:55-75), .../Flux/flux_scheme (flux.c:273-312),
      .../Boundary/<region name>/{type, u, v, w, p, T} (boundary.c:55-183)
  FV/Reconstruction/reconstruction (reconstruction.c:44-55),
      FV/Limiter/limiter (limiter.c:44-50)
  TimeDisc/{timestep, max_iter, transient, abort_residual, t_start, t_end}
      (timedisc.c:64-80), TimeDisc/Explicit/scheme (explicit.c:47-60),
      TimeDisc/Implicit/{scheme, max_iter_inner, ...} (implicit.c:77-112)
  Mesh/mesh_file, Output/i_output_data (output.c:20-23),
  Restart/{use_restart, restart_file} (restart.c:20-30)
and, for settings the reference does not have, a GPU subtree:
  GPU/precision ("FP64" | "Mixed"), GPU/renumbering ("None" | "Morton" |
  "RCM"), GPU/cfl (explicit steps' CFL number; 0 or less: calc_ns_timestep
  with cfl_scale / dfl_scale, as the reference)
HDF5 files cannot be read or written in this build (no HDF5 library): the
mesh is passed in (``meshgen`` / ``gmsh``), and output / restart files are the
NumPy containers of ``output`` with the same datasets.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field

import numpy as np

from . import cases, meshgen as mg

_MISSING = object()

BOUNDARY_TYPES = {"flow": mg.BC_FLOW, "inflow": mg.BC_INFLOW, "outflow": mg.BC_OUTFLOW,
                  "wall-adiabatic": mg.BC_WALL_ADIABATIC, "wall-isothermal": mg.BC_WALL_ISOTHERMAL,
                  "wall-slip": mg.BC_WALL_SLIP, "symmetry": mg.BC_SYMMETRY, "state": mg.BC_STATE,
                  "function": mg.BC_FUNCTION}
FLUX = {"AUSM": cases.AUSM, "Rusanov": cases.RUSANOV}
RECONSTRUCTION = {"First-Order": cases.FIRST_ORDER, "Linear": cases.LINEAR}
LIMITER = {"Barth-Jespersenn": cases.BARTH_JESPERSEN, "None": cases.NO_LIMITER}
EXPLICIT = {"Euler": "euler", "RK3-3": "rk33", "RK4-5": "rk45"}
IMPLICIT = {"Euler": "euler", "BDF-2": "bdf2"}
PRECISION = {"FP64": "fp64", "Mixed": "mixed"}
RENUMBERING = {"None": "none", "Morton": "morton", "RCM": "rcm"}


def _get(tree, path, default=_MISSING):
    node = tree
    for key in path.split("/"):
        if not isinstance(node, dict) or key not in node:
            if default is _MISSING:
                raise KeyError(f"parameter {path} missing")
            return default
        node = node[key]
    if isinstance(node, dict) and "value" in node:
        return node["value"]
    return node


def _pick(table, name, what):
    if name not in table:
        raise ValueError(f"{what} {name!r} not supported (one of {sorted(table)})")
    return table[name]


@dataclass
class Simulation:
    title: str
    mesh_file: str
    params: dict                       # fv3d_config physics and scheme options
    boundaries: dict                   # region name -> (type code, (u, v, w, p, T))
    implicit: bool
    scheme: str                        # euler / rk33 / rk45, or euler / bdf2 when implicit
    max_iter: int
    transient: bool
    abort_residual: float
    t_start: float
    t_end: float
    max_iter_inner: int = 100
    i_output_data: int = -1
    use_restart: bool = False
    restart_file: str = ""
    precision: str = "fp64"
    renumbering: str = "morton"
    cfl: float = 0.0
    extra: dict = field(default_factory=dict)

    def regions(self, mesh):
        """region_type and region_prim arrays in the mesh's region order."""
        types, prims = [], []
        flow = self.boundaries.get(mesh.region_names[0], (None, None))[1]
        for name in mesh.region_names:
            if name not in self.boundaries:
                raise KeyError(f"no boundary condition for region {name!r}")
            t, prim = self.boundaries[name]
            if t in (mg.BC_OUTFLOW, mg.BC_WALL_ADIABATIC, mg.BC_WALL_SLIP, mg.BC_SYMMETRY) and flow is not None:
                prim = flow      # no state of their own: a finite placeholder
            elif t == mg.BC_WALL_ISOTHERMAL and flow is not None:
                prim = flow[:4] + (prim[4],)
            types.append(t)
            prims.append(prim)
        return np.asarray(types, dtype=np.int64), np.asarray(prims, dtype=np.float64)

    def initial_state(self, mesh):
        """set_solution with calc_ns_exact_function (navier_stokes.c:133-152):
        every cell takes the flow region's state."""
        t, (u, v, w, p, T) = self.boundaries[mesh.region_names[0]]
        if t != mg.BC_FLOW:
            raise ValueError("region 0 must be the flow region")
        rho = p / (self.params["R_mix"] * T)
        one = np.ones(mesh.n_cells)
        return cases.prim_to_cons(rho * one, u * one, v * one, w * one, p * one, self.params["kappa"])


def load_simulation(src) -> Simulation:
    """Parse a simulation parameter file (path, JSON text or dict)."""
    if isinstance(src, dict):
        tree = src
    elif src.lstrip().startswith("{"):
        tree = json.loads(src)
    else:
        with open(src) as f:
            tree = json.load(f)
    eq = _get(tree, "Equation/equation", "Navier-Stokes")
    if eq != "Navier-Stokes":
        raise ValueError(f"equation {eq!r} not supported")
    ns = "Equation/Navier-Stokes/"
    params = dict(kappa=float(_get(tree, ns + "kappa", 1.4)), R_mix=float(_get(tree, ns + "R_mix", 8.31446261815324 / 28.96e-3)),
                  mu_mix=float(_get(tree, ns + "mu_mix", 18.13e-6)), Pr=float(_get(tree, ns + "Pr", 0.718)),
                  cfl_scale=float(_get(tree, ns + "cfl_scale", 1.0)), dfl_scale=float(_get(tree, ns + "dfl_scale", 1.0)),
                  flux_scheme=_pick(FLUX, _get(tree, ns + "Flux/flux_scheme", "AUSM"), "flux scheme"),
                  reconstruction=_pick(RECONSTRUCTION, _get(tree, "FV/Reconstruction/reconstruction", "Linear"),
                                       "reconstruction"),
                  limiter=_pick(LIMITER, _get(tree, "FV/Limiter/limiter", "Barth-Jespersenn"), "limiter"),
                  gradient=cases.GREEN_GAUSS)
    boundaries = {}
    for name, b in _get(tree, ns + "Boundary", {}).items():
        t = _pick(BOUNDARY_TYPES, b["type"], "boundary type")
        if t == mg.BC_FUNCTION:
            raise ValueError("the 'function' boundary type is not supported (the reference cannot configure it)")
        prim = [float(b.get(k, 0.0)) for k in ("u", "v", "w", "p", "T")]
        boundaries[name] = (t, tuple(prim))
    use_restart = bool(_get(tree, "Restart/use_restart", False))
    restart_file = str(_get(tree, "Restart/restart_file", ""))
    if use_restart and restart_file.endswith(".h5"):
        raise ValueError("HDF5 restart files cannot be read in this build: give the .npz output file")
    implicit = _pick({"Explicit": False, "Implicit": True}, _get(tree, "TimeDisc/timestep", "Explicit"), "timestep")
    if implicit:
        scheme = _pick(IMPLICIT, _get(tree, "TimeDisc/Implicit/scheme", "Euler"), "implicit scheme")
    else:
        scheme = _pick(EXPLICIT, _get(tree, "TimeDisc/Explicit/scheme", "RK3-3"), "explicit scheme")
    inner = _get(tree, "TimeDisc/Implicit/max_iter_inner", _get(tree, "TimeDisc/Implicit/max_iter", 100))
    return Simulation(title=str(_get(tree, "General/title", "untitled")), mesh_file=str(_get(tree, "Mesh/mesh_file", "")),
                      params=params, boundaries=boundaries, implicit=implicit, scheme=scheme,
                      max_iter=int(_get(tree, "TimeDisc/max_iter", 1000)),
                      transient=bool(_get(tree, "TimeDisc/transient", True)),
                      abort_residual=float(_get(tree, "TimeDisc/abort_residual", 1e-10)),
                      t_start=float(_get(tree, "TimeDisc/t_start", 0.0)), t_end=float(_get(tree, "TimeDisc/t_end", 0.2)),
                      max_iter_inner=int(inner), i_output_data=int(_get(tree, "Output/i_output_data", -1)),
                      use_restart=use_restart, restart_file=restart_file,
                      precision=_pick(PRECISION, _get(tree, "GPU/precision", "FP64"), "precision"),
                      renumbering=_pick(RENUMBERING, _get(tree, "GPU/renumbering", "Morton"), "renumbering"),
                      cfl=float(_get(tree, "GPU/cfl", 0.0)))


def run(sim: Simulation, mesh, precision=None, cfl=None, check=True, output_dir=None):
    """The reference's program flow on the GPU: set up the solver from the
    parameters, set_solution (or read_restart_data), timedisc with
    write_output into output_dir (None: no files).  precision and cfl
    default to the file's GPU settings; cfl <= 0 takes calc_ns_timestep as
    written (cfl_scale, dfl_scale), as the reference does; returns the
    final conserved state, the timedisc stats, the residual rows and the
    output files written."""
    from . import api, output
    precision = sim.precision if precision is None else precision
    cfl = sim.cfl if cfl is None else cfl
    rt, rp = sim.regions(mesh)
    written = []
    with api.Solver(mesh, sim.params, rt, rp, precision, sim.renumbering) as s:
        iter_start, t_start = 0, sim.t_start
        if sim.use_restart:
            r = output.read_restart(sim.restart_file)
            if r["phi_total"].shape != (mesh.n_cells, 10):
                raise ValueError("restart file does not match the mesh")
            s.set_state(r["phi_total"][:, :5])
            iter_start, t_start = r["iter"], r["t"]
            if sim.implicit and r["phi_old"]:
                s.set_bdf_history(sim.scheme, r["phi_old"])
        else:
            s.set_state(sim.initial_state(mesh))

        def on_output(it, t):
            written.append(output.write_output(s, sim.title, it, t, output_dir))

        st, rows = s.timedisc(sim.scheme, implicit=sim.implicit, max_iter=sim.max_iter, is_transient=sim.transient,
                              abort_residual=sim.abort_residual, t_start=t_start, t_end=sim.t_end, cfl=cfl,
                              max_iter_inner=sim.max_iter_inner, check=check, iter_start=iter_start,
                              i_output_data=sim.i_output_data if output_dir is not None else 0,
                              on_output=on_output if output_dir is not None else None)
        return s.get_conserved(), st, rows, written
