"""Solution output and restart files (write_output, output.c:92-191;
read_restart_data, restart.c:50-178) in a NumPy container.

The reference writes HDF5 files; no HDF5 library exists in this build, so the
same datasets go into ``<title>.<iter:09d>.npz`` (the reference's
``<title>.<iter:09d>.h5``):

  iter, t                 the attributes
  phi_total (n_cells, 10) conserved and primitive variables, reference order
  phi_dt    (n_cells, 5)  time derivative of the last residual evaluation
  n_stages, phi_old:<k>   implicit runs: the BDF history (k < n_stages)

A restart reads ``phi_total`` / ``phi_dt`` by the names the writer uses (the
reference's serial reader asks for "solver_data->phi_total", a dataset its
writer never creates) and the history when the scheme keeps one.
"""
from __future__ import annotations

import os

import numpy as np


def output_path(title, iter_, directory="."):
    return os.path.join(directory, f"{title}.{int(iter_):09d}.npz")


def write_output(solver, title, iter_, t, directory="."):
    """The datasets write_output stores, from a solver context (api.Solver)."""
    data = {"iter": np.int64(iter_), "t": np.float64(t), "phi_total": solver.get_state(),
            "phi_dt": solver.get_time_derivative()}
    hist = solver.bdf_history()
    if hist:
        data["n_stages"] = np.int64(len(hist))
        for k, a in enumerate(hist):
            data[f"phi_old:{k}"] = a
    path = output_path(title, iter_, directory)
    with open(path, "wb") as f:
        np.savez(f, **data)
    return path


def read_restart(path):
    """read_restart_data: iter, t, phi_total, phi_dt and phi_old (a list,
    empty when the file has no history)."""
    with np.load(path) as z:
        n = int(z["n_stages"]) if "n_stages" in z else 0
        return {"iter": int(z["iter"]), "t": float(z["t"]), "phi_total": np.array(z["phi_total"]),
                "phi_dt": np.array(z["phi_dt"]), "phi_old": [np.array(z[f"phi_old:{k}"]) for k in range(n)]}
