"""Loads a golden fixture (tests/golden/*.npz) back into a mesh + case."""
import glob
import os

import numpy as np

from fv3d_gb300 import meshgen as mg

HERE = os.path.dirname(os.path.abspath(__file__))
PARAM_KEYS = ["kappa", "R_mix", "mu_mix", "Pr", "cfl_scale", "dfl_scale", "flux_scheme",
              "reconstruction", "limiter", "gradient"]


def names():
    """The small fixtures (the full-run fixtures fullrun_*.npz hold no mesh)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                  if not os.path.basename(p).startswith("fullrun_"))


def load(name):
    z = dict(np.load(os.path.join(HERE, "golden", name + ".npz")))
    m = {k[5:]: v for k, v in z.items() if k.startswith("mesh_")}
    nr = m["region_is_boundary"].shape[0]
    mesh = mg.Mesh(region_names=[f"r{i}" for i in range(nr)], name=name,
                   **{k: v for k, v in m.items()})
    params = {}
    for k, v in zip(PARAM_KEYS, z["params"]):
        params[k] = int(v) if k in ("flux_scheme", "reconstruction", "limiter", "gradient") else float(v)
    return mesh, params, z
