"""Explicit run on the GPU: the 1,572,864-cell tetrahedral Taylor-Green
case, 500 RK3 steps in mixed precision, the state back in reference cell
order."""
from fv3d_gb300 import api, cases
c = cases.tgv_tet(64)
with api.from_case(c, "mixed") as s:
    stats = s.step_explicit("rk33", 500, cfl=0.5)
    u = s.get_conserved()                  # (n_cells, 5), reference cell order
