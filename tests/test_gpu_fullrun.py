"""The benchmark configurations at their stated step counts against the FP64
CPU solution (committed fixtures written by tests/golden/make_fullrun.py):

  tgv_tet64  1,572,864 tetrahedra, 500 RK3-3 steps: the reference's own C
             sources (explicit.c:96-140 and the residual they call)
  tgv_hex64  262,144 jittered hexahedra with least-squares gradients, 200
             RK3-3 steps: the FP64 restatement (least squares has no
             reference counterpart)
  euler16    4,096 hexahedra, first-order Euler, 100 RK3-3 steps: the
             reference's own sources

The fixtures hold the final state of a fixed subsample of cells, the L2 norm
per conserved variable and the volume-weighted totals of the whole state,
and the time reached.  Bars: FP64 <= 1e-10 relative L2 per variable, mixed
FP32/FP64 <= 1e-5.  Measured on GB300 (sampled cells, largest variable):
tgv_tet64 FP64 1.0e-15, mixed 3.7e-8; tgv_hex64 FP64 1.4e-15, mixed 7.3e-7;
euler16 FP64 1.7e-16, mixed 3.5e-8.
"""
import os

import numpy as np
import pytest

from fv3d_gb300 import api, cases
from parity import rel_l2

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
MAKERS = {"tgv_tet64": lambda: cases.tgv_tet(64), "tgv_hex64": lambda: cases.tgv_hex(64),
          "euler16": lambda: cases.euler16(16)}
STATE_TOL = {"fp64": 1e-10, "mixed": 1e-5}
# reference speed for the relative-L2 floor of components that start at zero
U_REF = {"tgv_tet64": 1.0, "tgv_hex64": 1.0, "euler16": 0.5}


def fixture(name):
    path = os.path.join(HERE, "golden", f"fullrun_{name}.npz")
    if not os.path.exists(path):
        pytest.skip(f"{path} not generated")
    return dict(np.load(path))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(MAKERS))
def test_full_run_matches_cpu_fp64_solution(name, precision):
    z = fixture(name)
    c = MAKERS[name]()
    steps, cfl = int(z["steps"]), float(z["cfl"])
    with api.from_case(c, precision) as s:
        st = s.step_explicit("rk33", steps, cfl=cfl)
        u = s.get_conserved()
    assert st["steps"] == steps
    t_err = abs(st["t"] / float(z["t"]) - 1)
    err = rel_l2(u[z["cells"]], z["u"], U_REF[name])
    # norms of components that stay ~0 (rho v, rho w of the Euler stream along
    # x) are compared against the floor |rho| u_ref, as rel_l2 does
    l2_err = np.abs(np.linalg.norm(u, axis=0) - z["l2"]) / np.maximum(z["l2"], z["l2"][0] * U_REF[name])
    vol = c.mesh.cell_volume[:, None]
    tot = (u * vol).sum(axis=0)
    scale = np.maximum(np.abs(c.u0 * vol).sum(axis=0), np.abs(c.u0[:, 0] * vol[:, 0]).sum())
    tot_err = np.abs(tot - z["totals"]) / scale
    print(f"{name} {precision}: sampled rel L2 {err}, time {t_err:.2e}, "
          f"norms {l2_err.max():.2e}, totals {tot_err.max():.2e}")
    tol = STATE_TOL[precision]
    assert t_err < (1e-12 if precision == "fp64" else 1e-5), t_err
    assert err.max() < tol, err
    assert l2_err.max() < tol, l2_err
    assert tot_err.max() < (1e-12 if precision == "fp64" else 1e-6), tot_err
