"""Full-size workloads on the GPU: the jittered-hex LSQ case (64^3 hexes,
262,144 cells) and the tetrahedral case (1,572,864 cells) at the sizes and
step counts of the benchmark configurations.

The CPU oracle is too slow for hundreds of steps at these sizes, so:
  * the FP64 GPU path is checked against the oracle directly for one
    residual evaluation (tets) and two RK3 steps (hexes) at full size,
  * the mixed path is checked against the FP64 GPU path (itself pinned to
    the oracle) over the full step counts, and
  * size-independent properties: conservation of mass, momentum and energy
    on the periodic box, and bit-identical repeats.
"""
import numpy as np
import pytest

from fv3d_gb300 import api, cases
from oracle import oracle as orc
from parity import rel_l2, rel_max

pytestmark = pytest.mark.gpu

FP64_RESIDUAL_TOL = 1e-12
FP64_STATE_TOL = 1e-10
# mixed against FP64 after the full step count (FP32 faces): measured on
# GB300 7.1e-7 (hexes, 200 steps) and 7.3e-8 (tets, 500 steps)
MIXED_FULL_TOL = 1e-5


@pytest.fixture(scope="module")
def hex64():
    return cases.tgv_hex(64)


@pytest.fixture(scope="module")
def tet64():
    return cases.tgv_tet(64)


def totals(c, u):
    """Volume-weighted sums of the five conserved variables."""
    return (np.asarray(u)[:, :5] * c.mesh.cell_volume[:, None]).sum(axis=0)


def test_hex64_lsq_fp64_two_steps_match_oracle(hex64):
    c = hex64
    o = orc.Oracle("restated")
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0)
    t = 0.0
    for k in range(2):
        dt = o.timestep_convective(0.5)
        o.step_lserkw2(1, k, t, dt)
        t += dt
    with api.from_case(c, "fp64") as s:
        s.step_explicit("rk33", 2, cfl=0.5)
        err = rel_l2(s.get_conserved(), o.conserved())
    assert err.max() < FP64_STATE_TOL, err


def test_tet64_residual_fp64_matches_oracle(tet64):
    c = tet64
    o = orc.Oracle("restated")
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0)
    r_ref = o.time_derivative(0.0)
    with api.from_case(c, "fp64") as s:
        r = s.time_derivative(0.0)
    assert rel_max(r, r_ref) < FP64_RESIDUAL_TOL


@pytest.mark.parametrize("which", ["hex64", "tet64"])
def test_mixed_follows_fp64_over_full_run(which, request):
    """200 RK3 steps (hexes) / 500 RK3 steps (tets), CFL 0.5."""
    c = request.getfixturevalue(which)
    steps = c.steps
    out = {}
    for prec in ("fp64", "mixed"):
        with api.from_case(c, prec) as s:
            st = s.step_explicit("rk33", steps, cfl=0.5)
            out[prec] = (s.get_conserved(), st["t"])
    u64, t64 = out["fp64"]
    umx, tmx = out["mixed"]
    assert np.all(np.isfinite(umx))
    assert abs(tmx / t64 - 1) < 1e-5
    err = rel_l2(umx, u64)
    assert err.max() < MIXED_FULL_TOL, err
    # conservation on the periodic box: the face fluxes cancel pairwise
    t0 = totals(c, c.u0)
    scale = np.abs(c.u0[:, :5] * c.mesh.cell_volume[:, None]).sum(axis=0)
    scale = np.maximum(scale, scale[0])   # rho*w starts at zero: floor by the mass
    drift64 = np.abs(totals(c, u64) - t0) / scale
    driftmx = np.abs(totals(c, umx) - t0) / scale
    print(which, "mixed vs fp64", err, "drift fp64", drift64, "drift mixed", driftmx)
    assert drift64.max() < 1e-12, drift64
    assert driftmx.max() < 1e-6, driftmx


def test_tet64_mixed_bit_identical_repeats(tet64):
    c = tet64
    outs = []
    for _ in range(2):
        with api.from_case(c, "mixed") as s:
            s.step_explicit("rk33", 50, cfl=0.5)
            outs.append(s.get_conserved())
    assert np.array_equal(outs[0], outs[1])


def test_mixed_elements_follow_fp64_and_conserve():
    """Hexahedra, prisms and pyramids (24^3 box, 30,000-odd cells of 5 and
    6 faces): the mixed path follows the FP64 path over 100 RK3 steps and
    both conserve mass, momentum and energy on the periodic box."""
    c = cases.tgv_mixed(24)
    out = {}
    for prec in ("fp64", "mixed"):
        with api.from_case(c, prec) as s:
            s.step_explicit("rk33", 100, cfl=0.5)
            out[prec] = s.get_conserved()
    err = rel_l2(out["mixed"], out["fp64"])
    assert err.max() < MIXED_FULL_TOL, err
    t0 = totals(c, c.u0)
    scale = np.abs(c.u0[:, :5] * c.mesh.cell_volume[:, None]).sum(axis=0)
    scale = np.maximum(scale, scale[0])
    assert (np.abs(totals(c, out["fp64"]) - t0) / scale).max() < 1e-12
    assert (np.abs(totals(c, out["mixed"]) - t0) / scale).max() < 1e-6
