"""Implicit steady solve (pseudo-transient Newton-Krylov, FGMRES, block
Jacobi) on the channel case, checked through the C ABI.

The converged GPU state is handed to the CPU oracle: its FP64 residual (the
reference's discretisation, restated) must be reduced by the same factor,
i.e. the GPU solution satisfies the reference's discrete steady equations.
"""
import numpy as np
import pytest

from fv3d_gb300 import api, cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-8


def small_channel():
    c = cases.channel(12, 8, 4)
    return c


@pytest.fixture(scope="module")
def oracle():
    return orc.Oracle("restated")


def oracle_residual_norm(o, c, u):
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(u)
    return np.linalg.norm(o.time_derivative(0.0))


@pytest.mark.parametrize("jv", ["fp64", "fp32"])
def test_channel_converges_and_satisfies_reference_equations(oracle, jv):
    c = small_channel()
    with api.from_case(c, "fp64") as s:
        st = s.solve_implicit(jv_precision=jv, tol_rel=TOL)
        hist = s.implicit_history()
        u = s.get_conserved()
    assert st["converged"] == 1 and st["rel_res"] <= TOL
    assert hist[-1] / hist[0] <= TOL
    r0 = oracle_residual_norm(oracle, c, c.u0)
    r1 = oracle_residual_norm(oracle, c, u)
    assert r1 / r0 <= 10 * TOL, (r1 / r0)


def test_fp32_and_fp64_jv_reach_the_same_steady_state():
    c = small_channel()
    sols = []
    for jv in ("fp64", "fp32"):
        with api.from_case(c, "fp64") as s:
            s.solve_implicit(jv_precision=jv, tol_rel=TOL)
            sols.append(s.get_conserved())
    # both satisfy the FP64 steady equations to 1e-8 (checked against the
    # oracle above); the states agree to the accuracy that implies
    scale = np.maximum(np.abs(sols[0]).max(axis=0), 0.3 * np.abs(sols[0][:, 0]).max())
    assert (np.abs(sols[0] - sols[1]).max(axis=0) / scale).max() < 1e-6


def test_lumped_blocks_match_reference_jacobian(oracle):
    """The reference's lumped blocks (implicit.c:61-119: every cell perturbed
    at once by +-eps/2, eps = 1e-4 ||U_v||) from the GPU FP64 residual against
    the oracle's calc_jacobian_numerical.  Off-diagonal entries only: the
    diagonal also carries 1/dt, global in the reference and local here."""
    c = small_channel()
    oracle.init(c.mesh, c.params, c.region_type, c.region_prim)
    oracle.set_conserved(c.u0)
    oracle.step_newton(0, 0.0, 1e-3, scheme=0, solver=1, max_iter_inner=3, is_transient=False)
    ref = oracle.jacobian()                       # [cell, col, row]
    with api.from_case(c, "fp64") as s:
        s.solve_implicit(preconditioner="lumped", tol_rel=1e-12, max_newton=1, check=False)
        gpu = s.blocks()
    off = ~np.eye(5, dtype=bool)
    scale = np.abs(ref).max()
    assert np.abs(gpu[:, off] - ref[:, off]).max() / scale < 1e-6


def test_lumped_blocks_available():
    c = small_channel()
    with api.from_case(c, "fp64") as s:
        st = s.solve_implicit(preconditioner="lumped", tol_rel=1e-3, max_newton=5, check=False)
        b = s.blocks()
    assert np.all(np.isfinite(b))
    assert st["newton_steps"] >= 1


@pytest.mark.parametrize("pc", ["none", "block_jacobi"])
def test_sync_chunk_does_not_change_the_solve(pc):
    """Arnoldi steps launched in chunks of 1, 7 or 31 between host
    synchronisations: the same Krylov and Newton counts and bitwise the same
    state (a chunk only moves the Givens rotations in time; steps computed
    past a cycle's convergence are discarded)."""
    c = small_channel()
    out = []
    with api.from_case(c, "fp64") as s:
        for se in (1, 7, 31):
            s.set_state(c.u0)
            st = s.solve_implicit(preconditioner=pc, max_newton=6, max_restarts=1, sync_every=se, check=False)
            out.append(((st["newton_steps"], st["gmres_iterations"], st["rel_res"]), s.get_conserved()))
    for stats, u in out[1:]:
        assert stats == out[0][0]
        assert np.array_equal(u, out[0][1])


# the relative L2 error of the FP32 finite-difference product against the
# FP64 one: FP32 residuals (rounding ~1e-7 of the face fluxes) divided by a
# step of 5e-4 (1 + |U|) / |z|; measured on GB300 5.5e-4 to 7.3e-4 on the
# walled 12x8x4 channel for every boundary type (the FP64 product against the
# oracle's: 3.2e-10 to 4.1e-10)
JV_FP32_TOL = 2e-3


@pytest.mark.parametrize("btype", [None, "isothermal", "slip", "symmetry", "state", "outflow"])
def test_jacobian_vector_fp32_and_fp64_against_the_oracle(oracle, btype):
    """The implicit solve's matrix-free product J z on the walled channel
    (every boundary type): the FP64 product against the same finite
    difference of the oracle's residual, and the FP32 product (what the
    solve runs) against the FP64 one, on random directions z."""
    from fv3d_gb300 import meshgen as mg
    from test_gpu_parity import perturbed, walled_channel
    bt = {None: None, "isothermal": mg.BC_WALL_ISOTHERMAL, "slip": mg.BC_WALL_SLIP,
          "symmetry": mg.BC_SYMMETRY, "state": mg.BC_STATE, "outflow": mg.BC_OUTFLOW}[btype]
    c = walled_channel(bt, 12, 8, 4)
    u = perturbed(c)
    oracle.init(c.mesh, c.params, c.region_type, c.region_prim)
    rng = np.random.default_rng(11)
    with api.Solver(c.mesh, c.params, c.region_type, c.region_prim, "mixed") as s:
        s.set_state(u)
        for trial in range(3):
            z = rng.standard_normal(u.shape) * np.abs(u).mean(axis=0)
            j64 = s.jacobian_vector(z, "fp64", 1e-7)
            j32 = s.jacobian_vector(z, "fp32")
            eps = 1e-7 * (1 + np.linalg.norm(u)) / np.linalg.norm(z)
            oracle.set_conserved(u)
            r0 = oracle.time_derivative(0.0)
            oracle.set_conserved(u + eps * z)
            j_ref = (oracle.time_derivative(0.0) - r0) / eps
            e64 = np.linalg.norm(j64 - j_ref) / np.linalg.norm(j_ref)
            e32 = np.linalg.norm(j32 - j64) / np.linalg.norm(j64)
            print(btype, trial, "Jv fp64 vs oracle", e64, "fp32 vs fp64", e32)
            assert e64 < 1e-6, e64
            assert e32 < JV_FP32_TOL, e32
        # the products leave the state and its FP32 records as they were
        assert np.array_equal(s.get_conserved(), u)
        r = s.time_derivative(0.0)
    oracle.set_conserved(u)
    assert np.abs(r - oracle.time_derivative(0.0)).max() / np.abs(r).max() < 1e-5
