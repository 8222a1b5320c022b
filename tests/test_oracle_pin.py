"""Pins the FP64 restatement oracle (oracle/fv3d_oracle.c) to the reference.

* against the committed golden fixtures produced by the reference's own C
  sources (tests/golden/make_golden.py) - runs everywhere;
* against a live build of the reference sources (oracle/_ref) where the
  reference tree is present.
The bar is bit-identity: both are FP64 C with the same operation order and no
floating-point contraction.
"""
import numpy as np
import pytest

import golden_io
from conftest import reference_tree_present
from fv3d_gb300 import cases, meshgen as mg
from oracle import oracle as orc


@pytest.fixture(scope="module")
def restated():
    return orc.Oracle("restated")


@pytest.mark.parametrize("name", golden_io.names())
def test_restated_matches_golden(restated, name):
    mesh, params, z = golden_io.load(name)
    o = restated
    o.init(mesh, params, z["region_type"], z["region_prim"])
    o.set_conserved(z["u_in"])
    assert np.array_equal(o.total(), z["total"])
    assert np.array_equal(o.time_derivative(0.0), z["dphi"])
    for g, key in zip(o.gradients(), ("gx", "gy", "gz")):
        assert np.array_equal(g, z[key]), key
    left, right = o.face_states()
    assert np.array_equal(left, z["left"]) and np.array_equal(right, z["right"])
    assert np.array_equal(o.flux(), z["flux"])
    assert o.timestep_convective(0.5) == z["dt_conv"]
    assert o.calc_ns_timestep() == z["dt_ns"]
    for k, (scheme, nsteps) in enumerate(z["rk_plan"]):
        for s in range(nsteps):
            dt = o.timestep_convective(0.5)
            o.step_lserkw2(int(scheme), s, 0.0, dt)
            o.time_derivative(0.0)
            assert np.array_equal(o.conserved(), z[f"rk{k}_s{scheme}_n{s}"]), (k, s)
            assert np.array_equal(o.global_residual(dt), z[f"rk{k}_s{scheme}_n{s}_res"])
    if int(z["newton"]):
        o.set_conserved(z["u_in"])
        for it in range(int(z["newton"])):
            dt = o.timestep_convective(1.0)
            ni, nl = o.step_newton(it, 0.0, dt, scheme=1, solver=1, krylov_dims=15,
                                   krylov_restarts=2)
            assert [ni, nl] == list(z[f"newton{it}_iters"])
            assert np.array_equal(o.conserved(), z[f"newton{it}"])
        assert np.array_equal(o.jacobian(), z["jacobian"])


def test_reference_quirk_dt_zero_without_viscosity(restated):
    """calc_ns_timestep returns 0 when mu=0 (navier_stokes.c:188,192)."""
    c = cases.euler16(4)
    restated.init(c.mesh, c.params, c.region_type, c.region_prim)
    restated.set_conserved(c.u0)
    assert restated.calc_ns_timestep() == 0.0
    assert restated.timestep_convective(0.5) > 0.0


@pytest.mark.skipif(not reference_tree_present(), reason="reference tree absent")
@pytest.mark.parametrize("maker", [
    lambda: cases.euler16(3),
    lambda: cases.tgv_tet(3),
    lambda: cases.tgv_hex(3),
    lambda: cases.channel(4, 4, 4),
    lambda: cases.tgv_mixed(3),
])
def test_restated_matches_reference_build(restated, maker):
    ref = orc.Oracle("reference")
    c = maker()
    c.params["gradient"] = cases.GREEN_GAUSS
    if c.name == "channel":
        c.region_type[2] = mg.BC_OUTFLOW
    for o in (ref, restated):
        o.init(c.mesh, c.params, c.region_type, c.region_prim)
        o.set_conserved(c.u0)
    for s in range(4):
        dt = ref.timestep_convective(0.5)
        assert dt == restated.timestep_convective(0.5)
        ref.step_lserkw2(1, s, 0.0, dt)
        restated.step_lserkw2(1, s, 0.0, dt)
        assert np.array_equal(ref.conserved(), restated.conserved())
    assert np.array_equal(ref.time_derivative(0.1), restated.time_derivative(0.1))


def test_oracle_rejects_corrupt_mesh(restated):
    """A boundary face without a valid boundary index is refused, not run."""
    c = cases.channel(4, 4, 4)
    bad = c.mesh.face_boundary.copy()
    bad[np.nonzero(bad >= 0)[0][0]] = 10 ** 6
    c.mesh.face_boundary = bad
    with pytest.raises(RuntimeError, match="boundary index"):
        restated.init(c.mesh, c.params, c.region_type, c.region_prim)


@pytest.mark.skipif(not reference_tree_present(), reason="reference tree absent")
@pytest.mark.parametrize("scheme", [0, 1])            # backward Euler, BDF2 (implicit.c:37-38)
@pytest.mark.parametrize("maker", [
    lambda: cases.channel(4, 4, 3),
    lambda: cases.tgv_mixed(3),
])
def test_restated_newton_matches_reference_build(restated, maker, scheme):
    """timestep_newton (implicit.c:224-351) with calc_jacobian_numerical:
    the same inner iteration counts, states and Jacobian blocks, bitwise."""
    ref = orc.Oracle("reference")
    c = maker()
    if c.name == "channel":
        c.region_type[2] = mg.BC_OUTFLOW
        c.params["mu_mix"] = 0.01
    c.params["gradient"] = cases.GREEN_GAUSS
    for o in (ref, restated):
        o.init(c.mesh, c.params, c.region_type, c.region_prim)
        o.set_conserved(c.u0)
    for it in range(3):
        dt = ref.timestep_convective(1.0)
        a = ref.step_newton(it, 0.0, dt, scheme=scheme, solver=1, krylov_dims=15, krylov_restarts=2)
        b = restated.step_newton(it, 0.0, dt, scheme=scheme, solver=1, krylov_dims=15, krylov_restarts=2)
        assert a == b, it
        assert np.array_equal(ref.conserved(), restated.conserved()), it
    assert np.array_equal(ref.jacobian(), restated.jacobian())
