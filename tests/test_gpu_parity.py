"""GPU (sm_103a) hot path against the CPU oracle, through the C ABI.

Tolerances: FP64 path <= 1e-12 relative per residual evaluation and
<= 1e-10 relative L2 per conserved variable after the stated steps; mixed
path <= 1e-5 relative L2 after the stated steps (FP32 faces, FP64 state).
"""
import numpy as np
import pytest

import golden_io
from fv3d_gb300 import api, cases, meshgen as mg
from oracle import oracle as orc
from parity import rel_l2, rel_max

pytestmark = pytest.mark.gpu

FP64_RESIDUAL_TOL = 1e-12
FP64_STATE_TOL = 1e-10
MIXED_STATE_TOL = 1e-5


@pytest.fixture(scope="module")
def oracle():
    return orc.Oracle("restated")


def perturbed(c, amp=0.01, seed=5):
    rng = np.random.default_rng(seed)
    u = c.u0.copy()
    u[:, 0] *= 1.0 + amp * rng.uniform(-1, 1, u.shape[0])
    u[:, 1:4] += amp * rng.uniform(-1, 1, (u.shape[0], 3)) * u[:, :1]
    u[:, 4] *= 1.0 + amp * rng.uniform(-1, 1, u.shape[0])
    return u


SMALL = {
    "euler_hex4": lambda: cases.euler16(4),
    "tgv_tet3_gg": lambda: cases.tgv_tet(3),
    "tgv_hex4_lsq": lambda: cases.tgv_hex(4),
    "channel_pressure_outlet": lambda: cases.channel(6, 4, 4),
    # hexahedra, prisms and pyramids: cells of 5 and 6 faces (padded slots)
    "tgv_mixed5_gg": lambda: cases.tgv_mixed(5),
    "tgv_mixed5_lsq": lambda: cases.tgv_mixed(5, gradient=cases.LEAST_SQUARES),
}


def boundary_variants():
    out = []
    for t in (mg.BC_OUTFLOW, mg.BC_WALL_ISOTHERMAL, mg.BC_WALL_SLIP, mg.BC_SYMMETRY, mg.BC_STATE):
        out.append((f"channel_outlet_type{t}", t))
    return out


@pytest.mark.parametrize("name", list(SMALL))
@pytest.mark.parametrize("renumber", ["none", "morton", "rcm"])
def test_residual_fp64_matches_oracle(oracle, name, renumber):
    c = SMALL[name]()
    u = perturbed(c)
    oracle.init(c.mesh, c.params, c.region_type, c.region_prim)
    oracle.set_conserved(u)
    r_ref = oracle.time_derivative(0.0)
    with api.Solver(c.mesh, c.params, c.region_type, c.region_prim, "fp64", renumber) as s:
        s.set_state(u)
        r = s.time_derivative(0.0)
        assert rel_max(r, r_ref) < FP64_RESIDUAL_TOL
        # state export in the reference phi_total layout
        assert rel_max(s.get_state(), oracle.total()[: c.mesh.n_cells]) < 1e-14


@pytest.mark.parametrize("label,btype", boundary_variants())
def test_boundary_types_fp64(oracle, label, btype):
    c = cases.channel(6, 4, 4)
    c.params["mu_mix"] = 0.01
    c.region_type[2] = btype
    c.region_prim[2] = [0.2, 0.01, 0.0, 1 / 1.4, 0.9 / 1.4]
    if btype == mg.BC_WALL_ISOTHERMAL:
        c.region_type[3] = btype
        c.region_prim[3] = [0.0, 0.0, 0.0, 1 / 1.4, 0.8 / 1.4]
    u = perturbed(c)
    oracle.init(c.mesh, c.params, c.region_type, c.region_prim)
    oracle.set_conserved(u)
    r_ref = oracle.time_derivative(0.0)
    with api.Solver(c.mesh, c.params, c.region_type, c.region_prim, "fp64") as s:
        s.set_state(u)
        assert rel_max(s.time_derivative(0.0), r_ref) < FP64_RESIDUAL_TOL


def walled_channel(btype, nx, ny, nz, limiter=None):
    """The channel (inflow, adiabatic walls, pressure outlet, periodic z)
    with its outlet region replaced by `btype` (None keeps the pressure
    outlet; an isothermal outlet makes the walls isothermal too), viscous."""
    c = cases.channel(nx, ny, nz)
    c.params["mu_mix"] = 0.01
    if limiter is not None:
        c.params["limiter"] = limiter
    if btype is not None:
        c.region_type[2] = btype
        c.region_prim[2] = [0.2, 0.01, 0.0, 1 / 1.4, 0.9 / 1.4]
        if btype == mg.BC_WALL_ISOTHERMAL:
            c.region_type[3] = btype
            c.region_prim[3] = [0.0, 0.0, 0.0, 1 / 1.4, 0.8 / 1.4]
    return c


# every boundary type the GPU implements, on the outlet region; the inflow
# and the adiabatic walls are in every variant
MIXED_BOUNDARY_VARIANTS = [("pressure_outlet", None), ("outflow", mg.BC_OUTFLOW),
                           ("isothermal", mg.BC_WALL_ISOTHERMAL), ("slip", mg.BC_WALL_SLIP),
                           ("symmetry", mg.BC_SYMMETRY), ("state", mg.BC_STATE)]
# the mixed residual against the FP64 oracle, relative to its largest entry
# (FP32 face arithmetic on a residual that is O(1 %) of the face fluxes)
MIXED_RESIDUAL_TOL = 1e-5


@pytest.mark.parametrize("size", [(6, 4, 4), (12, 8, 4)])
@pytest.mark.parametrize("label,btype", MIXED_BOUNDARY_VARIANTS)
def test_boundary_types_mixed_residual(oracle, label, btype, size):
    """The production (mixed FP32/FP64) kernels on boundary faces: ghost
    states (boundary.c:188-320), ghost gradients (boundary.c:325-412) and
    the ghost side's viscous flux, against the FP64 oracle."""
    c = walled_channel(btype, *size)
    u = perturbed(c)
    oracle.init(c.mesh, c.params, c.region_type, c.region_prim)
    oracle.set_conserved(u)
    r_ref = oracle.time_derivative(0.0)
    with api.Solver(c.mesh, c.params, c.region_type, c.region_prim, "mixed") as s:
        s.set_state(u)
        err = rel_max(s.time_derivative(0.0), r_ref)
    print(label, size, "mixed residual rel max err", err)
    assert err < MIXED_RESIDUAL_TOL, err


@pytest.mark.parametrize("limiter", [cases.NO_LIMITER, cases.BARTH_JESPERSEN])
@pytest.mark.parametrize("label,btype", MIXED_BOUNDARY_VARIANTS)
def test_boundary_types_mixed_20_rk3_steps(oracle, label, btype, limiter):
    """20 RK3 steps at CFL 0.5 on the 12x8x4 walled channel: FP64 GPU and
    mixed against the oracle."""
    c = walled_channel(btype, 12, 8, 4, limiter)
    c.u0 = perturbed(c)
    u_ref, t_ref = run_oracle(oracle, c, "rk33", 20, 0.5)
    with api.from_case(c, "fp64") as s:
        st = s.step_explicit("rk33", 20, cfl=0.5)
        e64 = rel_l2(s.get_conserved(), u_ref, u_ref=0.3)
        assert abs(st["t"] / t_ref - 1) < 1e-12
    with api.from_case(c, "mixed") as s:
        st = s.step_explicit("rk33", 20, cfl=0.5)
        emx = rel_l2(s.get_conserved(), u_ref, u_ref=0.3)
        assert abs(st["t"] / t_ref - 1) < 1e-5
    print(label, limiter, "fp64", e64.max(), "mixed", emx.max())
    assert e64.max() < FP64_STATE_TOL, e64
    assert emx.max() < MIXED_STATE_TOL, emx


@pytest.mark.parametrize("btype", [None, mg.BC_WALL_SLIP, mg.BC_WALL_ISOTHERMAL, mg.BC_STATE])
def test_boundary_types_mixed_tets_20_rk3_steps(oracle, btype):
    """The tetrahedral production kernels (4 face slots: the persistent
    staged gradient pass) on boundary faces: the channel split into Kuhn
    tetrahedra, Barth-Jespersen, viscous, 20 RK3 steps against the oracle."""
    c = cases.channel(12, 6, 4, tets=True)
    c.params.update(limiter=cases.BARTH_JESPERSEN, mu_mix=0.01)
    if btype is not None:
        c.region_type[2] = btype
        c.region_prim[2] = [0.2, 0.01, 0.0, 1 / 1.4, 0.9 / 1.4]
        if btype == mg.BC_WALL_ISOTHERMAL:
            c.region_type[3] = btype
            c.region_prim[3] = [0.0, 0.0, 0.0, 1 / 1.4, 0.8 / 1.4]
    c.u0 = perturbed(c)
    u_ref, t_ref = run_oracle(oracle, c, "rk33", 20, 0.5)
    with api.from_case(c, "mixed") as s:
        st = s.step_explicit("rk33", 20, cfl=0.5)
        emx = rel_l2(s.get_conserved(), u_ref, u_ref=0.3)
        assert abs(st["t"] / t_ref - 1) < 1e-5
    print(btype, "tets mixed", emx.max())
    assert emx.max() < MIXED_STATE_TOL, emx


@pytest.mark.parametrize("name", golden_io.names())
def test_residual_fp64_matches_reference_golden(name):
    """Against outputs of the reference's own C code (committed fixtures)."""
    mesh, params, z = golden_io.load(name)
    with api.Solver(mesh, params, z["region_type"], z["region_prim"], "fp64") as s:
        s.set_state(z["u_in"])
        assert rel_max(s.time_derivative(0.0), z["dphi"]) < FP64_RESIDUAL_TOL
        for k, (scheme, nsteps) in enumerate(z["rk_plan"]):
            for st in range(nsteps):
                s.step_explicit(["euler", "rk33", "rk45"][int(scheme)], 1, cfl=0.5)
                key = f"rk{k}_s{scheme}_n{st}"
                assert rel_max(s.get_conserved(), z[key]) < FP64_STATE_TOL, key


def test_timestep_and_residual_norm(oracle):
    c = cases.tgv_tet(4)
    oracle.init(c.mesh, c.params, c.region_type, c.region_prim)
    oracle.set_conserved(c.u0)
    with api.from_case(c, "fp64") as s:
        assert abs(s.timestep(0.5) / oracle.timestep_convective(0.5) - 1) < 1e-14
        assert abs(s.timestep(0.0) / oracle.calc_ns_timestep() - 1) < 1e-14
        dt = 1e-3
        s.time_derivative(0.0)
        oracle.time_derivative(0.0)
        assert rel_max(s.global_residual(dt), oracle.global_residual(dt)) < 1e-12


def run_oracle(oracle, c, scheme, steps, cfl):
    oracle.init(c.mesh, c.params, c.region_type, c.region_prim)
    oracle.set_conserved(c.u0)
    t = 0.0
    for k in range(steps):
        dt = oracle.timestep_convective(cfl)
        if scheme == "ssprk3":
            oracle.step_ssprk3(t, dt)
        else:
            oracle.step_lserkw2({"euler": 0, "rk33": 1, "rk45": 2}[scheme], k, t, dt)
        t += dt
    return oracle.conserved(), t


def test_euler16_ssprk3_100_steps(oracle):
    """Plain FP64 explicit Euler on the periodic 16^3 box: SSP-RK3, CFL 0.5,
    100 steps, against the CPU oracle."""
    c = cases.euler16(16)
    u_ref, t_ref = run_oracle(oracle, c, "ssprk3", 100, 0.5)
    with api.from_case(c, "fp64") as s:
        st = s.step_explicit("ssprk3", 100, cfl=0.5)
        err = rel_l2(s.get_conserved(), u_ref, u_ref=0.5)
    assert st["steps"] == 100 and abs(st["t"] / t_ref - 1) < 1e-12
    assert err.max() < FP64_STATE_TOL, err


@pytest.mark.parametrize("scheme", ["euler", "rk33", "rk45"])
def test_euler16_low_storage_schemes(oracle, scheme):
    c = cases.euler16(8)
    u_ref, _ = run_oracle(oracle, c, scheme, 20, 0.5)
    with api.from_case(c, "fp64") as s:
        s.step_explicit(scheme, 20, cfl=0.5)
        assert rel_l2(s.get_conserved(), u_ref, 0.5).max() < FP64_STATE_TOL


@pytest.mark.parametrize("maker,steps", [
    (lambda: cases.tgv_hex(8), 20),
    (lambda: cases.tgv_tet(8), 20),
    (lambda: cases.tgv_mixed(6), 20),
    (lambda: cases.tgv_mixed(6, gradient=cases.LEAST_SQUARES), 20),
])
def test_navier_stokes_fp64_and_mixed(oracle, maker, steps):
    c = maker()
    u_ref, _ = run_oracle(oracle, c, "rk33", steps, 0.5)
    with api.from_case(c, "fp64") as s:
        s.step_explicit("rk33", steps, cfl=0.5)
        e64 = rel_l2(s.get_conserved(), u_ref)
    with api.from_case(c, "mixed") as s:
        s.step_explicit("rk33", steps, cfl=0.5)
        emx = rel_l2(s.get_conserved(), u_ref)
    assert e64.max() < FP64_STATE_TOL, e64
    assert emx.max() < MIXED_STATE_TOL, emx


@pytest.mark.parametrize("scheme", ["euler", "rk45", "ssprk3"])
def test_mixed_precision_other_schemes(oracle, scheme):
    """The mixed path with forward Euler, Carpenter-Kennedy RK4(5) and
    SSP-RK3 against the FP64 oracle (RK3 is covered above)."""
    c = cases.tgv_tet(6)
    u_ref, t_ref = run_oracle(oracle, c, scheme, 10, 0.5)
    with api.from_case(c, "mixed") as s:
        st = s.step_explicit(scheme, 10, cfl=0.5)
        err = rel_l2(s.get_conserved(), u_ref)
    assert abs(st["t"] / t_ref - 1) < 1e-5
    assert err.max() < MIXED_STATE_TOL, err


def test_deterministic_and_renumbering_invariant():
    """No atomics in the accumulation: repeated runs are bit-identical, and
    because every cell sums its faces in reference face order the result does
    not depend on the renumbering either."""
    c = cases.tgv_tet(6)
    outs = []
    for renumber in ("morton", "morton", "rcm", "none"):
        with api.from_case(c, "mixed", renumber) as s:
            s.step_explicit("rk33", 5, cfl=0.5)
            outs.append(s.get_conserved())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_nonfinite_state_is_reported():
    c = cases.tgv_tet(4)
    u = c.u0.copy()
    u[7, 4] = np.nan
    with api.Solver(c.mesh, c.params, c.region_type, c.region_prim, "fp64") as s:
        s.set_state(u)
        with pytest.raises(api.FV3DError) as e:
            s.step_explicit("rk33", 3, cfl=0.5)
        assert e.value.status == 3  # FV3D_ERR_NONFINITE


def test_corrupt_mesh_rejected():
    c = cases.channel(4, 4, 4)
    fc = c.mesh.face_cells.copy()
    fc[5, 0] = c.mesh.n_cells + 10
    c.mesh.face_cells = fc
    with pytest.raises(api.FV3DError) as e:
        api.Solver(c.mesh, c.params, c.region_type, c.region_prim, "fp64")
    assert e.value.status == 8  # FV3D_ERR_BOUNDS


def test_empty_and_oversized_meshes_rejected():
    """No cells (empty arrays) and more than 8 face slots per cell are
    refused with FV3D_ERR_INVALID_ARG before anything reaches the device."""
    import dataclasses
    c = cases.euler16(4)
    m = c.mesh
    empty = dataclasses.replace(
        m, cell_x=m.cell_x[:0], cell_volume=m.cell_volume[:0], cell_dx=m.cell_dx[:0],
        cell_n_faces=m.cell_n_faces[:0], cell_faces=m.cell_faces[:0])
    with pytest.raises(api.FV3DError) as e:
        api.Solver(empty, c.params, c.region_type, c.region_prim, "fp64")
    assert e.value.status == 1  # FV3D_ERR_INVALID_ARG
    wide = dataclasses.replace(m, cell_faces=np.hstack([m.cell_faces, np.full((m.n_cells, 3), -1, np.int32)]))
    with pytest.raises(api.FV3DError) as e:
        api.Solver(wide, c.params, c.region_type, c.region_prim, "fp64")
    assert e.value.status == 1


def test_hdf5_load_unsupported():
    c = cases.euler16(4)
    with api.from_case(c) as s:
        st = s.lib.fv3d_mesh_load_h5(s.h, b"mesh.h5")
        assert st == 2  # FV3D_ERR_UNSUPPORTED


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_profile_step_runs_the_step(precision):
    """fv3d_profile_step times the launches of real steps: the state it
    leaves is bitwise the one the step graphs give, and its per-launch
    times are positive."""
    c = cases.tgv_tet(4)
    with api.from_case(c, precision) as s:
        s.step_explicit("rk33", 3, cfl=0.5)
        u_graph = s.get_conserved()
    with api.from_case(c, precision) as s:
        ms = s.profile_step("rk33", 3, 0.5)
        assert np.all(ms > 0)
        assert np.array_equal(s.get_conserved(), u_graph)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mesh_from_gmsh_41_file(oracle, tmp_path, precision):
    """A walled channel written as a Gmsh MSH 4.1 file (the reference
    preprocessor's format) and read back: the GPU residual on that mesh
    against the oracle's (tests/test_gmsh.py shows the file's mesh equals
    the generator's)."""
    import os
    from fv3d_gb300 import gmsh
    nx, ny, nz = 6, 4, 4
    xs = np.linspace(0, 2, nx + 1)
    ys = mg.stretched_coords(ny, 1.0, 1.1)
    zs = np.linspace(0, 1, nz + 1)
    nodes, cn, sh = mg._structured(nx, ny, nz, xs, ys, zs, (False, False, False), 0.0, 0, (2.0, 1.0, 1.0))

    def tag(x):
        return 1 if abs(x[0]) < 1e-12 else (2 if abs(x[0] - 2.0) < 1e-12 else 3)

    count, first = {}, {}
    for c in range(cn.shape[0]):
        for lf in mg.HEX_FACES:
            key = tuple(sorted(cn[c, lf]))
            count[key] = count.get(key, 0) + 1
            first.setdefault(key, cn[c, lf])
    bnd = [(tag(nodes[list(k)].mean(axis=0)), list(first[k])) for k, n in count.items() if n == 1]
    p = os.path.join(tmp_path, "channel41.msh")
    gmsh.write_msh(p, nodes, cn, "hex", bnd, {(2, 1): "inflow", (2, 2): "outlet", (2, 3): "wall", (3, 4): "fluid"},
                   version="4.1")
    mesh = gmsh.read_msh(p)
    assert mesh.region_names == ["flow", "inflow", "outlet", "wall"]
    c = cases.channel(nx, ny, nz)          # physics, region conditions and state (walls also at z here)
    c.params["mu_mix"] = 0.01
    u = perturbed(c)
    oracle.init(mesh, c.params, c.region_type, c.region_prim)
    oracle.set_conserved(u)
    r_ref = oracle.time_derivative(0.0)
    with api.Solver(mesh, c.params, c.region_type, c.region_prim, precision) as s:
        s.set_state(u)
        err = rel_max(s.time_derivative(0.0), r_ref)
    assert err < (FP64_RESIDUAL_TOL if precision == "fp64" else MIXED_RESIDUAL_TOL), err
