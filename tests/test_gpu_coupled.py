"""The cell-coupling preconditioner of the implicit solve (FV3D_PC_COUPLED)
against its CPU definition in oracle/coupling.py, through the C ABI.

  * the operators the GPU applies (P_A = I/dt - dR1/dU of the first-order
    inviscid residual with the case's flux, matrix-free by the exact FP32
    derivative of each face flux; P_R the first-order Rusanov Jacobian,
    analytic, wave speed frozen, its slot blocks matrix-free), written out as
    blocks by their own arithmetic, equal the CPU's (coloured finite
    differences of the oracle's residual; the analytic Rusanov assembly) to
    FP32 precision, on the hexahedral channel (6 face slots, AUSM), the
    Kuhn-split tetrahedral channel (4 slots, Rusanov) and the mixed
    hexahedron / prism / pyramid box (AUSM);
  * the nested solve (inner GMRES(10) on P_A right-preconditioned by two
    Rusanov block-Jacobi sweeps, FGMRES(30) outside, FP64 Jacobian-vector
    products) takes the CPU solve's Newton and Krylov counts on the 12x8x4
    channel, and its converged state satisfies the oracle's steady equations;
    on tetrahedra too it cuts the Krylov work five-fold or more.
"""
import numpy as np
import pytest

from fv3d_gb300 import api, cases
from oracle import coupling as cp
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-8


def perturbed_channel(nx=12, ny=8, nz=4, seed=3, tets=False):
    return perturbed(cases.channel(nx, ny, nz, tets=tets), seed)


def perturbed(c, seed=3):
    rng = np.random.default_rng(seed)
    U = c.u0.copy()
    U[:, 0] *= 1 + 0.02 * rng.uniform(-1, 1, len(U))
    U[:, 1:4] += 0.02 * rng.uniform(-1, 1, (len(U), 3))
    U[:, 4] *= 1 + 0.01 * rng.uniform(-1, 1, len(U))
    c.u0 = U
    return c


def local_dt(c, U, cfl):
    kappa = c.params["kappa"]
    rho = U[:, 0]
    vel = U[:, 1:4] / rho[:, None]
    p = (kappa - 1.0) * (U[:, 4] - 0.5 * (U[:, 1:4] * vel).sum(1))
    a = np.sqrt(kappa * p / rho)
    return cfl * c.mesh.cell_volume / ((np.abs(vel) + a[:, None]) * c.mesh.cell_dx).sum(1)


def block_errors(P, diag, slots, nbr, inverse_diag=False):
    """Relative Frobenius errors of the GPU's diagonal and slot blocks
    against the sparse CPU matrix P."""
    P = P.tocsr()
    ed, eo = [], []
    for i in range(diag.shape[0]):
        ref = P[5 * i:5 * i + 5, 5 * i:5 * i + 5].toarray()
        if inverse_diag:
            ref = np.linalg.inv(ref)
        ed.append(np.linalg.norm(diag[i] - ref) / np.linalg.norm(ref))
        for k, j in enumerate(nbr[i]):
            if j < 0:
                assert np.all(slots[i, k] == 0)
                continue
            ref = P[5 * i:5 * i + 5, 5 * j:5 * j + 5].toarray()
            eo.append(np.linalg.norm(slots[i, k] - ref) / max(np.linalg.norm(ref), 1e-300))
    return np.array(ed), np.array(eo)


def test_coupled_blocks_match_the_cpu_definition():
    check_blocks(perturbed_channel())


def tet_channel_rusanov():
    c = perturbed_channel(6, 4, 4, tets=True)
    c.params["flux_scheme"] = cases.RUSANOV
    return c


# 4 face slots: the Kuhn-split channel (walls, inflow, outlet, periodic z)
# with the Rusanov flux; 5 and 6: the jittered hexahedron / prism / pyramid
# periodic box with AUSM
OTHER_CELLS = {"tet_channel_rusanov": (tet_channel_rusanov, False),
               "mixed_box_ausm": (lambda: perturbed(cases.tgv_mixed(6)), True)}


@pytest.mark.parametrize("name", list(OTHER_CELLS))
def test_coupled_blocks_on_tetrahedra_and_mixed_cells(name):
    make, cancelling = OTHER_CELLS[name]
    check_blocks(make(), cancelling)


def check_blocks(c, cancelling=False):
    U = c.u0
    with api.from_case(c, "fp64") as s:
        s.solve_implicit(preconditioner="coupled", jv_precision="fp64", max_newton=1, check=False)
        da, oa, nba = s.coupled_blocks("ausm")
        dr, orr, nbr = s.coupled_blocks("rusanov")
    assert np.array_equal(nba, nbr)
    # every face of every cell appears once among its slots
    fc = c.mesh.face_cells
    inner = fc[:, 1] >= 0
    pairs = set(map(tuple, fc[inner])) | set(map(tuple, fc[inner][:, ::-1]))
    got = {(i, int(j)) for i in range(c.mesh.n_cells) for j in nba[i] if j >= 0}
    assert got == pairs
    dt = local_dt(c, U, 100.0)
    o = orc.Oracle("restated")
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    colouring = cp.distance2_colouring(c.mesh)
    import scipy.sparse as sp
    PA = sp.diags(np.repeat(1.0 / dt, 5)) - cp.first_order_jacobian_fd(o, c, U, c.params["flux_scheme"], colouring)
    ed, eo = block_errors(PA, da, oa, nba)
    print("P_A blocks: diag median %.2e max %.2e, slots median %.2e max %.2e"
          % (np.median(ed), ed.max(), np.median(eo), eo.max()))
    # FP32 forward-mode derivatives against FP64 forward differences: measured
    # median 3e-7, largest 4e-6 (a block of small entries).  A diagonal block
    # is a sum over the cell's faces that nearly cancels where the state is
    # nearly uniform around a closed cell (1/dt is small at CFL 100), so its
    # FP32 rounding is relative to the face terms: with cancelling, the
    # error is measured against the summed norms of the cell's slot blocks
    # (the size of those terms) where that is larger than the block itself
    if cancelling:
        flux_part = np.linalg.norm(da - np.eye(5)[None] / dt[:, None, None], axis=(1, 2))
        terms = np.linalg.norm(oa, axis=(2, 3)).sum(1)
        ratio = np.maximum(1.0, terms / flux_part)
        print("P_A diagonal: face terms / block median %.1f max %.1f" % (np.median(ratio), ratio.max()))
        ed = ed / ratio
    assert np.median(ed) < 1e-6 and ed.max() < 2e-5, (np.median(ed), ed.max())
    assert np.median(eo) < 1e-6 and eo.max() < 2e-5, (np.median(eo), eo.max())
    PR = cp.coupling_matrix(c.mesh, U, c.params["kappa"], c.params["mu_mix"], dt, cp.ghost_derivative(o, c.mesh, U))
    ed, eo = block_errors(PR, dr, orr, nbr, inverse_diag=True)
    print("P_R blocks: inverse diag median %.2e max %.2e, slots median %.2e max %.2e"
          % (np.median(ed), ed.max(), np.median(eo), eo.max()))
    assert np.median(ed) < 1e-6 and ed.max() < 1e-4
    assert np.median(eo) < 1e-6 and eo.max() < 1e-4


def oracle_residual_norm(c, u):
    o = orc.Oracle("restated")
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(u)
    return np.linalg.norm(o.time_derivative(0.0))


def test_nested_solve_takes_the_cpu_counts_and_reaches_the_oracle_tolerance():
    """12x8x4 channel, AUSM second order, viscous, from the inflow state:
    FGMRES(30) to eta = 0.01, no restarts, FP64 Jacobian-vector products;
    inner GMRES(10), two undamped sweeps, rebuilt every Newton step (the CPU
    definition's; the inner GMRES is flexible here, which in exact
    arithmetic is the same solve).
    CPU (oracle/coupling.py): 6 Newton steps, 88 Krylov iterations;
    unpreconditioned 42 / 1,260."""
    c = cases.channel(12, 8, 4)
    steps_cpu, rel_cpu, krylov_cpu = cp.solve_steady(c, "nested", 10)
    with api.from_case(c, "fp64") as s:
        st = s.solve_implicit(preconditioner="coupled", jv_precision="fp64", tol_rel=TOL, eta=1e-2,
                              max_restarts=0, inner_dim=10, inner_sweeps=2, inner_omega=1.0, pc_refresh=1)
        u = s.get_conserved()
    print("GPU", st["newton_steps"], st["gmres_iterations"], "CPU", steps_cpu, krylov_cpu)
    assert st["converged"] == 1
    assert abs(st["newton_steps"] - steps_cpu) <= 1
    assert abs(st["gmres_iterations"] - krylov_cpu) <= max(3, 0.05 * krylov_cpu)
    r0 = oracle_residual_norm(c, c.u0)
    assert oracle_residual_norm(c, u) / r0 <= 10 * TOL


@pytest.mark.parametrize("jv", ["fp32", "fp64", "fp32_fp64_arnoldi"])
def test_coupled_cuts_the_krylov_work(jv):
    """Against the solve without a preconditioner and with block Jacobi:
    far fewer Krylov iterations to the same tolerance, and the answers agree
    (Jacobian-vector products from FP32 or FP64 residuals; with FP32 ones
    the Arnoldi basis in FP32 or in FP64)."""
    c = cases.channel(12, 8, 4)
    out = {}
    for pc in ("none", "coupled"):
        with api.from_case(c, "fp64") as s:
            st = s.solve_implicit(preconditioner=pc, jv_precision=jv, tol_rel=TOL,
                                  max_restarts=3 if pc == "none" else 0)
            out[pc] = (st, s.get_conserved())
    print(jv, {k: (v[0]["newton_steps"], v[0]["gmres_iterations"], v[0]["wall_ms"]) for k, v in out.items()})
    assert out["coupled"][0]["gmres_iterations"] * 5 < out["none"][0]["gmres_iterations"]
    a, b = out["coupled"][1], out["none"][1]
    scale = np.maximum(np.abs(a).max(axis=0), 0.3 * np.abs(a[:, 0]).max())
    assert (np.abs(a - b).max(axis=0) / scale).max() < 1e-6
    r0 = oracle_residual_norm(c, c.u0)
    assert oracle_residual_norm(c, a) / r0 <= 10 * TOL


def test_coupled_solve_on_tetrahedra():
    """The Kuhn-split 12x8x4 channel (2,304 tetrahedra, 4 face slots):
    the coupled solve reaches the tolerance with a fifth of the Krylov
    iterations of the solve without a preconditioner, at the same state."""
    c = cases.channel(12, 8, 4, tets=True)
    out = {}
    for pc in ("none", "coupled"):
        with api.from_case(c, "fp64") as s:
            st = s.solve_implicit(preconditioner=pc, tol_rel=TOL, max_restarts=3 if pc == "none" else 0)
            out[pc] = (st, s.get_conserved())
    print({k: (v[0]["newton_steps"], v[0]["gmres_iterations"], v[0]["wall_ms"]) for k, v in out.items()})
    assert out["coupled"][0]["converged"] == 1 and out["none"][0]["converged"] == 1
    assert out["coupled"][0]["gmres_iterations"] * 5 < out["none"][0]["gmres_iterations"]
    a, b = out["coupled"][1], out["none"][1]
    scale = np.maximum(np.abs(a).max(axis=0), 0.3 * np.abs(a[:, 0]).max())
    assert (np.abs(a - b).max(axis=0) / scale).max() < 1e-6
    r0 = oracle_residual_norm(c, c.u0)
    assert oracle_residual_norm(c, a) / r0 <= 10 * TOL


def test_coupled_inner_settings_and_repeat():
    """Other inner iteration and sweep counts also converge (down to one
    sweep, whose first sweep writes the direction itself, and one inner
    iteration, which forms no second basis vector); the same solve twice in
    one context (graphs replayed) gives bitwise the same state."""
    c = cases.channel(12, 8, 4)
    with api.from_case(c, "fp64") as s:
        runs = []
        for m, sw, om in ((5, 2, 0.7), (10, 2, 1.0), (10, 4, 0.7), (10, 2, 1.0), (3, 1, 0.7), (1, 3, 0.7)):
            s.set_state(c.u0)
            st = s.solve_implicit(preconditioner="coupled", tol_rel=TOL, inner_dim=m, inner_sweeps=sw,
                                  inner_omega=om)
            runs.append((st["newton_steps"], st["gmres_iterations"], s.get_conserved()))
            print(m, sw, om, st["newton_steps"], st["gmres_iterations"])
            assert st["converged"] == 1
    assert runs[1][:2] == runs[3][:2] and np.array_equal(runs[1][2], runs[3][2])
    with api.from_case(c, "fp64") as s:
        for bad in (dict(inner_dim=31), dict(inner_sweeps=9), dict(inner_omega=2.5)):
            with pytest.raises(api.FV3DError):
                s.solve_implicit(preconditioner="coupled", **bad)
