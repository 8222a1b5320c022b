"""CPU checks of the cell-coupling preconditioner definition in
oracle/coupling.py (test infrastructure for a GPU version): the analytic
first-order Rusanov blocks against finite differences of the oracle's
first-order residual, and what the preconditioners do to the
pseudo-transient Newton-Krylov solve of a small channel."""
import numpy as np
import pytest
import scipy.sparse as sp

from fv3d_gb300 import cases
from oracle import coupling as cp
from oracle import oracle as orc


def _blocks(M, i, j):
    return M[5 * i:5 * i + 5, 5 * j:5 * j + 5]


def test_rusanov_blocks_match_finite_differences():
    """d R_1 / dU (first order, inviscid, Rusanov) assembled analytically
    with lambda frozen and the ghosts' derivative at boundary faces agrees
    with coloured finite differences of the oracle's residual: interior
    couplings exactly where lambda is smooth, diagonal blocks to the frozen
    lambda's share."""
    c = cases.channel(12, 8, 4)
    rng = np.random.default_rng(3)
    U = c.u0.copy()
    U[:, 0] *= 1 + 0.02 * rng.uniform(-1, 1, len(U))
    U[:, 1:4] += 0.02 * rng.uniform(-1, 1, (len(U), 3))
    o = orc.Oracle("restated")
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    ghosts = cp.ghost_derivative(o, c.mesh, U)
    J_an = -cp.coupling_matrix(c.mesh, U, c.params["kappa"], 0.0, np.full(len(U), np.inf), ghosts).toarray()
    J_fd = cp.first_order_jacobian_fd(o, c, U, cases.RUSANOV, cp.distance2_colouring(c.mesh)).toarray()
    boundary = set(c.mesh.face_cells[c.mesh.face_cells[:, 1] < 0, 0].tolist())
    diag = {True: [], False: []}
    for i in range(len(U)):
        d = np.linalg.norm(_blocks(J_fd, i, i) - _blocks(J_an, i, i)) / np.linalg.norm(_blocks(J_fd, i, i))
        diag[i in boundary].append(d)
    off = [np.linalg.norm(_blocks(J_fd, a, b) - _blocks(J_an, a, b)) / np.linalg.norm(_blocks(J_fd, a, b))
           for a, b in c.mesh.face_cells if b >= 0]
    assert np.median(diag[False]) < 0.01 and max(diag[False]) < 0.03
    assert max(diag[True]) < 0.08          # ghosts frozen instead: 24-45 %
    assert np.median(off) < 1e-3 and max(off) < 0.05
    # nothing outside the face stencil
    mask = np.kron(np.eye(len(U)), np.ones((5, 5))) > 0
    for a, b in c.mesh.face_cells:
        if b >= 0:
            mask[5 * a:5 * a + 5, 5 * b:5 * b + 5] = mask[5 * b:5 * b + 5, 5 * a:5 * a + 5] = True
    assert np.abs(J_fd[~mask]).max() == 0.0


def test_coupling_preconditioners_cut_the_krylov_work():
    """On the 12x8x4 channel (AUSM, second order, viscous) to 1e-8:
    measured 42 Newton steps / 1,260 Krylov iterations without a
    preconditioner, 24 / 720 with 4 Rusanov Jacobi sweeps, 6 / 89 with the
    nested AUSM solve."""
    c = cases.channel(12, 8, 4)
    runs = {name: cp.solve_steady(c, kind, k)
            for name, (kind, k) in {"none": ("none", 0), "jacobi4": ("jacobi", 4), "nested": ("nested", 10)}.items()}
    for name, (steps, rel, krylov) in runs.items():
        assert rel <= 1e-8, (name, rel)
    assert runs["jacobi4"][2] <= 0.7 * runs["none"][2]
    assert runs["nested"][2] <= 0.15 * runs["none"][2]
    assert runs["nested"][0] <= 10


@pytest.mark.parametrize("kind", ["jacobi", "sgs"])
def test_ausm_jacobian_sweeps_do_not_converge(kind):
    """The AUSM first-order Jacobian is the better operator, but 8
    stationary sweeps on P z = r at CFL 1e4 end farther from the exact z
    than z = 0 does, while 8 sweeps on the Rusanov matrix come closer
    (why the nested solve puts the Rusanov sweeps inside)."""
    c = cases.channel(12, 8, 4)
    o = orc.Oracle("restated")
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    U = c.u0.copy()
    o.set_conserved(U)
    r = o.time_derivative(0.0)
    vol, dx, kappa = c.mesh.cell_volume, c.mesh.cell_dx, c.params["kappa"]
    rho = U[:, 0]
    vel = U[:, 1:4] / rho[:, None]
    p = (kappa - 1.0) * (U[:, 4] - 0.5 * (U[:, 1:4] * vel).sum(1))
    dt = 1e4 * vol / ((np.abs(vel) + np.sqrt(kappa * p / rho)[:, None]) * dx).sum(1)
    J = cp.first_order_jacobian_fd(o, c, U, c.params["flux_scheme"], cp.distance2_colouring(c.mesh))
    P = (sp.diags(np.repeat(1.0 / dt, 5)) - J).tocsr()
    M = cp.make_preconditioner(P, kind, 8)
    # the sweeps' error on P z = r grows instead of shrinking
    z = M(r)
    lu = cp.make_preconditioner(P, "lu", 0)(r)
    assert np.linalg.norm(z - lu) > np.linalg.norm(lu)
    Pr = cp.coupling_matrix(c.mesh, U, kappa, c.params["mu_mix"], dt, cp.ghost_derivative(o, c.mesh, U))
    zr = cp.make_preconditioner(Pr, kind, 8)(r)
    lur = cp.make_preconditioner(Pr, "lu", 0)(r)
    # Jacobi moves information one cell per sweep: 8 sweeps close 29 %
    assert np.linalg.norm(zr - lur) < {"jacobi": 0.9, "sgs": 0.5}[kind] * np.linalg.norm(lur)
