"""Test infrastructure: CPU definition (NumPy, FP64) of a preconditioner that
couples cells for the pseudo-transient Newton-Krylov solve, and the solve
itself, so that a GPU version can be checked against it.  Nothing here is
on the product path.

The system each Newton step solves is (I/dt_c - dR/dU) dU = R(U), R the
finite-volume time derivative (finite_volume.c:81-124), dt_c the local
pseudo time step.  The preconditioner approximates dR/dU by the Jacobian of
a first-order, inviscid Rusanov residual (riemann_rusanonv, flux.c:320-336):
per face F = 1/2 (F(U_0) + F(U_1)) - 1/2 lam (U_1 - U_0) with
lam = max(|u.n| + c) over both sides, differentiated with lam frozen:

    dF/dU_0 = 1/2 (A(U_0) + lam I),   dF/dU_1 = 1/2 (A(U_1) - lam I)

(A the Jacobian of the normal Euler flux), plus, at a boundary face, the
ghost state's dependence on its interior cell (update_boundaries,
boundary.c:188-320): dF/dU_0 += 1/2 (A(U_g) - lam I) dU_g/dU_0, the latter
by finite differences of the oracle's ghost states.  lam also carries a
viscous term 2 mu / (rho d) (the usual spectral-radius form).  The
residual's own flux scheme (AUSM on the channel) is not used for the
preconditioner: its Jacobian is far from diagonally dominant at large CFL
and sweeps on it diverge.

Applied as k block-Jacobi sweeps z <- D^-1 (v - O z) (D the 5x5 diagonal
blocks, O the face couplings) or as symmetric block Gauss-Seidel sweeps in
cell order.

The Jacobian of the residual's own first-order flux (AUSM) approximates
the system far better (its exact solve needs a fraction of the Krylov
iterations), but sweeps on it diverge; "nested" solves it by a short inner
GMRES right-preconditioned by Rusanov sweeps.  Its blocks come from
finite differences of the oracle's first-order inviscid residual over a
distance-2 colouring of the cells (five perturbed residuals per colour).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl


def euler_flux_jacobian(U, n, kappa):
    """(N, 5, 5) Jacobians d(F.n)/dU of the Euler flux in conserved
    variables, with |u.n| + c of each state."""
    rho = U[:, 0]
    u = U[:, 1:4] / rho[:, None]
    q2 = (u * u).sum(1)
    p = (kappa - 1.0) * (U[:, 4] - 0.5 * rho * q2)
    H = (U[:, 4] + p) / rho
    un = (u * n).sum(1)
    phi = 0.5 * (kappa - 1.0) * q2
    A = np.zeros((U.shape[0], 5, 5))
    A[:, 0, 1:4] = n
    for i in range(3):
        A[:, 1 + i, 0] = phi * n[:, i] - u[:, i] * un
        for j in range(3):
            A[:, 1 + i, 1 + j] = u[:, i] * n[:, j] - (kappa - 1.0) * u[:, j] * n[:, i] + (i == j) * un
        A[:, 1 + i, 4] = (kappa - 1.0) * n[:, i]
    A[:, 4, 0] = un * (phi - H)
    A[:, 4, 1:4] = H[:, None] * n - (kappa - 1.0) * u * un[:, None]
    A[:, 4, 4] = kappa * un
    return A, np.abs(un) + np.sqrt(kappa * p / rho), rho


def ghost_derivative(oracle, mesh, U):
    """Ghost conserved states (n_boundaries, 5) and d(ghost)/d(interior cell
    state) (n_boundaries, 5, 5) from an initialised oracle: each ghost
    depends on its own cell only, so five perturbations of all cells at once
    give every block."""
    nc = U.shape[0]
    bcell = mesh.face_cells[mesh.boundary_face, 0]
    oracle.set_conserved(U)
    g0 = oracle.total()[nc:, :5].copy()
    G = np.zeros((g0.shape[0], 5, 5))
    for v in range(5):
        h = 1e-7 * np.maximum(np.abs(U[:, v]), 1e-3)
        Up = U.copy()
        Up[:, v] += h
        oracle.set_conserved(Up)
        G[:, :, v] = (oracle.total()[nc:, :5] - g0) / h[bcell][:, None]
    oracle.set_conserved(U)
    return g0, G


def coupling_matrix(mesh, U, kappa, mu, dt, ghosts):
    """Sparse (5 nc, 5 nc) P = I/dt - J_Rusanov described above."""
    nc = U.shape[0]
    fc, n, area, vol = mesh.face_cells, mesh.face_n, mesh.face_area, mesh.cell_volume
    c0, c1 = fc[:, 0], fc[:, 1]
    inner = c1 >= 0
    A0, l0, r0 = euler_flux_jacobian(U[c0], n, kappa)
    A1 = np.zeros_like(A0)
    lam = l0.copy()
    d = 2.0 * np.linalg.norm(mesh.face_x - mesh.cell_x[c0], axis=1)
    rho_f = r0.copy()
    ii = np.nonzero(inner)[0]
    A1[ii], l1, r1 = euler_flux_jacobian(U[c1[ii]], n[ii], kappa)
    lam[ii] = np.maximum(l0[ii], l1)
    d[ii] = (np.linalg.norm(mesh.face_x[ii] - mesh.cell_x[c0[ii]], axis=1)
             + np.linalg.norm(mesh.face_dist_cell_2[ii], axis=1))
    rho_f[ii] = 0.5 * (r0[ii] + r1)
    bf = np.nonzero(~inner)[0]
    g0, G = ghosts
    bidx = mesh.face_boundary[bf]
    Ag, lg, _ = euler_flux_jacobian(g0[bidx], n[bf], kappa)
    lam[bf] = np.maximum(l0[bf], lg)
    lam = lam + 2.0 * mu / (rho_f * d)
    I = np.eye(5)
    dF0 = 0.5 * (A0 + lam[:, None, None] * I)
    dF1 = 0.5 * (A1 - lam[:, None, None] * I)
    dF0[bf] += 0.5 * np.einsum("fij,fjk->fik", Ag - lam[bf, None, None] * I, G[bidx])
    # dR_a/dU = -(A_f / V_a) dF/dU for the cell the normal leaves, + for the other
    w0 = (area / vol[c0])[:, None, None]
    w1 = (area[ii] / vol[c1[ii]])[:, None, None]
    blocks = [w0 * dF0, w0[ii] * dF1[ii], -w1 * dF1[ii], -w1 * dF0[ii]]   # blocks of -J
    rows = [c0, c0[ii], c1[ii], c1[ii]]
    cols = [c0, c1[ii], c1[ii], c0[ii]]
    B = np.concatenate(blocks)
    R = np.concatenate(rows)
    Cc = np.concatenate(cols)
    rr = np.broadcast_to((5 * R)[:, None, None] + np.arange(5)[None, :, None], B.shape)
    cc = np.broadcast_to((5 * Cc)[:, None, None] + np.arange(5)[None, None, :], B.shape)
    P = sp.csr_matrix((B.ravel(), (rr.ravel(), cc.ravel())), shape=(5 * nc, 5 * nc))
    return (P + sp.diags(np.repeat(1.0 / dt, 5))).tocsr()


def distance2_colouring(mesh):
    """Greedy colouring in which no two cells of a colour are neighbours or
    share a neighbour (so a perturbation of all cells of one colour changes
    each residual through one cell only); with the neighbour lists."""
    nc = mesh.n_cells
    nbrs = [[] for _ in range(nc)]
    for a, b in mesh.face_cells:
        if b >= 0:
            nbrs[a].append(int(b))
            nbrs[b].append(int(a))
    colour = np.full(nc, -1)
    for i in range(nc):
        used = {colour[j] for j in nbrs[i]}
        for j in nbrs[i]:
            used.update(colour[k] for k in nbrs[j])
        col = 0
        while col in used:
            col += 1
        colour[i] = col
    return colour, nbrs


def first_order_jacobian_fd(oracle, case, U, flux_scheme, colouring):
    """Sparse d R_1 / dU of the first-order inviscid residual with the given
    flux, by coloured finite differences; leaves the oracle set up for the
    case's own configuration again."""
    colour, nbrs = colouring
    p1 = dict(case.params)
    p1.update(reconstruction=0, flux_scheme=flux_scheme, mu_mix=0.0)   # 0: First-Order (reconstruction.c:44-55 order)
    oracle.init(case.mesh, p1, case.region_type, case.region_prim)
    oracle.set_conserved(U)
    r0 = oracle.time_derivative(0.0)
    rows, cols, vals = [], [], []
    for col in range(colour.max() + 1):
        cells = np.nonzero(colour == col)[0]
        for v in range(5):
            h = 1e-7 * np.maximum(np.abs(U[cells, v]), 1e-3)
            Up = U.copy()
            Up[cells, v] += h
            oracle.set_conserved(Up)
            d = oracle.time_derivative(0.0) - r0
            for ci, hi in zip(cells, h):
                for rc in [ci] + nbrs[ci]:
                    rows.append(5 * rc + np.arange(5))
                    cols.append(np.full(5, 5 * ci + v))
                    vals.append(d[rc] / hi)
    oracle.init(case.mesh, case.params, case.region_type, case.region_prim)
    oracle.set_conserved(U)
    n = 5 * U.shape[0]
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def make_preconditioner(P, kind, sweeps):
    """z = M^-1 v for 'none', 'jacobi' (k sweeps), 'sgs' (k symmetric
    sweeps in cell order) or 'lu' (exact, a bound)."""
    if kind == "none":
        return lambda v: v
    if kind == "lu":
        f = spl.splu(P.tocsc())
        return lambda v: f.solve(v.ravel()).reshape(v.shape)
    Pc = P.tocoo()
    bi, bj = Pc.row // 5, Pc.col // 5

    def part(sel):
        return sp.csr_matrix((Pc.data[sel], (Pc.row[sel], Pc.col[sel])), shape=P.shape)

    D, L, U = part(bi == bj), part(bi > bj), part(bi < bj)
    Dinv = spl.splu(D.tocsc())
    if kind == "jacobi":
        O = (L + U).tocsr()

        def apply(v):
            b = v.ravel()
            z = Dinv.solve(b)
            for _ in range(sweeps - 1):
                z = Dinv.solve(b - O @ z)
            return z.reshape(v.shape)
        return apply
    if kind == "sgs":
        DL, DU = spl.splu((D + L).tocsc()), spl.splu((D + U).tocsc())

        def apply(v):
            b = v.ravel()
            z = np.zeros_like(b)
            for _ in range(sweeps):
                z = DL.solve(b - U @ z)
                z = DU.solve(b - L @ z)
            return z.reshape(v.shape)
        return apply
    raise ValueError(kind)


def solve_steady(case, kind="jacobi", sweeps=4, tol=1e-8, max_newton=150, m=30, eta=1e-2,
                 cfl0=100.0, cfl_max=1e4):
    """Pseudo-transient Newton-Krylov to |R| / |R_0| <= tol with the
    switched-evolution-relaxation CFL ramp, FGMRES(m) to a relative eta and
    finite-difference Jacobian-vector products; returns (Newton steps,
    final relative residual, Krylov iterations)."""
    from . import oracle as orc
    o = orc.Oracle("restated")
    o.init(case.mesh, case.params, case.region_type, case.region_prim)
    kappa, mu = case.params["kappa"], case.params["mu_mix"]
    vol, dx = case.mesh.cell_volume, case.mesh.cell_dx
    U = case.u0.copy()

    def resid(u):
        o.set_conserved(u)
        return o.time_derivative(0.0)

    def local_dt(u, cfl):
        rho = u[:, 0]
        vel = u[:, 1:4] / rho[:, None]
        p = (kappa - 1.0) * (u[:, 4] - 0.5 * (u[:, 1:4] * vel).sum(1))
        c = np.sqrt(kappa * p / rho)
        return cfl * vol / ((np.abs(vel) + c[:, None]) * dx).sum(1)

    colouring = distance2_colouring(case.mesh) if kind == "nested" else None
    r = resid(U)
    res0 = np.linalg.norm(r)
    res = res0
    krylov = 0
    steps = 0
    while steps < max_newton and res / res0 > tol:
        cfl = cfl0 if steps == 0 else min(cfl_max, max(cfl0, cfl0 * res0 / res))
        dt = local_dt(U, cfl)
        unorm = np.linalg.norm(U)
        rU = r

        def matvec(z):
            eps = 1e-7 * (1.0 + unorm) / np.linalg.norm(z)
            return z / dt[:, None] - (resid(U + eps * z) - rU) / eps

        if kind == "none":
            M = make_preconditioner(None, "none", 0)
        elif kind == "nested":
            # inner GMRES(sweeps) on I/dt - dR_1/dU (first-order AUSM), right-
            # preconditioned by 2 Jacobi sweeps of the Rusanov matrix
            Pa = (sp.diags(np.repeat(1.0 / dt, 5))
                  - first_order_jacobian_fd(o, case, U, case.params["flux_scheme"], colouring)).tocsr()
            Mr = make_preconditioner(coupling_matrix(case.mesh, U, kappa, mu, dt, ghost_derivative(o, case.mesh, U)),
                                     "jacobi", 2)

            def M(v, Pa=Pa, Mr=Mr):
                return fgmres(lambda z: (Pa @ z.ravel()).reshape(z.shape), Mr, v, sweeps, 0.0)[0]
        else:
            P = coupling_matrix(case.mesh, U, kappa, mu, dt, ghost_derivative(o, case.mesh, U))
            M = make_preconditioner(P, kind, sweeps)
        dU, its = fgmres(matvec, M, r, m, eta)
        krylov += its
        U = U + dU
        r = resid(U)
        res = np.linalg.norm(r)
        steps += 1
    return steps, res / res0, krylov


def fgmres(matvec, M, b, m, eta):
    """One cycle of flexible GMRES(m) from x0 = 0 (modified Gram-Schmidt,
    twice; Givens rotations): returns (x, iterations)."""
    beta = np.linalg.norm(b)
    V = [b / beta]
    Z = []
    H = np.zeros((m + 1, m))
    g = np.zeros(m + 1)
    g[0] = beta
    cs, sn = np.zeros(m), np.zeros(m)
    k = m
    for j in range(m):
        z = M(V[j])
        Z.append(z)
        w = matvec(z)
        for _ in range(2):
            for i in range(j + 1):
                h = np.vdot(w, V[i])
                H[i, j] += h
                w = w - h * V[i]
        H[j + 1, j] = np.linalg.norm(w)
        V.append(w / H[j + 1, j])
        for i in range(j):
            a, c = H[i, j], H[i + 1, j]
            H[i, j], H[i + 1, j] = cs[i] * a + sn[i] * c, -sn[i] * a + cs[i] * c
        rr = np.hypot(H[j, j], H[j + 1, j])
        cs[j], sn[j] = H[j, j] / rr, H[j + 1, j] / rr
        H[j, j], H[j + 1, j] = rr, 0.0
        g[j + 1], g[j] = -sn[j] * g[j], cs[j] * g[j]
        if abs(g[j + 1]) <= eta * beta:
            k = j + 1
            break
    y = np.linalg.solve(np.triu(H[:k, :k]), g[:k])
    return sum(y[i] * Z[i] for i in range(k)), k
