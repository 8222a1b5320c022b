"""Test infrastructure: CPU study (NumPy / SciPy, FP64) of what a per-cell
map can add to the block-Jacobi sweeps of the Rusanov matrix P_R that the
cell-coupling preconditioner uses (oracle/coupling.py builds P_R).  Nothing
here is on the product path.

The sweeps solve P_R z = b for right-hand sides that look like the inner
Krylov vectors (powers of P_R applied to random vectors, normalised).  Three
per-cell maps are fitted with full knowledge of the exact solutions, so each
is an upper bound for what a per-cell network could learn from local inputs:

  * a 5x5 matrix W_c per cell as the first sweep's map, z_0 = W_c b_c,
    least-squares fitted to (P_R^-1 b)_c;
  * a 5x5 matrix per cell as the sweep's update, z <- z + W_c r_c, fitted to
    the remaining error e_c from the residual r_c along damped sweeps;
  * a damping factor per cell, z <- z + w_c D_c^-1 r_c, fitted to minimise
    the residual after the update.

Each is compared with plain sweeps (w = 1) and with one global damping.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from . import coupling as cp
from . import oracle as orc


def rusanov_system(case, cfl=1e4):
    """P_R at the case's initial state and local time steps at `cfl`, with
    its block diagonal D and off-diagonal part O."""
    U = case.u0.copy()
    o = orc.Oracle("restated")
    o.init(case.mesh, case.params, case.region_type, case.region_prim)
    kappa, mu = case.params["kappa"], case.params["mu_mix"]
    vol, dx = case.mesh.cell_volume, case.mesh.cell_dx
    rho = U[:, 0]
    vel = U[:, 1:4] / rho[:, None]
    p = (kappa - 1.0) * (U[:, 4] - 0.5 * (U[:, 1:4] * vel).sum(1))
    a = np.sqrt(kappa * p / rho)
    dt = cfl * vol / ((np.abs(vel) + a[:, None]) * dx).sum(1)
    P = cp.coupling_matrix(case.mesh, U, kappa, mu, dt, cp.ghost_derivative(o, case.mesh, U)).tocsr()
    Pc = P.tocoo()
    bi, bj = Pc.row // 5, Pc.col // 5
    D = sp.csr_matrix((Pc.data[bi == bj], (Pc.row[bi == bj], Pc.col[bi == bj])), shape=P.shape)
    return P, D, (P - D).tocsr(), spl.inv(D.tocsc()).tocsr()


def krylov_like(P, count, seed=0):
    """Right-hand sides: random vectors with 0..5 applications of P, normalised."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        v = rng.standard_normal(P.shape[0])
        for _ in range(rng.integers(0, 6)):
            v = P @ v
            v /= np.linalg.norm(v)
        out.append(v / np.linalg.norm(v))
    return np.array(out)


def sweeps(P, Dinv, b, k, omega=1.0, z0=None, w_cell=None):
    """k damped block-Jacobi sweeps from z0 (default omega D^-1 b counted as
    the first); w_cell: a damping factor per cell instead of omega."""
    w = omega if w_cell is None else np.repeat(w_cell, 5)
    z = w * (Dinv @ b) if z0 is None else z0.copy()
    for _ in range(k - (1 if z0 is None else 0)):
        z = z + w * (Dinv @ (b - P @ z))
    return z


def study(case, k=4, n_train=30, n_test=10, seed=0):
    """Relative errors |z - P^-1 b| / |P^-1 b| after k sweeps (mean over the
    test vectors) for each map; see the module docstring."""
    P, D, O, Dinv = rusanov_system(case)
    nc, n = case.mesh.n_cells, P.shape[0]
    lu = spl.splu(P.tocsc())
    B = krylov_like(P, n_train + n_test, seed)
    X = np.array([lu.solve(b) for b in B])
    tr, te = range(n_train), range(n_train, n_train + n_test)

    def err(z, t):
        return np.linalg.norm(z - X[t]) / np.linalg.norm(X[t])

    out = {"plain": np.mean([err(sweeps(P, Dinv, B[t], k), t) for t in te]),
           "damped_0.7": np.mean([err(sweeps(P, Dinv, B[t], k, 0.7), t) for t in te])}
    # per-cell first-sweep map
    W = np.zeros((nc, 5, 5))
    for c in range(nc):
        s = slice(5 * c, 5 * c + 5)
        W[c] = np.linalg.lstsq(B[list(tr)][:, s], X[list(tr)][:, s], rcond=None)[0].T
    out["per_cell_first_map"] = np.mean([
        err(sweeps(P, Dinv, B[t], k - 1, 1.0, np.einsum("cij,cj->ci", W, B[t].reshape(nc, 5)).ravel()), t)
        for t in te])
    # per-cell update map fitted to the error along damped sweeps
    R, E = [], []
    for t in tr:
        z = np.zeros(n)
        for _ in range(k):
            r = B[t] - P @ z
            R.append(r)
            E.append(X[t] - z)
            z = z + 0.7 * (Dinv @ r)
    R, E = np.array(R), np.array(E)
    W2 = np.zeros((nc, 5, 5))
    for c in range(nc):
        s = slice(5 * c, 5 * c + 5)
        W2[c] = np.linalg.lstsq(R[:, s], E[:, s], rcond=None)[0].T

    def update_map(b):
        z = np.zeros(n)
        for _ in range(k):
            z = z + np.einsum("cij,cj->ci", W2, (b - P @ z).reshape(nc, 5)).ravel()
        return z
    out["per_cell_update_map"] = np.mean([err(update_map(B[t]), t) for t in te])
    # per-cell damping minimising the residual after one update
    rows, rhs = [], []
    cell = np.repeat(np.arange(nc), 5)
    for t in tr:
        z = np.zeros(n)
        for _ in range(k):
            r = B[t] - P @ z
            d = Dinv @ r
            rows.append(P @ sp.csr_matrix((d, (np.arange(n), cell)), shape=(n, nc)))
            rhs.append(r)
            z = z + 0.7 * d
    w = spl.lsqr(sp.vstack(rows).tocsr(), np.concatenate(rhs), damp=1e-3, atol=1e-10, btol=1e-10,
                 iter_lim=5000)[0]
    out["per_cell_damping"] = np.mean([err(sweeps(P, Dinv, B[t], k, w_cell=w), t) for t in te])
    out["per_cell_damping_range"] = (float(np.percentile(w, 5)), float(np.percentile(w, 95)))
    return out
