"""Error measures shared by the parity tests."""
import numpy as np


def rel_l2(a, b, u_ref=1.0):
    """Relative L2 error per conserved variable of `a` against reference `b`
    (both (n, 5)).  Variables whose reference is ~0 (e.g. rho_v in a stream
    along x) are normalised by ||rho|| * u_ref instead."""
    a = np.asarray(a)[:, :5]
    b = np.asarray(b)[:, :5]
    nb = np.linalg.norm(b, axis=0)
    floor = nb[0] * u_ref
    return np.linalg.norm(a - b, axis=0) / np.maximum(nb, floor)


def rel_max(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))
