"""Every discretisation choice on both cell types, against the CPU oracle.

The parity suites pin the configurations the benchmarks run (Rusanov,
Green-Gauss and Barth-Jespersen on tetrahedra; AUSM, least squares and
Barth-Jespersen on hexahedra) and the boundary types; this matrix runs the
rest of the product: tetrahedra and hexahedra, Green-Gauss and least-squares
gradients, Rusanov and AUSM fluxes, with and without the limiter, viscous
and inviscid, plus first-order reconstruction with viscous fluxes (gradients
for the stresses only).  Each case takes 10 RK3 steps at CFL 0.5 from a
perturbed Taylor-Green state on the FP64 path (<= 1e-10 relative L2 per
variable) and the mixed path (<= 1e-5) against the oracle's FP64 solution:
the mixed path takes a different kernel for each of these combinations (4
face slots: the persistent staged gradient pass for Green-Gauss, the
one-tile-per-CTA one for least squares; 6 slots: the one-tile-per-CTA pass
on 64-cell tiles; first order: the unstaged pass).
"""
import itertools

import numpy as np
import pytest

from fv3d_gb300 import api, cases
from oracle import oracle as orc
from parity import rel_l2

pytestmark = pytest.mark.gpu

FP64_STATE_TOL = 1e-10
MIXED_STATE_TOL = 1e-5


@pytest.fixture(scope="module")
def oracle():
    return orc.Oracle("restated")


def perturbed(c, amp=0.01, seed=11):
    rng = np.random.default_rng(seed)
    u = c.u0.copy()
    u[:, 0] *= 1.0 + amp * rng.uniform(-1, 1, u.shape[0])
    u[:, 1:4] += amp * rng.uniform(-1, 1, (u.shape[0], 3)) * u[:, :1]
    u[:, 4] *= 1.0 + amp * rng.uniform(-1, 1, u.shape[0])
    return u


def make(cell, gradient, flux, limiter, viscous, recon=cases.LINEAR):
    c = cases.tgv_tet(5) if cell == "tet" else cases.tgv_hex(6)
    c.params.update(gradient=gradient, flux_scheme=flux, limiter=limiter, reconstruction=recon,
                    mu_mix=(1.0 / 400.0) if viscous else 0.0)
    c.u0 = perturbed(c)
    return c


def run_oracle(o, c, steps):
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0)
    t = 0.0
    for k in range(steps):
        dt = o.timestep_convective(0.5)
        o.step_lserkw2(1, k, t, dt)
        t += dt
    return o.conserved(), t


def check(o, c, steps=10):
    u_ref, t_ref = run_oracle(o, c, steps)
    errs = {}
    for precision, tol in (("fp64", FP64_STATE_TOL), ("mixed", MIXED_STATE_TOL)):
        with api.from_case(c, precision) as s:
            st = s.step_explicit("rk33", steps, cfl=0.5)
            err = rel_l2(s.get_conserved(), u_ref, u_ref=0.3)
        assert abs(st["t"] / t_ref - 1) < (1e-12 if precision == "fp64" else 1e-5), precision
        errs[precision] = err.max()
        assert err.max() < tol, (precision, err)
    return errs


GRADIENTS = {"gg": cases.GREEN_GAUSS, "lsq": cases.LEAST_SQUARES}
FLUXES = {"rusanov": cases.RUSANOV, "ausm": cases.AUSM}
LIMITERS = {"bj": cases.BARTH_JESPERSEN, "nolim": cases.NO_LIMITER}
MATRIX = list(itertools.product(["tet", "hex"], GRADIENTS, FLUXES, LIMITERS, ["viscous", "inviscid"]))


@pytest.mark.parametrize("cell,gradient,flux,limiter,visc", MATRIX,
                         ids=["-".join(m) for m in MATRIX])
def test_second_order_matrix(oracle, cell, gradient, flux, limiter, visc):
    c = make(cell, GRADIENTS[gradient], FLUXES[flux], LIMITERS[limiter], visc == "viscous")
    print(cell, gradient, flux, limiter, visc, check(oracle, c))


@pytest.mark.parametrize("cell", ["tet", "hex"])
@pytest.mark.parametrize("gradient", list(GRADIENTS))
def test_first_order_viscous(oracle, cell, gradient):
    """First-order reconstruction with viscous fluxes: the gradients feed
    the stresses only."""
    c = make(cell, GRADIENTS[gradient], cases.AUSM, cases.NO_LIMITER, True, recon=cases.FIRST_ORDER)
    print(cell, gradient, "first order viscous", check(oracle, c))
