"""The benchmark workloads: meshes, physics parameters and initial states.

Each case is a synthetic stand-in with the shapes, sizes and value
distributions of the named configurations (no public dataset is involved):

  euler16   FP64 first-order Euler, periodic unit cube 16^3 hexes, Rusanov,
            Gaussian density pulse (amplitude 0.1, sigma 0.1) in a uniform
            stream u=(0.5,0,0), p=1/gamma; SSP-RK3, CFL 0.5, 100 steps
  tgv_hex   second-order Navier-Stokes, [0,2pi]^3 with 64^3 hexes whose nodes
            are jittered by +-10 % of the spacing, AUSM, least-squares
            gradients + Barth-Jespersen, Re=1600, Pr=0.71, Taylor-Green
            vortex at Mach 0.1; RK3, CFL 0.5, 200 steps
  tgv_tet   each hex of a periodic 64^3 box split into 6 tets (1,572,864
            cells), Rusanov, Green-Gauss + Barth-Jespersen, Re=1600, TGV at
            Mach 0.8; RK3, 500 steps
  channel   implicit channel 96x48x48 stretched hexes (ratio 1.1), no-slip
            walls y=0,1, inflow rho=1 u=0.3 p=1/gamma, pressure outlet,
            periodic z, Re=1000, Pr=0.71, second-order AUSM (no limiter)

Physics parameters use the reference's names (navier_stokes.c:19-24, 55-66).
Flux / reconstruction / limiter codes follow the reference's option order
(flux.c:273, solver_type.h:212-226).
"""
from __future__ import annotations

from dataclasses import dataclass
import numpy as np

from . import meshgen as mg

AUSM, RUSANOV = 0, 1
FIRST_ORDER, LINEAR = 0, 1
BARTH_JESPERSEN, NO_LIMITER = 0, 1
GREEN_GAUSS, LEAST_SQUARES = 0, 1


@dataclass
class Case:
    name: str
    mesh: mg.Mesh
    params: dict
    region_type: np.ndarray
    region_prim: np.ndarray     # (n_regions, 5): u, v, w, p, T
    u0: np.ndarray              # (n_cells, 5) conserved initial state
    scheme: str                 # "ssprk3" | "rk33" | "implicit"
    cfl: float
    steps: int


def prim_to_cons(rho, u, v, w, p, kappa):
    """eos.c:120-127 applied to arrays."""
    ru, rv, rw = u * rho, v * rho, w * rho
    re = (1.0 / (kappa - 1.0)) * p + 0.5 * (u * ru + v * rv + w * rw)
    return np.stack([rho, ru, rv, rw, re], axis=1)


def taylor_green(x, mach, kappa=1.4):
    """TGV with rho0 = V0 = L = 1, R = 1: p0 = 1/(kappa M^2), T0 = p0."""
    X, Y, Z = x[:, 0], x[:, 1], x[:, 2]
    p0 = 1.0 / (kappa * mach * mach)
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(X)
    p = p0 + (1.0 / 16.0) * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0)
    rho = p / p0
    return prim_to_cons(rho, u, v, w, p, kappa), p0


def euler16(n=16) -> Case:
    kappa = 1.4
    mesh = mg.periodic_hex_box(n, 1.0, name=f"euler_hex{n}")
    x = mesh.cell_x
    r2 = ((x - 0.5) ** 2).sum(axis=1)
    rho = 1.0 + 0.1 * np.exp(-r2 / (2 * 0.1 ** 2))
    ones = np.ones_like(rho)
    u0 = prim_to_cons(rho, 0.5 * ones, 0 * ones, 0 * ones, ones / kappa, kappa)
    params = dict(kappa=kappa, R_mix=1.0, mu_mix=0.0, Pr=0.71, cfl_scale=0.5,
                  dfl_scale=1.0, flux_scheme=RUSANOV, reconstruction=FIRST_ORDER,
                  limiter=BARTH_JESPERSEN, gradient=GREEN_GAUSS)
    prim = np.array([[0.5, 0.0, 0.0, 1 / kappa, 1 / kappa]])
    return Case("euler16", mesh, params, np.array([mg.BC_FLOW]), prim, u0, "ssprk3", 0.5, 100)


def tgv_hex(n=64, seed=20240601) -> Case:
    kappa, mach = 1.4, 0.1
    mesh = mg.periodic_hex_box(n, 2 * np.pi, jitter=0.1, seed=seed, name=f"tgv_hex{n}")
    u0, p0 = taylor_green(mesh.cell_x, mach, kappa)
    params = dict(kappa=kappa, R_mix=1.0, mu_mix=1.0 / 1600.0, Pr=0.71, cfl_scale=0.5,
                  dfl_scale=1.0, flux_scheme=AUSM, reconstruction=LINEAR,
                  limiter=BARTH_JESPERSEN, gradient=LEAST_SQUARES)
    prim = np.array([[0.0, 0.0, 0.0, p0, p0]])
    return Case("tgv_hex", mesh, params, np.array([mg.BC_FLOW]), prim, u0, "rk33", 0.5, 200)


def tgv_tet(n=64) -> Case:
    kappa, mach = 1.4, 0.8
    mesh = mg.periodic_tet_box(n, 2 * np.pi, name=f"tgv_tet{n}")
    u0, p0 = taylor_green(mesh.cell_x, mach, kappa)
    params = dict(kappa=kappa, R_mix=1.0, mu_mix=1.0 / 1600.0, Pr=0.71, cfl_scale=0.5,
                  dfl_scale=1.0, flux_scheme=RUSANOV, reconstruction=LINEAR,
                  limiter=BARTH_JESPERSEN, gradient=GREEN_GAUSS)
    prim = np.array([[0.0, 0.0, 0.0, p0, p0]])
    return Case("tgv_tet", mesh, params, np.array([mg.BC_FLOW]), prim, u0, "rk33", 0.5, 500)


def tgv_mixed(n=16, gradient=GREEN_GAUSS, jitter=0.1, seed=20240601) -> Case:
    """Taylor-Green vortex on the mixed hexahedron / prism / pyramid box
    (cells of 5 and 6 faces, faces of 3 and 4 nodes): AUSM, Barth-Jespersen,
    viscous."""
    kappa, mach = 1.4, 0.3
    mesh = mg.mixed_box(n, 2 * np.pi, jitter=jitter, seed=seed, name=f"tgv_mixed{n}")
    u0, p0 = taylor_green(mesh.cell_x, mach, kappa)
    params = dict(kappa=kappa, R_mix=1.0, mu_mix=1.0 / 1600.0, Pr=0.71, cfl_scale=0.5,
                  dfl_scale=1.0, flux_scheme=AUSM, reconstruction=LINEAR,
                  limiter=BARTH_JESPERSEN, gradient=gradient)
    prim = np.array([[0.0, 0.0, 0.0, p0, p0]])
    return Case("tgv_mixed", mesh, params, np.array([mg.BC_FLOW]), prim, u0, "rk33", 0.5, 50)


def channel(nx=96, ny=48, nz=48, ratio=1.1, tets=False) -> Case:
    kappa = 1.4
    mesh = mg.channel(nx, ny, nz, 2.0, 1.0, 1.0, ratio, tets=tets)
    p_in = 1.0 / kappa
    T_in = p_in / 1.0          # rho = 1, R = 1
    # second-order AUSM without a limiter: the configuration names none and
    # the flow is smooth and subsonic; with Barth-Jespersen the steady
    # residual stalls near 1e-7 (its min(1, y) is not differentiable)
    params = dict(kappa=kappa, R_mix=1.0, mu_mix=0.3 / 1000.0, Pr=0.71, cfl_scale=1.0,
                  dfl_scale=1.0, flux_scheme=AUSM, reconstruction=LINEAR,
                  limiter=NO_LIMITER, gradient=GREEN_GAUSS)
    rt = np.array([mg.BC_FLOW, mg.BC_INFLOW, mg.BC_PRESSURE_OUTLET, mg.BC_WALL_ADIABATIC])
    prim = np.array([[0.3, 0.0, 0.0, p_in, T_in],
                     [0.3, 0.0, 0.0, p_in, T_in],
                     [0.0, 0.0, 0.0, p_in, T_in],
                     [0.0, 0.0, 0.0, p_in, T_in]])
    ones = np.ones(mesh.n_cells)
    u0 = prim_to_cons(ones, 0.3 * ones, 0 * ones, 0 * ones, p_in * ones, kappa)
    return Case("channel", mesh, params, rt, prim, u0, "implicit", 100.0, 0)


def make(name: str, **kw) -> Case:
    return {"euler16": euler16, "tgv_hex": tgv_hex, "tgv_tet": tgv_tet, "tgv_mixed": tgv_mixed,
            "channel": channel}[name](**kw)
