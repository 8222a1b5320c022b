// Navier-Stokes physics for the FV3D residual on sm_103a: equation of state,
// boundary ghost states, Rusanov / AUSM convective fluxes and the viscous
// flux.  Templated on the face arithmetic type R (double for the FP64 path,
// float for the mixed path).  Expressions keep the reference's operation
// order (src/FV3D/src/navier_stokes/*.c) so the FP64 path tracks the
// reference to rounding.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fv3d {

// variable order of the reference (navier_stokes.c:107-117)
enum { RHO = 0, MX = 1, MY = 2, MZ = 3, EN = 4, VU = 5, VV = 6, VW = 7, PR = 8, TT = 9 };

// region / boundary types (navier_stokes_module.h:47-59) + pressure outlet
enum {
  BC_FLOW = 0, BC_INFLOW = 1, BC_OUTFLOW = 2, BC_WALL_ADIABATIC = 3,
  BC_WALL_ISOTHERMAL = 4, BC_WALL_SLIP = 5, BC_SYMMETRY = 6, BC_STATE = 7,
  BC_FUNCTION = 8, BC_PRESSURE_OUTLET = 9
};

constexpr int MAX_REGIONS = 16;

// Physics constants, set once per context (navier_stokes.c:85-124).
struct PhysConst {
  double kappa, km1, kp1, s_km1, s_kp1, R_mix, mu, heat_lambda;
  int flux;             // 0 AUSM, 1 Rusanov
  int n_regions;
  int region_type[MAX_REGIONS];
  double region_phi[MAX_REGIONS][10];  // conserved + primitive region states
  // FP32 copies for the mixed path (kappa, km1, s_km1, s_kp1, R, mu, heat, -)
  float f32[8];
  float region_phi_f[MAX_REGIONS][10];
};

template <class R>
struct Phys {
  R kappa, km1, s_km1, s_kp1, R_mix, mu, heat_lambda;
  int flux;
  __device__ __forceinline__ void load(const PhysConst& c) {
    kappa = (R)c.kappa; km1 = (R)c.km1; s_km1 = (R)c.s_km1; s_kp1 = (R)c.s_kp1;
    R_mix = (R)c.R_mix; mu = (R)c.mu; heat_lambda = (R)c.heat_lambda; flux = c.flux;
  }
};

template <class R> __device__ __forceinline__ R rmax(R a, R b) { return (a > b) ? a : b; }
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return (a < b) ? a : b; }
template <class R> __device__ __forceinline__ R rabs(R a) { return (a < (R)0) ? -a : a; }

template <class R>
__device__ __forceinline__ R dot3(const R* a, const R* b) {
  R s = a[0] * b[0];
  s += a[1] * b[1];
  s += a[2] * b[2];
  return s;
}

// eos.c:81-92
template <class R>
__device__ __forceinline__ void cons_to_prims(R* q, const Phys<R>& ph) {
  q[VU] = q[MX] / q[RHO];
  q[VV] = q[MY] / q[RHO];
  q[VW] = q[MZ] / q[RHO];
  q[PR] = ph.km1 * (q[EN] - (R)0.5 * dot3(&q[MX], &q[VU]));
  q[PR] = rmax((R)1.00E-10, q[PR]);
  q[TT] = q[PR] / (q[RHO] * ph.R_mix);
}

// eos.c:120-127
template <class R>
__device__ __forceinline__ void prims_to_cons(R* q, const Phys<R>& ph) {
  q[MX] = q[VU] * q[RHO];
  q[MY] = q[VV] * q[RHO];
  q[MZ] = q[VW] * q[RHO];
  q[EN] = ph.s_km1 * q[PR] + (R)0.5 * dot3(&q[VU], &q[MX]);
}

// eos.c:55-75
template <class R>
__device__ __forceinline__ R wall_pressure(const R* q, const Phys<R>& ph) {
  if (q[VU] <= (R)0) {
    R c = sqrt(ph.kappa * q[PR] / q[RHO]);
    return q[PR] * pow(rmax((R)1e-4, (R)1 + (R)0.5 * ph.km1 * q[VU] / c), (R)2 * ph.kappa * ph.s_km1);
  }
  R ar = (R)2 * ph.s_kp1 / q[VU];
  R br = ph.km1 * ph.s_kp1 * q[PR];
  return q[PR] + q[VU] / ar * (R)0.5 * (q[VU] + sqrt(q[VU] * q[VU] + (R)4 * ar * (q[PR] + br)));
}

// Ghost state of a boundary face from the interior cell's full state `in`
// (boundary.c:188-320; pressure outlet is new: interior state at the region
// pressure).
template <class R>
__device__ __forceinline__ void ghost_state(const R* in, int region, const R* n, const R* t1,
                                            const R* t2, const PhysConst& pc, const Phys<R>& ph,
                                            R* g) {
#pragma unroll
  for (int j = 0; j < 10; ++j) g[j] = in[j];
  const int type = pc.region_type[region];
  switch (type) {
    case BC_INFLOW:
    case BC_STATE:
#pragma unroll
      for (int j = 0; j < 10; ++j) g[j] = (R)pc.region_phi[region][j];
      break;
    case BC_PRESSURE_OUTLET:
      g[PR] = (R)pc.region_phi[region][PR];
      g[TT] = g[PR] / (g[RHO] * ph.R_mix);
      break;
    case BC_WALL_ADIABATIC:
    case BC_WALL_ISOTHERMAL:
    case BC_WALL_SLIP:
    case BC_SYMMETRY: {
      g[VU] = dot3(&in[VU], n);
      g[VV] = dot3(&in[VU], t1);
      g[VW] = dot3(&in[VU], t2);
      g[PR] = wall_pressure(g, ph);
      if (type == BC_WALL_SLIP || type == BC_SYMMETRY) {
        g[VU] = (R)0;
        g[TT] = g[PR] / (g[RHO] * ph.R_mix);
      } else {
        g[VU] = (R)0; g[VV] = (R)0; g[VW] = (R)0;
        if (type == BC_WALL_ISOTHERMAL) g[TT] = (R)pc.region_phi[region][TT];
        g[RHO] = g[PR] / (ph.R_mix * g[TT]);
      }
      R a = g[VU] * n[0] + g[VV] * t1[0] + g[VW] * t2[0];
      R b = g[VU] * n[1] + g[VV] * t1[1] + g[VW] * t2[1];
      R c = g[VU] * n[2] + g[VV] * t1[2] + g[VW] * t2[2];
      g[VU] = a; g[VV] = b; g[VW] = c;
      break;
    }
    default:  // outflow: interior copy
      break;
  }
  prims_to_cons(g, ph);
}

// Ghost gradient (boundary.c:325-412): interior copy, normal part removed on
// slip walls / symmetry planes.  g[3] = (x, y, z) components of one variable.
template <class R>
__device__ __forceinline__ void ghost_gradient(int type, const R* n, const R* t1, const R* t2,
                                               R* gx, R* gy, R* gz) {
  if (type != BC_WALL_SLIP && type != BC_SYMMETRY) return;
  R a1 = *gx * t1[0] + *gy * t1[1] + *gz * t1[2];
  R a2 = *gx * t2[0] + *gy * t2[1] + *gz * t2[2];
  R a0 = (R)0;
  *gx = a0 * n[0] + a1 * t1[0] + a2 * t2[0];
  *gy = a0 * n[1] + a1 * t1[1] + a2 * t2[1];
  *gz = a0 * n[2] + a1 * t1[2] + a2 * t2[2];
}

// flux.c:56-73: rotate momentum into (n, t1, t2) and recover primitives
template <class R>
__device__ __forceinline__ void rotate_in(const R* q, const R* n, const R* t1, const R* t2,
                                          const Phys<R>& ph, R* o) {
  o[RHO] = q[RHO];
  o[MX] = dot3(&q[MX], n);
  o[MY] = dot3(&q[MX], t1);
  o[MZ] = dot3(&q[MX], t2);
  o[EN] = q[EN];
  cons_to_prims(o, ph);
}

// flux.c:203-210 + 320-336
template <class R>
__device__ __forceinline__ void flux_rusanov(const R* l, const R* r, const Phys<R>& ph, R* f) {
  R cl = sqrt(ph.kappa * l[PR] / l[RHO]);
  R cr = sqrt(ph.kappa * r[PR] / r[RHO]);
  R lam = rmax(rabs(l[VU]) + cl, rabs(r[VU]) + cr);
  R fl[5], fr[5];
  fl[0] = l[MX]; fl[1] = l[MX] * l[VU] + l[PR]; fl[2] = l[MX] * l[VV]; fl[3] = l[MX] * l[VW];
  fl[4] = (l[EN] + l[PR]) * l[VU];
  fr[0] = r[MX]; fr[1] = r[MX] * r[VU] + r[PR]; fr[2] = r[MX] * r[VV]; fr[3] = r[MX] * r[VW];
  fr[4] = (r[EN] + r[PR]) * r[VU];
#pragma unroll
  for (int j = 0; j < 5; ++j) f[j] = (R)0.5 * (fl[j] + fr[j]) - (R)0.5 * lam * (r[j] - l[j]);
}

// flux.c:344-406
template <class R>
__device__ __forceinline__ void flux_ausm(const R* l, const R* r, const Phys<R>& ph, R* f) {
  R cl = sqrt(ph.kappa * l[PR] / l[RHO]);
  R cr = sqrt(ph.kappa * r[PR] / r[RHO]);
  R ml = l[VU] / cl, mr = r[VU] / cr;
  R hl = (l[EN] + l[PR]) / l[RHO];
  R hr = (r[EN] + r[PR]) / r[RHO];
  R mp, pp, mm, pm;
  if (ml <= (R)-1) { mp = 0; pp = 0; }
  else if (ml < (R)1) {
    mp = (R)0.25 * (ml + (R)1) * (ml + (R)1);
    pp = (R)0.25 * l[PR] * ((R)1 + ml) * ((R)1 + ml) * ((R)2 - ml);
  } else { mp = ml; pp = l[PR]; }
  if (mr <= (R)-1) { mm = mr; pm = r[PR]; }
  else if (mr < (R)1) {
    mm = (R)-0.25 * (mr - (R)1) * (mr - (R)1);
    pm = (R)0.25 * r[PR] * ((R)1 - mr) * ((R)1 - mr) * ((R)2 + mr);
  } else { mm = 0; pm = 0; }
  R up = rmax((R)0, mp + mm), um = rmin((R)0, mp + mm);
  R ml_ = up * cl * l[RHO], mr_ = um * cr * r[RHO];
  f[0] = ml_;
  f[1] = ml_ * l[VU] + pp;
  f[2] = ml_ * l[VV];
  f[3] = ml_ * l[VW];
  f[4] = ml_ * hl;
  f[0] += mr_;
  f[1] += mr_ * r[VU] + pm;
  f[2] += mr_ * r[VV];
  f[3] += mr_ * r[VW];
  f[4] += mr_ * hr;
}

// Normal viscous flux of one side (flux.c:215-263 dotted with n): stresses
// from the gradients of the conserved momenta (as the reference computes
// them), heat flux from grad T.  gm = gradients of (rho_u, rho_v, rho_w, T),
// layout [var][xyz].  Returns components 1..4 (component 0 is zero).
template <class R>
__device__ __forceinline__ void viscous_side(const R* q, const R* gm, const R* n,
                                             const Phys<R>& ph, R* fv, R* gv, R* hv) {
  const R s23 = (R)(2.0 / 3.0), s43 = (R)(4.0 / 3.0), mu = ph.mu;
  // gm[v*3 + d]: v = 0 rho_u, 1 rho_v, 2 rho_w, 3 T
  R txx = mu * (s43 * gm[0] - s23 * gm[4] - s23 * gm[8]);
  R tyy = mu * (-s23 * gm[0] + s43 * gm[4] - s23 * gm[8]);
  R tzz = mu * (-s23 * gm[0] - s23 * gm[4] + s43 * gm[8]);
  R txy = mu * (gm[1] + gm[3]);
  R txz = mu * (gm[2] + gm[6]);
  R tyz = mu * (gm[5] + gm[7]);
  const R k = ph.heat_lambda;
  fv[0] = -txx; fv[1] = -txy; fv[2] = -txz;
  fv[3] = -txx * q[VU] - txy * q[VV] - txz * q[VW] - k * gm[9];
  gv[0] = -txy; gv[1] = -tyy; gv[2] = -tyz;
  gv[3] = -txy * q[VU] - tyy * q[VV] - tyz * q[VW] - k * gm[10];
  hv[0] = -txz; hv[1] = -tyz; hv[2] = -tzz;
  hv[3] = -txz * q[VU] - tyz * q[VV] - tzz * q[VW] - k * gm[11];
  (void)n;
}

// Kahan-compensated accumulator (mixed path); plain sum for double.
template <class R, bool KAHAN>
struct Acc {
  R s, c;
  __device__ __forceinline__ Acc() : s((R)0), c((R)0) {}
  __device__ __forceinline__ void add(R x) {
    if (KAHAN) {
      R y = x - c;
      R t = s + y;
      c = (t - s) - y;
      s = t;
    } else {
      s += x;
    }
  }
  __device__ __forceinline__ void sub(R x) {
    if (KAHAN) add(-x);
    else s -= x;
  }
  // compensated total (c carries the negated low-order part)
  __device__ __forceinline__ R value() const { return KAHAN ? s - c : s; }
};

}  // namespace fv3d
