// First-order face flux of the implicit solve's preconditioners (FP64).
#pragma once

#include "kernels.cuh"

namespace fv3d {

// global-frame convective flux . n (FP64): AUSM or Rusanov (flux.c:320-406)
// of the conserved states l, r (cell-centre values: first order), plus, when
// visc and mu != 0, a two-point viscous flux over the centre distance n[3]
__device__ inline void fo_flux(const double* l, const double* r, const double* n, const PhysConst& pc,
                               double* F, bool visc = true) {
  const double km1 = pc.km1, kappa = pc.kappa;
  const double irl = 1.0 / l[0], irr = 1.0 / r[0];
  const double ul = l[1] * irl, vl = l[2] * irl, wl = l[3] * irl;
  const double ur = r[1] * irr, vr = r[2] * irr, wr = r[3] * irr;
  const double pl = fmax(1.00E-10, km1 * (l[4] - 0.5 * (l[1] * ul + l[2] * vl + l[3] * wl)));
  const double pr = fmax(1.00E-10, km1 * (r[4] - 0.5 * (r[1] * ur + r[2] * vr + r[3] * wr)));
  const double unl = ul * n[0] + vl * n[1] + wl * n[2];
  const double unr = ur * n[0] + vr * n[1] + wr * n[2];
  const double cl = sqrt(kappa * pl * irl), cr = sqrt(kappa * pr * irr);
  if (pc.flux == 1) {
    const double lam = fmax(fabs(unl) + cl, fabs(unr) + cr);
    F[0] = 0.5 * (l[0] * unl + r[0] * unr) - 0.5 * lam * (r[0] - l[0]);
    for (int d = 0; d < 3; ++d)
      F[1 + d] = 0.5 * (l[1 + d] * unl + pl * n[d] + r[1 + d] * unr + pr * n[d]) - 0.5 * lam * (r[1 + d] - l[1 + d]);
    F[4] = 0.5 * ((l[4] + pl) * unl + (r[4] + pr) * unr) - 0.5 * lam * (r[4] - l[4]);
  } else {
    const double Ml = unl / cl, Mr = unr / cr;
    double mp, pp, mm, pm;
    if (Ml <= -1.0) { mp = 0.0; pp = 0.0; }
    else if (Ml < 1.0) { mp = 0.25 * (Ml + 1.0) * (Ml + 1.0); pp = 0.25 * pl * (1.0 + Ml) * (1.0 + Ml) * (2.0 - Ml); }
    else { mp = Ml; pp = pl; }
    if (Mr <= -1.0) { mm = Mr; pm = pr; }
    else if (Mr < 1.0) { mm = -0.25 * (Mr - 1.0) * (Mr - 1.0); pm = 0.25 * pr * (1.0 - Mr) * (1.0 - Mr) * (2.0 + Mr); }
    else { mm = 0.0; pm = 0.0; }
    const double mdl = fmax(0.0, mp + mm) * cl * l[0];
    const double mdr = fmin(0.0, mp + mm) * cr * r[0];
    F[0] = mdl + mdr;
    F[1] = mdl * ul + mdr * ur + (pp + pm) * n[0];
    F[2] = mdl * vl + mdr * vr + (pp + pm) * n[1];
    F[3] = mdl * wl + mdr * wr + (pp + pm) * n[2];
    F[4] = mdl * (l[4] + pl) * irl + mdr * (r[4] + pr) * irr;
  }
  // two-point viscous flux across the face: -mu du/dn, -(mu u.du/dn + k dT/dn)
  if (visc && pc.mu != 0.0) {
    const double id = 1.0 / n[3];  // n[3] carries the centre distance
    const double mu = pc.mu, k = pc.heat_lambda;
    const double Tl = pl * irl / pc.R_mix, Tr = pr * irr / pc.R_mix;
    const double du = ur - ul, dv = vr - vl, dw = wr - wl;
    F[1] -= mu * du * id;
    F[2] -= mu * dv * id;
    F[3] -= mu * dw * id;
    F[4] -= (mu * (0.5 * (ul + ur) * du + 0.5 * (vl + vr) * dv + 0.5 * (wl + wr) * dw) + k * (Tr - Tl)) * id;
  }
}


}  // namespace fv3d
