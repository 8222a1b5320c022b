// Mixed-precision explicit stage for sm_103a: two launches per RK stage.
//
//  k_mx_sides        (gradient pass, cell-gather) per cell: neighbour states
//                    -> Green-Gauss / least-squares gradients and the
//                    Barth-Jespersen bounds in registers, then for each of the
//                    cell's faces the limited reconstructed state and that
//                    side's viscous normal flux; one 48-byte record per face
//                    side (the ghost side of a boundary face is written by its
//                    interior cell).
//  k_mx_flux_update  (flux + update pass, cell-gather) per cell: for each of
//                    its faces the convective flux from both side records
//                    plus the averaged viscous flux, summed with Kahan
//                    compensation in ascending reference face id, -sum/V,
//                    fused FP64 RK update, FP32 shadow state, next time step.
//
// Each face flux is evaluated by both of its cells from identical inputs with
// identical instructions, so the two contributions cancel exactly and the
// scheme stays conservative; no face-flux buffer and no atomics.
// Fluxes are evaluated in the global frame: the reference rotates momenta
// into (n, t1, t2), applies the 1-D flux and rotates back (flux.c:56-84),
// which for Rusanov and AUSM is algebraically the global-frame formula below.
#pragma once

#include "kernels.cuh"

namespace fv3d {

constexpr int FS = 12;  // floats per face-side record: q[0..7], viscous (mx, my, mz, e)

struct MxArgs {
  int nc, nf, nf_int, mcf;
  const int* __restrict__ cface;     // [nc][mcf]
  const int2* __restrict__ fcell;    // [nf] (cell 0, cell 1 or ghost)
  const float4* __restrict__ geoN;   // [nf] (n, A)
  const float4* __restrict__ geoD;   // [2][nf] (d_side, lambda)
  const float4* __restrict__ lsqW;   // [2][nf] (w_side, 0)
  const int* __restrict__ fregion;   // [nf - nf_int]
  const float* __restrict__ rvol;    // [nc]
  const double* __restrict__ vol;    // [nc]
  const double* __restrict__ dx;     // [nc][3]
  float* Uf;                         // [nc][8]
  float* fs;                         // [nf][2][FS]
  double* U;                         // [5][nc]
  double* K;                         // [5][nc]
  double* U0;                        // [5][nc]
  double* dphi;                      // [5][nc]
  DevScalars* sc;
  PhysConst pc;
};

struct MxPhys {
  float kappa, km1, s_km1, s_kp1, R, mu, heat;
  int flux;
  __device__ __forceinline__ void load(const PhysConst& c) {
    kappa = (float)c.kappa; km1 = (float)c.km1; s_km1 = (float)c.s_km1; s_kp1 = (float)c.s_kp1;
    R = (float)c.R_mix; mu = (float)c.mu; heat = (float)c.heat_lambda; flux = c.flux;
  }
};

__device__ __forceinline__ void mx_load_state(const float* __restrict__ Uf, int c, float* q) {
  const float4* s = reinterpret_cast<const float4*>(Uf) + 2 * (size_t)c;
  float4 x = __ldg(s), y = __ldg(s + 1);
  q[RHO] = x.x; q[MX] = x.y; q[MY] = x.z; q[MZ] = x.w; q[EN] = y.x; q[PR] = y.y; q[TT] = y.z;
  const float ir = 1.0f / x.x;
  q[VU] = x.y * ir; q[VV] = x.z * ir; q[VW] = x.w * ir;
}

// eos.c:55-75 with the face-normal velocity un
__device__ __forceinline__ float mx_wall_pressure(float rho, float p, float un, const MxPhys& ph) {
  if (un <= 0.f) {
    float c = sqrtf(ph.kappa * p / rho);
    return p * powf(fmaxf(1e-4f, 1.f + 0.5f * ph.km1 * un / c), 2.f * ph.kappa * ph.s_km1);
  }
  float ar = 2.f * ph.s_kp1 / un;
  float br = ph.km1 * ph.s_kp1 * p;
  return p + un / ar * 0.5f * (un + sqrtf(un * un + 4.f * ar * (p + br)));
}

// boundary.c:188-320 without the (n, t1, t2) rotation; pressure outlet new
__device__ __forceinline__ void mx_ghost(const float* in, int region, const float* n,
                                         const PhysConst& pc, const MxPhys& ph, float* g) {
#pragma unroll
  for (int j = 0; j < 10; ++j) g[j] = in[j];
  const int type = pc.region_type[region];
  if (type == BC_INFLOW || type == BC_STATE) {
#pragma unroll
    for (int j = 0; j < 10; ++j) g[j] = (float)pc.region_phi[region][j];
  } else if (type == BC_PRESSURE_OUTLET) {
    g[PR] = (float)pc.region_phi[region][PR];
    g[TT] = g[PR] / (g[RHO] * ph.R);
  } else if (type == BC_WALL_ADIABATIC || type == BC_WALL_ISOTHERMAL || type == BC_WALL_SLIP ||
             type == BC_SYMMETRY) {
    const float un = in[VU] * n[0] + in[VV] * n[1] + in[VW] * n[2];
    g[PR] = mx_wall_pressure(in[RHO], in[PR], un, ph);
    if (type == BC_WALL_SLIP || type == BC_SYMMETRY) {
      g[VU] = in[VU] - un * n[0];
      g[VV] = in[VV] - un * n[1];
      g[VW] = in[VW] - un * n[2];
      g[TT] = g[PR] / (g[RHO] * ph.R);
    } else {
      g[VU] = 0.f; g[VV] = 0.f; g[VW] = 0.f;
      if (type == BC_WALL_ISOTHERMAL) g[TT] = (float)pc.region_phi[region][TT];
      g[RHO] = g[PR] / (ph.R * g[TT]);
    }
  }
  // prim_to_con (eos.c:120-127)
  g[MX] = g[VU] * g[RHO];
  g[MY] = g[VV] * g[RHO];
  g[MZ] = g[VW] * g[RHO];
  g[EN] = ph.s_km1 * g[PR] + 0.5f * (g[VU] * g[MX] + g[VV] * g[MY] + g[VW] * g[MZ]);
}

// viscous normal flux of one side times the area: F_visc . (n A) for the
// momentum and energy rows (flux.c:215-263; stresses from the conserved
// momentum gradients as in the reference).  gm[v*3+d], v: rho_u, rho_v, rho_w, T.
__device__ __forceinline__ void mx_viscous(const float* q, const float* gm, const float* nA,
                                           const MxPhys& ph, float* v) {
  const float s23 = 2.0f / 3.0f, s43 = 4.0f / 3.0f, mu = ph.mu;
  const float txx = mu * (s43 * gm[0] - s23 * gm[4] - s23 * gm[8]);
  const float tyy = mu * (-s23 * gm[0] + s43 * gm[4] - s23 * gm[8]);
  const float tzz = mu * (-s23 * gm[0] - s23 * gm[4] + s43 * gm[8]);
  const float txy = mu * (gm[1] + gm[3]);
  const float txz = mu * (gm[2] + gm[6]);
  const float tyz = mu * (gm[5] + gm[7]);
  const float k = ph.heat;
  v[0] = -(txx * nA[0] + txy * nA[1] + txz * nA[2]);
  v[1] = -(txy * nA[0] + tyy * nA[1] + tyz * nA[2]);
  v[2] = -(txz * nA[0] + tyz * nA[1] + tzz * nA[2]);
  const float ex = -txx * q[VU] - txy * q[VV] - txz * q[VW] - k * gm[9];
  const float ey = -txy * q[VU] - tyy * q[VV] - tyz * q[VW] - k * gm[10];
  const float ez = -txz * q[VU] - tyz * q[VV] - tzz * q[VW] - k * gm[11];
  v[3] = ex * nA[0] + ey * nA[1] + ez * nA[2];
}

// ---------------------------------------------------------------------------
// gradient pass
// ---------------------------------------------------------------------------
template <int GMODE, bool LINEAR, bool LIMIT, bool VISC>
__global__ void __launch_bounds__(256) k_mx_sides(const __grid_constant__ MxArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nc) return;
  MxPhys ph;
  ph.load(a.pc);
  float q[10];
  mx_load_state(a.Uf, c, q);
  float g[NG][3];
  float mn[8], mxv[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) { mn[v] = q[v]; mxv[v] = q[v]; }
  const int* cf = a.cface + (size_t)c * a.mcf;
  if (GMODE != 0) {
    Acc<float, true> acc[NG][3];
    for (int k = 0; k < a.mcf; ++k) {
      const int e = cf[k];
      if (e < 0) break;
      const int f = e >> 1, side = e & 1;
      const float4 nA = __ldg(&a.geoN[f]);
      float qo[10];
      if (f >= a.nf_int) {
        const float n[3] = {nA.x, nA.y, nA.z};
        mx_ghost(q, a.fregion[f - a.nf_int], n, a.pc, ph, qo);
      } else {
        const int2 fc = __ldg(&a.fcell[f]);
        mx_load_state(a.Uf, side ? fc.x : fc.y, qo);
      }
      if (GMODE == 1) {
        const float lam = __ldg(&a.geoD[(size_t)side * a.nf + f]).w;
        const float sg = side ? -nA.w : nA.w;
        const float ax = nA.x * sg, ay = nA.y * sg, az = nA.z * sg;
        const float* q0 = side ? qo : q;
        const float* q1 = side ? q : qo;
#pragma unroll
        for (int v = 0; v < NG; ++v) {
          const int j = (v < 8) ? v : TT;
          const float mean = q0[j] + lam * (q1[j] - q0[j]);
          acc[v][0].add(mean * ax);
          acc[v][1].add(mean * ay);
          acc[v][2].add(mean * az);
        }
      } else {
        const float4 w = __ldg(&a.lsqW[(size_t)side * a.nf + f]);
#pragma unroll
        for (int v = 0; v < NG; ++v) {
          const int j = (v < 8) ? v : TT;
          const float dq = qo[j] - q[j];
          acc[v][0].add(w.x * dq);
          acc[v][1].add(w.y * dq);
          acc[v][2].add(w.z * dq);
        }
      }
      if (LIMIT) {
#pragma unroll
        for (int v = 0; v < 8; ++v) { mn[v] = fminf(mn[v], qo[v]); mxv[v] = fmaxf(mxv[v], qo[v]); }
      }
    }
    const float s = (GMODE == 1) ? __ldg(&a.rvol[c]) : 1.0f;
#pragma unroll
    for (int v = 0; v < NG; ++v)
#pragma unroll
      for (int d = 0; d < 3; ++d) g[v][d] = acc[v][d].value() * s;
  } else {
#pragma unroll
    for (int v = 0; v < NG; ++v) { g[v][0] = 0.f; g[v][1] = 0.f; g[v][2] = 0.f; }
  }
  // per face side: limited reconstruction + viscous flux
  for (int k = 0; k < a.mcf; ++k) {
    const int e = cf[k];
    if (e < 0) break;
    const int f = e >> 1, side = e & 1;
    const float4 nA4 = __ldg(&a.geoN[f]);
    const float nA[3] = {nA4.x * nA4.w, nA4.y * nA4.w, nA4.z * nA4.w};
    float r[12];
    if (LINEAR) {
      const float4 d = __ldg(&a.geoD[(size_t)side * a.nf + f]);
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const float slope = d.x * g[v][0] + d.y * g[v][1] + d.z * g[v][2];
        float inc = slope;
        if (LIMIT)  // min(1, y) * slope of limiter.c:86-106 without the division
          inc = (slope > 0.f) ? fminf(slope, mxv[v] - q[v]) : ((slope < 0.f) ? fmaxf(slope, mn[v] - q[v]) : 0.f);
        r[v] = q[v] + inc;
      }
    } else {
#pragma unroll
      for (int v = 0; v < 8; ++v) r[v] = q[v];
    }
    float gm[12];
    if (VISC) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        gm[d] = g[1][d]; gm[3 + d] = g[2][d]; gm[6 + d] = g[3][d]; gm[9 + d] = g[8][d];
      }
      mx_viscous(r, gm, nA, ph, &r[8]);
    } else {
      r[8] = r[9] = r[10] = r[11] = 0.f;
    }
    float4* dst = reinterpret_cast<float4*>(a.fs + ((size_t)f * 2 + side) * FS);
    dst[0] = make_float4(r[0], r[1], r[2], r[3]);
    dst[1] = make_float4(r[4], r[5], r[6], r[7]);
    dst[2] = make_float4(r[8], r[9], r[10], r[11]);
    if (f >= a.nf_int) {
      // ghost side: unlimited ghost of the cell-centre state
      // (reconstruction.c:249-253), gradient = interior gradient with the
      // normal part removed on slip walls / symmetry (boundary.c:377-405)
      const int region = a.fregion[f - a.nf_int];
      const float n[3] = {nA4.x, nA4.y, nA4.z};
      float gq[10];
      mx_ghost(q, region, n, a.pc, ph, gq);
      float rg[12];
#pragma unroll
      for (int v = 0; v < 8; ++v) rg[v] = gq[v];
      if (VISC) {
        const int type = a.pc.region_type[region];
        if (type == BC_WALL_SLIP || type == BC_SYMMETRY) {
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const float gn = gm[3 * v] * n[0] + gm[3 * v + 1] * n[1] + gm[3 * v + 2] * n[2];
            gm[3 * v] -= gn * n[0]; gm[3 * v + 1] -= gn * n[1]; gm[3 * v + 2] -= gn * n[2];
          }
        }
        mx_viscous(rg, gm, nA, ph, &rg[8]);
      } else {
        rg[8] = rg[9] = rg[10] = rg[11] = 0.f;
      }
      float4* gd = reinterpret_cast<float4*>(a.fs + ((size_t)f * 2 + 1) * FS);
      gd[0] = make_float4(rg[0], rg[1], rg[2], rg[3]);
      gd[1] = make_float4(rg[4], rg[5], rg[6], rg[7]);
      gd[2] = make_float4(rg[8], rg[9], rg[10], rg[11]);
    }
  }
}

// ---------------------------------------------------------------------------
// flux + update pass
// ---------------------------------------------------------------------------
// convective face flux in the global frame, times A
__device__ __forceinline__ void mx_conv_flux(const float* l, const float* r, const float4 nA,
                                             const MxPhys& ph, float* F) {
  const float n0 = nA.x, n1 = nA.y, n2 = nA.z, A = nA.w;
  // primitives of the (reconstructed) conserved states (eos.c:81-92)
  const float irl = 1.f / l[RHO], irr = 1.f / r[RHO];
  const float ul = l[MX] * irl, vl = l[MY] * irl, wl = l[MZ] * irl;
  const float ur = r[MX] * irr, vr = r[MY] * irr, wr = r[MZ] * irr;
  const float pl = fmaxf(1.00E-10f, ph.km1 * (l[EN] - 0.5f * (l[MX] * ul + l[MY] * vl + l[MZ] * wl)));
  const float pr = fmaxf(1.00E-10f, ph.km1 * (r[EN] - 0.5f * (r[MX] * ur + r[MY] * vr + r[MZ] * wr)));
  const float unl = ul * n0 + vl * n1 + wl * n2;
  const float unr = ur * n0 + vr * n1 + wr * n2;
  const float cl = sqrtf(ph.kappa * pl * irl), cr = sqrtf(ph.kappa * pr * irr);
  if (ph.flux == 1) {  // Rusanov, flux.c:320-336
    const float lam = fmaxf(fabsf(unl) + cl, fabsf(unr) + cr);
    const float ml = l[RHO] * unl, mr = r[RHO] * unr;
    F[0] = 0.5f * (ml + mr) - 0.5f * lam * (r[RHO] - l[RHO]);
    F[1] = 0.5f * (l[MX] * unl + pl * n0 + r[MX] * unr + pr * n0) - 0.5f * lam * (r[MX] - l[MX]);
    F[2] = 0.5f * (l[MY] * unl + pl * n1 + r[MY] * unr + pr * n1) - 0.5f * lam * (r[MY] - l[MY]);
    F[3] = 0.5f * (l[MZ] * unl + pl * n2 + r[MZ] * unr + pr * n2) - 0.5f * lam * (r[MZ] - l[MZ]);
    F[4] = 0.5f * ((l[EN] + pl) * unl + (r[EN] + pr) * unr) - 0.5f * lam * (r[EN] - l[EN]);
  } else {  // AUSM, flux.c:344-406
    const float Ml = unl / cl, Mr = unr / cr;
    float mp, pp, mm, pm;
    if (Ml <= -1.f) { mp = 0.f; pp = 0.f; }
    else if (Ml < 1.f) { mp = 0.25f * (Ml + 1.f) * (Ml + 1.f); pp = 0.25f * pl * (1.f + Ml) * (1.f + Ml) * (2.f - Ml); }
    else { mp = Ml; pp = pl; }
    if (Mr <= -1.f) { mm = Mr; pm = pr; }
    else if (Mr < 1.f) { mm = -0.25f * (Mr - 1.f) * (Mr - 1.f); pm = 0.25f * pr * (1.f - Mr) * (1.f - Mr) * (2.f + Mr); }
    else { mm = 0.f; pm = 0.f; }
    const float mdl = fmaxf(0.f, mp + mm) * cl * l[RHO];
    const float mdr = fminf(0.f, mp + mm) * cr * r[RHO];
    const float P = pp + pm;
    F[0] = mdl + mdr;
    F[1] = mdl * ul + mdr * ur + P * n0;
    F[2] = mdl * vl + mdr * vr + P * n1;
    F[3] = mdl * wl + mdr * wr + P * n2;
    F[4] = mdl * (l[EN] + pl) * irl + mdr * (r[EN] + pr) * irr;
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) F[j] *= A;
}

template <int MODE, bool DT, bool VISC>
__global__ void __launch_bounds__(256) k_mx_flux_update(const __grid_constant__ MxArgs a,
                                                        StageCoef co) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long lam_bits = 0x7ff0000000000000ull;
  bool finite = true;
  if (c < a.nc) {
    MxPhys ph;
    ph.load(a.pc);
    Acc<float, true> s[5];
    const int* cf = a.cface + (size_t)c * a.mcf;
    for (int k = 0; k < a.mcf; ++k) {
      const int e = cf[k];
      if (e < 0) break;
      const int f = e >> 1, side = e & 1;
      const float4* src = reinterpret_cast<const float4*>(a.fs + (size_t)f * 2 * FS);
      float l[12], r[12];
      float4 t;
      t = __ldg(src + 0); l[0] = t.x; l[1] = t.y; l[2] = t.z; l[3] = t.w;
      t = __ldg(src + 1); l[4] = t.x; l[5] = t.y; l[6] = t.z; l[7] = t.w;
      t = __ldg(src + 3); r[0] = t.x; r[1] = t.y; r[2] = t.z; r[3] = t.w;
      t = __ldg(src + 4); r[4] = t.x; r[5] = t.y; r[6] = t.z; r[7] = t.w;
      const float4 nA = __ldg(&a.geoN[f]);
      float F[5];
      mx_conv_flux(l, r, nA, ph, F);
      if (VISC) {
        const float4 vl = __ldg(src + 2), vr = __ldg(src + 5);
        F[1] += 0.5f * (vl.x + vr.x);
        F[2] += 0.5f * (vl.y + vr.y);
        F[3] += 0.5f * (vl.z + vr.z);
        F[4] += 0.5f * (vl.w + vr.w);
      }
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        if (side) s[j].sub(F[j]);
        else s[j].add(F[j]);
      }
    }
    const float rv = __ldg(&a.rvol[c]);
    double rr[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) rr[j] = (double)(-s[j].value() * rv);
    if (MODE == 0) {
#pragma unroll
      for (int j = 0; j < 5; ++j) a.dphi[(size_t)j * a.nc + c] = rr[j];
    } else {
      const double dt = a.sc->dt;
      const double dtg = dt * co.g;
      double u[5];
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const size_t i = (size_t)j * a.nc + c;
        double uj = a.U[i];
        if (MODE == 1) {
          const double kj = co.first ? rr[j] : fma(a.K[i], co.a, rr[j]);
          a.K[i] = kj;
          uj = fma(kj, dtg, uj);
        } else {
          if (co.first) {
            a.U0[i] = uj;
            uj = fma(dt, rr[j], uj);
          } else {
            uj = co.c0 * a.U0[i] + co.c1 * fma(dt, rr[j], uj);
          }
        }
        a.U[i] = uj;
        u[j] = uj;
        finite = finite && isfinite(uj);
      }
      float4* sh = reinterpret_cast<float4*>(a.Uf) + 2 * (size_t)c;
      const float4 o0 = sh[0], o1 = sh[1];
      const float rho = (float)u[0], mx = (float)u[1], my = (float)u[2], mz = (float)u[3];
      const float ir = 1.f / rho;
      const float vx = mx * ir, vy = my * ir, vz = mz * ir;
      const float ke = 0.5f * (mx * vx + my * vy + mz * vz);
      float p = (float)(a.pc.km1 * (u[4] - (double)ke));
      p = fmaxf(1.00E-10f, p);
      const float T = p * ir / ph.R;
      sh[0] = make_float4(rho, mx, my, mz);
      sh[1] = make_float4((float)u[4], p, T, 0.f);
      if (DT) {
        // calc_ns_timestep on the reference's phi_total: new density, the
        // stage-input u, v, w, p for the low-storage schemes (see
        // k_gather_update); new state for SSP-RK3
        float pu = vx, pv = vy, pw = vz, pp = p;
        if (MODE == 1) {
          const float io = 1.f / o0.x;
          pu = o0.y * io; pv = o0.z * io; pw = o0.w * io; pp = o1.y;
        }
        const float cs = sqrtf(ph.kappa * pp * ir);
        const double* d = a.dx + 3 * (size_t)c;
        const float ds = (fabsf(pu) + cs) * (float)d[0] + (fabsf(pv) + cs) * (float)d[1] +
                         (fabsf(pw) + cs) * (float)d[2];
        const double lam = (double)((float)a.vol[c] / ds);
        if (lam > 0.0) lam_bits = (unsigned long long)__double_as_longlong(lam);
      }
    }
  }
  if (MODE != 0) {
    if (!finite) atomicOr(&a.sc->status, 1);
    if (DT) {
      lam_bits = warp_min_u64(lam_bits);
      if ((threadIdx.x & 31) == 0 && lam_bits != 0x7ff0000000000000ull)
        atomicMin(&a.sc->lam_bits, lam_bits);
    }
  }
}

}  // namespace fv3d
