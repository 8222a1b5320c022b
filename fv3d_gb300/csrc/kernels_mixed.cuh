// Mixed-precision explicit stage for sm_103a: two launches per RK stage.
//
//  k_mx_sides        (gradient pass, cell-gather) per cell: neighbour states
//                    -> Green-Gauss / least-squares gradients and the
//                    Barth-Jespersen bounds in registers, then for each of the
//                    cell's faces the limited reconstructed conserved state
//                    and that side's viscous normal flux, written into the
//                    cell's face-side record of that slot (the ghost side of
//                    a boundary face is written by its interior cell).
//  k_mx_flux_update  (flux + update pass, cell-gather) per cell: for each of
//                    its faces the convective flux from both side records
//                    (its own, and the other side's through cother) plus
//                    the averaged viscous flux, summed in ascending
//                    reference face id, -sum/V, RK stage update, FP32
//                    stage state, next time step.
//
// Each face flux is evaluated by both of its cells from identical inputs with
// identical instructions, so the two contributions cancel exactly and the
// scheme stays conservative; no face-flux buffer and no atomics.
//
// Fluxes are evaluated in the global frame: the reference rotates momenta
// into (n, t1, t2), applies the 1-D flux and rotates back (flux.c:56-84),
// which for Rusanov and AUSM is algebraically the global-frame formula below.
//
// Precision: faces, gradients, limiter, residual in FP32.  The conserved
// state U_n is FP64; within a step the RK register and the increment
// dU = U_stage - U_n are FP32 (they are O(dt R), so FP32 rounding of them is
// far below the FP32 residual error), and the end of each step forms
// U_{n+1} = U_n + dU in FP64.  The stage state the next gradient pass reads
// is the FP32 record Uf = float(U_n) + dU.
#pragma once

#include "kernels.cuh"

namespace fv3d {

// minimum resident blocks of 256 threads for the gradient pass (a register
// cap; 2 keeps it spill-free)
#ifndef FV3D_SIDES_MINBLOCKS
#define FV3D_SIDES_MINBLOCKS 2
#endif
// unroll factor of the gradient-pass neighbour loop (1 keeps one neighbour
// live at a time: fewer registers, more resident warps)
#ifndef FV3D_SIDES_UNROLL
#define FV3D_SIDES_UNROLL 8
#endif
// second-order gradient passes staged through shared memory by bulk
// asynchronous copies (k_mx_sides_tma); 0 = k_mx_sides reading global memory
#ifndef FV3D_SIDES_TMA
#define FV3D_SIDES_TMA 1
#endif
#ifndef FV3D_TMA_MINBLOCKS
#define FV3D_TMA_MINBLOCKS 4
#endif

#ifndef FV3D_FLUX_MINBLOCKS
#define FV3D_FLUX_MINBLOCKS 1
#endif
// resident blocks of the 4-slot flux pass (48 registers at 5)
#ifndef FV3D_FLUX4_MINBLOCKS
#define FV3D_FLUX4_MINBLOCKS 5
#endif
#ifndef FV3D_FLUX_UNROLL
#define FV3D_FLUX_UNROLL 8
#endif
// the flux pass sums a cell's face fluxes in slot order (ascending
// reference face id) with compensated (Kahan) FP32 sums; 0 = plain sums
#ifndef FV3D_FLUX_KAHAN
#define FV3D_FLUX_KAHAN 1
#endif
constexpr bool kFluxKahan = FV3D_FLUX_KAHAN != 0;
constexpr int kSidesUnroll = FV3D_SIDES_UNROLL;
constexpr int kFluxUnroll = FV3D_FLUX_UNROLL;

// face-side record: one full 32-byte sector (rho, mx, my, mz), (E, vmx,
// vmy, vmz), v* = viscous normal flux times A; the side's viscous energy
// flux in fsv at the same index.  A cell's own sides are stored slot-major
// (record k * ncp + c for slot k of cell c), so the gradient pass writes and
// the flux pass reads them with contiguous warp accesses; the ghost side of
// boundary face nf_int + b is record mcf * ncp + b; cother gives each slot
// the index of its face's other side.

// cells per tile of the staged gradient pass (k_mx_sides_tma): one thread per
// cell; the per-cell arrays it stages are padded to whole tiles (ncp rows)
constexpr int kTile = 128;

struct MxArgs {
  int nc, nf, nf_int, mcf;
  int ncp;                           // nc rounded up to whole tiles
  const int* __restrict__ cface;     // [nc][mcf]
  const int* __restrict__ cnbr;      // [nc][mcf] neighbour cell, -1 ghost, -2 none
  const int2* __restrict__ fcell;    // [nf] (cell 0, cell 1 or ghost)
  const float4* __restrict__ slotN;  // [nc][mcf] face (n, A), cell 0 -> cell 1 orientation
  const float4* __restrict__ slotD;  // [nc][mcf] (d of this side, Green-Gauss weight)
  const float4* __restrict__ slotW;  // [nc][mcf] least-squares weights of this side
  const float4* __restrict__ slotNk; // [mcf][ncp] slotN again, slot-major (flux pass: a warp's
                                     // load of slot k is 512 contiguous bytes; staged gradient pass)
  const float4* __restrict__ slotDk; // [mcf][ncp] slotD, slot-major
  const float4* __restrict__ slotWk; // [mcf][ncp] slotW, slot-major (least squares only)
  const int* __restrict__ fregion;   // [nf - nf_int]
  const float4* __restrict__ cgeo;   // [ncp] (sum_f s_f n_f A_f, 1/V)
  const float4* __restrict__ cdx;    // [ncp] (dx, V)
  float* Uf;                         // [nc][8] stage state (rho, m, E, p, T, 1/rho)
  float* UfN;                        // [nc][8] float(U_n) + p, T
  const int* __restrict__ cother;    // [ncp][mcf] (the other side's record << 1) | side, -1 none
  float* fs;                         // [mcf * ncp + nb][8] face-side records: a cell's own sides
                                     // slot-major ([k][ncp]), then the ghost sides by boundary
  float* fsv;                        // [mcf * ncp + nb] viscous energy flux of each side, same index
  double* U;                         // [5][nc] conserved state U_n (FP64)
  float* kf;                         // [5][ncp] RK register (FP32)
  float* dU;                         // [5][ncp] U_stage - U_n (FP32)
  double* dphi;                      // [5][nc]
  DevScalars* sc;
  PhysConst pc;
};

struct MxPhys {
  float kappa, km1, s_km1, s_kp1, R, mu, heat;
  int flux;
  __device__ __forceinline__ void load(const PhysConst& c) {
    kappa = c.f32[0]; km1 = c.f32[1]; s_km1 = c.f32[2]; s_kp1 = c.f32[3];
    R = c.f32[4]; mu = c.f32[5]; heat = c.f32[6]; flux = c.flux;
  }
};

// record (rho, m, E), (E, p, T, 1/rho): every writer stores the IEEE
// reciprocal 1.0f / rho in the last word, so readers need no division
__device__ __forceinline__ void mx_unpack(const float4 x, const float4 y, float* q) {
  q[RHO] = x.x; q[MX] = x.y; q[MY] = x.z; q[MZ] = x.w; q[EN] = y.x; q[PR] = y.y; q[TT] = y.z;
  const float ir = y.w;
  q[VU] = x.y * ir; q[VV] = x.z * ir; q[VW] = x.w * ir;
}

// 32-byte records in one request: ld / st .v8.f32 (256-bit global
// accesses, sm_100 and later).  Every record passed here starts at a
// multiple of 32 bytes from a cudaMalloc base, as these require.
#ifndef FV3D_V8
#define FV3D_V8 1
#endif
__device__ __forceinline__ void ld_rec_nc(const float* p, float4& x, float4& y) {
#if FV3D_V8
  asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(x.x), "=f"(x.y), "=f"(x.z), "=f"(x.w), "=f"(y.x), "=f"(y.y), "=f"(y.z), "=f"(y.w)
               : "l"(p));
#else
  x = __ldg(reinterpret_cast<const float4*>(p));
  y = __ldg(reinterpret_cast<const float4*>(p) + 1);
#endif
}
// for a record this thread overwrites later in the same launch
__device__ __forceinline__ void ld_rec(const float* p, float4& x, float4& y) {
#if FV3D_V8
  asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(x.x), "=f"(x.y), "=f"(x.z), "=f"(x.w), "=f"(y.x), "=f"(y.y), "=f"(y.z), "=f"(y.w)
               : "l"(p) : "memory");
#else
  x = reinterpret_cast<const float4*>(p)[0];
  y = reinterpret_cast<const float4*>(p)[1];
#endif
}
__device__ __forceinline__ void st_rec(float* p, const float4 x, const float4 y) {
#if FV3D_V8
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(x.x), "f"(x.y), "f"(x.z),
               "f"(x.w), "f"(y.x), "f"(y.y), "f"(y.z), "f"(y.w)
               : "memory");
#else
  reinterpret_cast<float4*>(p)[0] = x;
  reinterpret_cast<float4*>(p)[1] = y;
#endif
}
__device__ __forceinline__ void ld_unpack(const float* rec, float* q) {
  float4 x, y;
  ld_rec_nc(rec, x, y);
  mx_unpack(x, y, q);
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
    for (int j = 0; j < 10; ++j) g[j] = pc.region_phi_f[region][j];
  } else if (type == BC_PRESSURE_OUTLET) {
    g[PR] = pc.region_phi_f[region][PR];
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
      if (type == BC_WALL_ISOTHERMAL) g[TT] = pc.region_phi_f[region][TT];
      g[RHO] = g[PR] / (ph.R * g[TT]);
    }
  }
  // prim_to_con (eos.c:120-127)
  g[MX] = g[VU] * g[RHO];
  g[MY] = g[VV] * g[RHO];
  g[MZ] = g[VW] * g[RHO];
  g[EN] = ph.s_km1 * g[PR] + 0.5f * (g[VU] * g[MX] + g[VV] * g[MY] + g[VW] * g[MZ]);
}

// Viscous stresses of a cell (flux.c:223-238: from the gradients of the
// conserved momenta, as the reference computes them).  gm[v*3+d], v: rho_u,
// rho_v, rho_w, T.  tau = (xx, yy, zz, xy, xz, yz).
__device__ __forceinline__ void mx_stress(const float* gm, const MxPhys& ph, float* tau) {
  const float s23 = 2.0f / 3.0f, s43 = 4.0f / 3.0f, mu = ph.mu;
  tau[0] = mu * (s43 * gm[0] - s23 * gm[4] - s23 * gm[8]);
  tau[1] = mu * (-s23 * gm[0] + s43 * gm[4] - s23 * gm[8]);
  tau[2] = mu * (-s23 * gm[0] - s23 * gm[4] + s43 * gm[8]);
  tau[3] = mu * (gm[1] + gm[3]);
  tau[4] = mu * (gm[2] + gm[6]);
  tau[5] = mu * (gm[5] + gm[7]);
}

// viscous normal flux of one side times the area: F_visc . (n A) for the
// momentum and energy rows (flux.c:240-262) with the side's reconstructed
// velocity q[VU..VW] and heat flux k grad T (gT).
__device__ __forceinline__ void mx_viscous(const float* q, const float* tau, const float* gT,
                                           const float* nA, const MxPhys& ph, float* v) {
  const float txx = tau[0], tyy = tau[1], tzz = tau[2], txy = tau[3], txz = tau[4], tyz = tau[5];
  const float k = ph.heat;
  v[0] = -(txx * nA[0] + txy * nA[1] + txz * nA[2]);
  v[1] = -(txy * nA[0] + tyy * nA[1] + tyz * nA[2]);
  v[2] = -(txz * nA[0] + tyz * nA[1] + tzz * nA[2]);
  // (-tau u - k grad T) . nA = u . (-tau nA) - k grad T . nA (tau symmetric)
  v[3] = q[VU] * v[0] + q[VV] * v[1] + q[VW] * v[2] - k * (gT[0] * nA[0] + gT[1] * nA[1] + gT[2] * nA[2]);
}

// min(1, y) * slope of limiter.c:86-106 without the division: slope capped
// by max - q when positive, by min - q when negative, 0 when 0.  The
// cell's own value is part of the neighbourhood min and max, so
// dmn = min - q <= 0 <= max - q = dmx and the clamp is that selection.
__device__ __forceinline__ float bj_limited(float slope, float dmn, float dmx) {
  return fminf(fmaxf(slope, dmn), dmx);
}

template <int MCF>
__device__ __forceinline__ void load_cface(const int* __restrict__ cf, int* e) {
  if (MCF == 4) {
    const int4 v = __ldg(reinterpret_cast<const int4*>(cf));
    e[0] = v.x; e[1] = v.y; e[2] = v.z; e[3] = v.w;
  } else if (MCF % 2 == 0) {
#pragma unroll
    for (int k = 0; k < MCF; k += 2) {
      const int2 v = __ldg(reinterpret_cast<const int2*>(cf) + k / 2);
      e[k] = v.x; e[k + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < MCF; ++k) e[k] = __ldg(cf + k);
  }
}

// ---------------------------------------------------------------------------
// gradient pass
// ---------------------------------------------------------------------------
template <int MCF, int GMODE, bool LINEAR, bool LIMIT, bool VISC>
__global__ void __launch_bounds__(256, FV3D_SIDES_MINBLOCKS) k_mx_sides(const __grid_constant__ MxArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nc) return;
  MxPhys ph;
  ph.load(a.pc);
  float q[10];
  ld_unpack(a.Uf + 8 * (size_t)c, q);
  int e[MCF], o[MCF];
  load_cface<MCF>(a.cface + (size_t)c * MCF, e);
  load_cface<MCF>(a.cnbr + (size_t)c * MCF, o);  // neighbour cell, -1 ghost, -2 none
  float g[NG][3];
#pragma unroll
  for (int v = 0; v < NG; ++v) { g[v][0] = 0.f; g[v][1] = 0.f; g[v][2] = 0.f; }
  float mn[8], mxv[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) { mn[v] = q[v]; mxv[v] = q[v]; }
  if (GMODE != 0) {
#pragma unroll kSidesUnroll
    for (int k = 0; k < MCF; ++k) {
      if (o[k] == -2) continue;
      const int f = e[k] >> 1, side = e[k] & 1;
      const float4 nA = __ldg(&a.slotN[(size_t)c * MCF + k]);
      float qo[10];
      if (o[k] < 0) {
        const float n[3] = {nA.x, nA.y, nA.z};
        mx_ghost(q, a.fregion[f - a.nf_int], n, a.pc, ph, qo);
      } else {
        ld_unpack(a.Uf + 8 * (size_t)o[k], qo);
      }
      if (GMODE == 1) {
        // Green-Gauss (reconstruction.c:43-71) in difference form:
        // s_f mean_f nA_f = s_f q_c nA_f + s_f w_f (q_o - q_c) nA_f with
        // w = lambda (cell 0 side) or 1 - lambda (cell 1 side); the q_c
        // terms are added once per cell through sum_f s_f nA_f below
        const float w = __ldg(&a.slotD[(size_t)c * MCF + k]).w * nA.w;
        const float sw = side ? -w : w;
        const float ax = nA.x * sw, ay = nA.y * sw, az = nA.z * sw;
#pragma unroll
        for (int v = 0; v < NG; ++v) {
          const int j = (v < 8) ? v : TT;
          const float dq = qo[j] - q[j];
          g[v][0] += dq * ax;
          g[v][1] += dq * ay;
          g[v][2] += dq * az;
        }
      } else {
        const float4 wl = __ldg(&a.slotW[(size_t)c * MCF + k]);
#pragma unroll
        for (int v = 0; v < NG; ++v) {
          const int j = (v < 8) ? v : TT;
          const float dq = qo[j] - q[j];
          g[v][0] += wl.x * dq;
          g[v][1] += wl.y * dq;
          g[v][2] += wl.z * dq;
        }
      }
      if (LIMIT) {
#pragma unroll
        for (int v = 0; v < 8; ++v) { mn[v] = fminf(mn[v], qo[v]); mxv[v] = fmaxf(mxv[v], qo[v]); }
      }
    }
    if (GMODE == 1) {
      const float4 cg = __ldg(&a.cgeo[c]);
#pragma unroll
      for (int v = 0; v < NG; ++v) {
        const int j = (v < 8) ? v : TT;
        g[v][0] = (g[v][0] + q[j] * cg.x) * cg.w;
        g[v][1] = (g[v][1] + q[j] * cg.y) * cg.w;
        g[v][2] = (g[v][2] + q[j] * cg.z) * cg.w;
      }
    }
  }
  float tau[6];
  if (VISC) {
    float gm[12];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      gm[d] = g[1][d]; gm[3 + d] = g[2][d]; gm[6 + d] = g[3][d]; gm[9 + d] = g[8][d];
    }
    mx_stress(gm, ph, tau);
  }
  // per face side: limited reconstruction + viscous flux
#pragma unroll
  for (int k = 0; k < MCF; ++k) {
    if (o[k] == -2) continue;
    const int f = e[k] >> 1, side = e[k] & 1;
    const float4 nA4 = __ldg(&a.slotN[(size_t)c * MCF + k]);
    const float nA[3] = {nA4.x * nA4.w, nA4.y * nA4.w, nA4.z * nA4.w};
    float r[12];
    if (LINEAR) {
      const float4 d = __ldg(&a.slotD[(size_t)c * MCF + k]);
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const float slope = d.x * g[v][0] + d.y * g[v][1] + d.z * g[v][2];
        float inc = slope;
        if (LIMIT) inc = bj_limited(slope, mn[v] - q[v], mxv[v] - q[v]);
        r[v] = q[v] + inc;
      }
    } else {
#pragma unroll
      for (int v = 0; v < 8; ++v) r[v] = q[v];
    }
    if (VISC) mx_viscous(r, tau, g[8], nA, ph, &r[8]);
    (void)side;
    const size_t own = (size_t)k * a.ncp + c;  // this side, slot-major
    st_rec(a.fs + own * 8, make_float4(r[0], r[1], r[2], r[3]),
           VISC ? make_float4(r[4], r[8], r[9], r[10]) : make_float4(r[4], 0.f, 0.f, 0.f));
    if (VISC) a.fsv[own] = r[11];
    if (o[k] == -1) {
      const size_t gi = (size_t)MCF * a.ncp + (f - a.nf_int);  // the ghost side's record
      // ghost side: unlimited ghost of the cell-centre state
      // (reconstruction.c:249-253), gradient = interior gradient with the
      // normal part removed on slip walls / symmetry (boundary.c:377-405)
      const int region = a.fregion[f - a.nf_int];
      const float n[3] = {nA4.x, nA4.y, nA4.z};
      float gq[10];
      mx_ghost(q, region, n, a.pc, ph, gq);
      float vg[4] = {0.f, 0.f, 0.f, 0.f};
      if (VISC) {
        const int type = a.pc.region_type[region];
        float tg[6], gT[3] = {g[8][0], g[8][1], g[8][2]};
#pragma unroll
        for (int j = 0; j < 6; ++j) tg[j] = tau[j];
        if (type == BC_WALL_SLIP || type == BC_SYMMETRY) {
          // ghost gradient without its normal part (boundary.c:377-405)
          float gm[12];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            gm[d] = g[1][d]; gm[3 + d] = g[2][d]; gm[6 + d] = g[3][d]; gm[9 + d] = g[8][d];
          }
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const float gn = gm[3 * v] * n[0] + gm[3 * v + 1] * n[1] + gm[3 * v + 2] * n[2];
            gm[3 * v] -= gn * n[0]; gm[3 * v + 1] -= gn * n[1]; gm[3 * v + 2] -= gn * n[2];
          }
          mx_stress(gm, ph, tg);
          gT[0] = gm[9]; gT[1] = gm[10]; gT[2] = gm[11];
        }
        mx_viscous(gq, tg, gT, nA, ph, vg);
        a.fsv[gi] = vg[3];
      }
      st_rec(a.fs + gi * 8, make_float4(gq[0], gq[1], gq[2], gq[3]), make_float4(gq[4], vg[0], vg[1], vg[2]));
    }
  }
}

// ---------------------------------------------------------------------------
// flux + update pass
// ---------------------------------------------------------------------------
// convective face flux in the global frame, times A.  l, r: (rho, m, E)
__device__ __forceinline__ void mx_conv_flux(const float* l, const float* r, const float4 nA,
                                             const MxPhys& ph, float* F) {
  const float n0 = nA.x, n1 = nA.y, n2 = nA.z, A = nA.w;
  // primitives of the (reconstructed) conserved states (eos.c:81-92)
  const float irl = 1.f / l[0], irr = 1.f / r[0];
  const float ul = l[1] * irl, vl = l[2] * irl, wl = l[3] * irl;
  const float ur = r[1] * irr, vr = r[2] * irr, wr = r[3] * irr;
  const float pl = fmaxf(1.00E-10f, ph.km1 * (l[4] - 0.5f * (l[1] * ul + l[2] * vl + l[3] * wl)));
  const float pr = fmaxf(1.00E-10f, ph.km1 * (r[4] - 0.5f * (r[1] * ur + r[2] * vr + r[3] * wr)));
  const float unl = ul * n0 + vl * n1 + wl * n2;
  const float unr = ur * n0 + vr * n1 + wr * n2;
  const float cl = sqrtf(ph.kappa * pl * irl), cr = sqrtf(ph.kappa * pr * irr);
  if (ph.flux == 1) {  // Rusanov, flux.c:320-336
    const float lam = fmaxf(fabsf(unl) + cl, fabsf(unr) + cr);
    const float ml = l[0] * unl, mr = r[0] * unr;
    F[0] = 0.5f * (ml + mr) - 0.5f * lam * (r[0] - l[0]);
    F[1] = 0.5f * (l[1] * unl + pl * n0 + r[1] * unr + pr * n0) - 0.5f * lam * (r[1] - l[1]);
    F[2] = 0.5f * (l[2] * unl + pl * n1 + r[2] * unr + pr * n1) - 0.5f * lam * (r[2] - l[2]);
    F[3] = 0.5f * (l[3] * unl + pl * n2 + r[3] * unr + pr * n2) - 0.5f * lam * (r[3] - l[3]);
    F[4] = 0.5f * ((l[4] + pl) * unl + (r[4] + pr) * unr) - 0.5f * lam * (r[4] - l[4]);
  } else {  // AUSM, flux.c:344-406
    const float Ml = unl / cl, Mr = unr / cr;
    float mp, pp, mm, pm;
    if (Ml <= -1.f) { mp = 0.f; pp = 0.f; }
    else if (Ml < 1.f) { mp = 0.25f * (Ml + 1.f) * (Ml + 1.f); pp = 0.25f * pl * (1.f + Ml) * (1.f + Ml) * (2.f - Ml); }
    else { mp = Ml; pp = pl; }
    if (Mr <= -1.f) { mm = Mr; pm = pr; }
    else if (Mr < 1.f) { mm = -0.25f * (Mr - 1.f) * (Mr - 1.f); pm = 0.25f * pr * (1.f - Mr) * (1.f - Mr) * (2.f + Mr); }
    else { mm = 0.f; pm = 0.f; }
    const float mdl = fmaxf(0.f, mp + mm) * cl * l[0];
    const float mdr = fminf(0.f, mp + mm) * cr * r[0];
    const float P = pp + pm;
    F[0] = mdl + mdr;
    F[1] = mdl * ul + mdr * ur + P * n0;
    F[2] = mdl * vl + mdr * vr + P * n1;
    F[3] = mdl * wl + mdr * wr + P * n2;
    F[4] = mdl * (l[4] + pl) * irl + mdr * (r[4] + pr) * irr;
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) F[j] *= A;
}

// FP32 stage state record from conserved floats
__device__ __forceinline__ void mx_make_state(float rho, float mx, float my, float mz, float E,
                                              const MxPhys& ph, float4& x, float4& y) {
  const float ir = 1.f / rho;
  const float ke = 0.5f * (mx * mx + my * my + mz * mz) * ir;
  const float p = fmaxf(1.00E-10f, ph.km1 * (E - ke));
  x = make_float4(rho, mx, my, mz);
  y = make_float4(E, p, p * ir / ph.R, ir);
}

// one face of a cell in the flux pass: the convective flux from both side
// records (this cell's m, the other side's o) plus the averaged viscous
// flux (the sides' viscous energy fluxes vm, vo), with this cell's sign
template <bool VISC>
__device__ __forceinline__ void mx_face_signed(const float4 m0, const float4 m1, const float4 o0, const float4 o1,
                                               const float4 nA, const float vm, const float vo, const int side,
                                               const MxPhys& ph, float* out) {
  // cell 0's side left, cell 1's right: both cells evaluate the face
  // from the same operands in the same order
  const float4 l0 = side ? o0 : m0, l1 = side ? o1 : m1;
  const float4 r0 = side ? m0 : o0, r1 = side ? m1 : o1;
  const float l[5] = {l0.x, l0.y, l0.z, l0.w, l1.x};
  const float r[5] = {r0.x, r0.y, r0.z, r0.w, r1.x};
  float F[5];
  mx_conv_flux(l, r, nA, ph, F);
  if (VISC) {
    const float2 ve = side ? make_float2(vo, vm) : make_float2(vm, vo);
    F[1] += 0.5f * (l1.y + r1.y);
    F[2] += 0.5f * (l1.z + r1.z);
    F[3] += 0.5f * (l1.w + r1.w);
    F[4] += 0.5f * (ve.x + ve.y);
  }
  // the second cell takes the flux with the opposite sign (sub(x) is
  // add(-x)): a select, not a divergent branch
  const float sg = side ? -1.f : 1.f;
#pragma unroll
  for (int j = 0; j < 5; ++j) out[j] = sg * F[j];
}

// slot k of cell c with both side records in global memory (the own side
// at k * ncp + c, the other side at e >> 1), added to s
template <bool VISC>
__device__ __forceinline__ void mx_face_global(const MxArgs& a, const MxPhys& ph, int k, int c, int e,
                                               Acc<float, kFluxKahan>* s) {
  const size_t own = (size_t)k * a.ncp + c, oth = (size_t)(e >> 1);
  float4 m0, m1, o0, o1;
  ld_rec_nc(a.fs + own * 8, m0, m1);  // this cell's side (a warp's loads contiguous)
  ld_rec_nc(a.fs + oth * 8, o0, o1);  // the other side
  const float4 nA = __ldg(&a.slotNk[own]);
  float vm = 0.f, vo = 0.f;
  if (VISC) { vm = __ldg(a.fsv + own); vo = __ldg(a.fsv + oth); }
  float F[5];
  mx_face_signed<VISC>(m0, m1, o0, o1, nA, vm, vo, e & 1, ph, F);
#pragma unroll
  for (int j = 0; j < 5; ++j) s[j].add(F[j]);
}

// the rest of the flux + update pass for cell c once its face sums s are
// complete: -sum/V, the RK update, the FP32 stage record and (DT) the
// cell's time-step bound
template <int MODE, bool DT, bool STORE>
__device__ __forceinline__ void mx_update_cell(const MxArgs& a, const StageCoef& co, const MxPhys& ph, const int c,
                                               const Acc<float, kFluxKahan>* s, unsigned long long& lam_bits,
                                               bool& finite) {
  const float rv = __ldg(&a.cgeo[c]).w;
  float rr[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) rr[j] = -s[j].value() * rv;
  if (MODE == 0 || STORE) {
#pragma unroll
    for (int j = 0; j < 5; ++j) a.dphi[(size_t)j * a.nc + c] = (double)rr[j];
  }
  if (MODE != 0) {
    const double dt = a.sc->dt;
    float du[5];
    if (MODE == 1) {
      const float gdt = (float)(dt * co.g);
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const size_t i = (size_t)j * a.ncp + c;
        const float kj = co.first ? rr[j] : fmaf(a.kf[i], (float)co.a, rr[j]);
        if (!co.last) a.kf[i] = kj;
        du[j] = co.first ? gdt * kj : fmaf(gdt, kj, a.dU[i]);
      }
    } else {
      const float fdt = (float)dt, c1 = (float)co.c1;
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const size_t i = (size_t)j * a.ncp + c;
        du[j] = co.first ? fdt * rr[j] : c1 * fmaf(fdt, rr[j], a.dU[i]);
      }
    }
    float* sh = a.Uf + 8 * (size_t)c;
    float4 o0 = make_float4(0.f, 0.f, 0.f, 0.f), o1 = o0;
    if (DT && MODE == 1) ld_rec(sh, o0, o1);  // stage-input state
    float un[5];
    if (co.last) {
      // end of step: U_{n+1} = U_n + dU in FP64, new base record
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const size_t i = (size_t)j * a.nc + c;
        const double uj = a.U[i] + (double)du[j];
        a.U[i] = uj;
        un[j] = (float)uj;
        finite = finite && isfinite(uj);
      }
      float4 x, y;
      mx_make_state(un[0], un[1], un[2], un[3], un[4], ph, x, y);
      st_rec(a.UfN + 8 * (size_t)c, x, y);
      st_rec(sh, x, y);
    } else {
      float4 b0, b1;
      ld_rec_nc(a.UfN + 8 * (size_t)c, b0, b1);
      un[0] = b0.x + du[0]; un[1] = b0.y + du[1]; un[2] = b0.z + du[2]; un[3] = b0.w + du[3];
      un[4] = b1.x + du[4];
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        a.dU[(size_t)j * a.ncp + c] = du[j];
        finite = finite && isfinite(du[j]);
      }
      float4 x, y;
      mx_make_state(un[0], un[1], un[2], un[3], un[4], ph, x, y);
      st_rec(sh, x, y);
    }
    if (DT) {
      // calc_ns_timestep on the reference's phi_total: new density, the
      // stage-input u, v, w, p for the low-storage schemes (see
      // k_gather_update); new state for SSP-RK3
      const float ir = 1.f / un[0];
      float pu = un[1] * ir, pv = un[2] * ir, pw = un[3] * ir;
      float pp = fmaxf(1.00E-10f, ph.km1 * (un[4] - 0.5f * (un[1] * pu + un[2] * pv + un[3] * pw)));
      if (MODE == 1) {
        const float io = o1.w;  // 1 / rho of the stage-input record
        pu = o0.y * io; pv = o0.z * io; pw = o0.w * io; pp = o1.y;
      }
      const float cs = sqrtf(ph.kappa * pp * ir);
      const float4 dxv = __ldg(&a.cdx[c]);
      const float ds = (fabsf(pu) + cs) * dxv.x + (fabsf(pv) + cs) * dxv.y + (fabsf(pw) + cs) * dxv.z;
      const double lam = (double)(dxv.w / ds);
      if (lam > 0.0) lam_bits = (unsigned long long)__double_as_longlong(lam);
    }
  }
}

// MODE 0: residual only; 1: low-storage RK stage; 2: SSP-RK3 stage.
// co.first / co.last mark the step's first and last stage.
// STORE: also store the stage's time derivative in dphi (co.store_r; a
// template flag: a run-time test of it costs the hot instantiations 2 %)
// resident blocks: 5 (48 registers) for 4 face slots, where the gathers
// need the warps (-4 % per stage); wider cells keep their registers
template <int MCF, int MODE, bool DT, bool VISC, bool STORE = false>
__global__ void __launch_bounds__(256, MCF == 4 ? FV3D_FLUX4_MINBLOCKS : FV3D_FLUX_MINBLOCKS)
    k_mx_flux_update(const __grid_constant__ MxArgs a, StageCoef co) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long lam_bits = 0x7ff0000000000000ull;
  bool finite = true;
  if (c < a.nc) {
    MxPhys ph;
    ph.load(a.pc);
    int e[MCF];
    load_cface<MCF>(a.cother + (size_t)c * MCF, e);
    // compensated FP32 sums in slot order (ascending reference face id):
    // at 5 resident blocks of the 4-face kernel (48 registers, about 120 B
    // spilled) they cost 1.5 % of a stage over plain sums, and they change
    // the state after 500 steps by nothing measurable (the faces' FP32
    // arithmetic dominates the error)
    Acc<float, kFluxKahan> s[5];
#pragma unroll kFluxUnroll
    for (int k = 0; k < MCF; ++k)
      if (e[k] >= 0) mx_face_global<VISC>(a, ph, k, c, e[k], s);
    mx_update_cell<MODE, DT, STORE>(a, co, ph, c, s, lam_bits, finite);
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

// ---------------------------------------------------------------------------
// gradient pass staged through shared memory.  Each CTA handles one tile of
// kTile consecutive cells (one thread per cell).  One elected thread issues
// bulk asynchronous copies (cp.async.bulk, the TMA unit) of the tile's
// contiguous per-cell data - state records, face slots, neighbours, cell
// geometry and the slot-major face geometry - into shared memory, completing
// on one mbarrier; the bytes in flight no longer occupy registers.  The
// arithmetic is that of k_mx_sides, operation for operation, so the face
// records are bitwise the same.  Neighbour states are gathered from global
// memory as before.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// global -> shared bulk copy; both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// wait for a phase with a time limit; false if it did not complete in time
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

// a cell's MCF face-slot ints from the shared-memory tile (plain shared
// loads: the read-only global path of load_cface must not see shared addresses)
template <int MCF>
__device__ __forceinline__ void load_slots_shared(const int* cf, int* e) {
  if (MCF == 4) {
    const int4 v = *reinterpret_cast<const int4*>(cf);
    e[0] = v.x; e[1] = v.y; e[2] = v.z; e[3] = v.w;
  } else if (MCF % 2 == 0) {
#pragma unroll
    for (int k = 0; k < MCF; k += 2) {
      const int2 v = reinterpret_cast<const int2*>(cf)[k / 2];
      e[k] = v.x; e[k + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < MCF; ++k) e[k] = cf[k];
  }
}

// shared-memory tile: byte offsets (all multiples of 16)
template <int MCF, int GMODE, int TL = kTile>
struct SidesTile {
  static constexpr int uf = 0;                                    // float [TL][8]
  static constexpr int cf = uf + TL * 32;                         // int [TL][MCF]
  static constexpr int cn = cf + TL * MCF * 4;                    // int [TL][MCF]
  static constexpr int cg = cn + TL * MCF * 4;                    // float4 [TL]
  static constexpr int sn = cg + TL * 16;                         // float4 [MCF][TL]
  static constexpr int sd = sn + MCF * TL * 16;                   // float4 [MCF][TL]
  static constexpr int sw = sd + MCF * TL * 16;                   // float4 [MCF][TL] (LSQ)
  static constexpr int bytes = sw + (GMODE == 2 ? MCF * TL * 16 : 0);
  static constexpr int bar = bytes;                               // mbarrier (8 bytes)
  static constexpr int total = bytes + 16;
};

// status bit set when a tile's copies did not arrive within the time limit
constexpr int kStatusStageTimeout = 4;

// one tile of the staged gradient pass, from the tile in shared memory
// (layout SidesTile) for the cell c0 + tid: the arithmetic of k_mx_sides
template <int MCF, int GMODE, bool LINEAR, bool LIMIT, bool VISC, int TL = kTile>
__device__ __forceinline__ void sides_tile(const MxArgs& a, const unsigned char* smem, int c0, int tid) {
  using L = SidesTile<MCF, GMODE, TL>;
  const int c = c0 + tid;
  if (c >= a.nc) return;
  MxPhys ph;
  ph.load(a.pc);
  const float4* sUf = reinterpret_cast<const float4*>(smem + L::uf);
  const float4* sN = reinterpret_cast<const float4*>(smem + L::sn);
  const float4* sD = reinterpret_cast<const float4*>(smem + L::sd);
  const float4* sW = reinterpret_cast<const float4*>(smem + L::sw);
  float q[10];
  mx_unpack(sUf[2 * tid], sUf[2 * tid + 1], q);
  int e[MCF], o[MCF];
  load_slots_shared<MCF>(reinterpret_cast<const int*>(smem + L::cf) + tid * MCF, e);
  load_slots_shared<MCF>(reinterpret_cast<const int*>(smem + L::cn) + tid * MCF, o);
  float g[NG][3];
#pragma unroll
  for (int v = 0; v < NG; ++v) { g[v][0] = 0.f; g[v][1] = 0.f; g[v][2] = 0.f; }
  float mn[8], mxv[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) { mn[v] = q[v]; mxv[v] = q[v]; }
#pragma unroll kSidesUnroll
  for (int k = 0; k < MCF; ++k) {
    if (o[k] == -2) continue;
    const int f = e[k] >> 1, side = e[k] & 1;
    const float4 nA = sN[k * TL + tid];
    float qo[10];
    if (o[k] < 0) {
      const float n[3] = {nA.x, nA.y, nA.z};
      mx_ghost(q, a.fregion[f - a.nf_int], n, a.pc, ph, qo);
    } else {
      // a neighbour inside this tile is already in shared memory
      const unsigned lo = (unsigned)(o[k] - c0);
      if (lo < (unsigned)TL) mx_unpack(sUf[2 * lo], sUf[2 * lo + 1], qo);
      else ld_unpack(a.Uf + 8 * (size_t)o[k], qo);
    }
    if (GMODE == 1) {
      const float w = sD[k * TL + tid].w * nA.w;
      const float sw = side ? -w : w;
      const float ax = nA.x * sw, ay = nA.y * sw, az = nA.z * sw;
#pragma unroll
      for (int v = 0; v < NG; ++v) {
        const int j = (v < 8) ? v : TT;
        const float dq = qo[j] - q[j];
        g[v][0] += dq * ax;
        g[v][1] += dq * ay;
        g[v][2] += dq * az;
      }
    } else {
      const float4 wl = sW[k * TL + tid];
#pragma unroll
      for (int v = 0; v < NG; ++v) {
        const int j = (v < 8) ? v : TT;
        const float dq = qo[j] - q[j];
        g[v][0] += wl.x * dq;
        g[v][1] += wl.y * dq;
        g[v][2] += wl.z * dq;
      }
    }
    if (LIMIT) {
#pragma unroll
      for (int v = 0; v < 8; ++v) { mn[v] = fminf(mn[v], qo[v]); mxv[v] = fmaxf(mxv[v], qo[v]); }
    }
  }
  if (GMODE == 1) {
    const float4 cg = reinterpret_cast<const float4*>(smem + L::cg)[tid];
#pragma unroll
    for (int v = 0; v < NG; ++v) {
      const int j = (v < 8) ? v : TT;
      g[v][0] = (g[v][0] + q[j] * cg.x) * cg.w;
      g[v][1] = (g[v][1] + q[j] * cg.y) * cg.w;
      g[v][2] = (g[v][2] + q[j] * cg.z) * cg.w;
    }
  }
  float tau[6];
  if (VISC) {
    float gm[12];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      gm[d] = g[1][d]; gm[3 + d] = g[2][d]; gm[6 + d] = g[3][d]; gm[9 + d] = g[8][d];
    }
    mx_stress(gm, ph, tau);
  }
#pragma unroll
  for (int k = 0; k < MCF; ++k) {
    if (o[k] == -2) continue;
    const int f = e[k] >> 1, side = e[k] & 1;
    const float4 nA4 = sN[k * TL + tid];
    const float nA[3] = {nA4.x * nA4.w, nA4.y * nA4.w, nA4.z * nA4.w};
    float r[12];
    if (LINEAR) {
      const float4 d = sD[k * TL + tid];
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const float slope = d.x * g[v][0] + d.y * g[v][1] + d.z * g[v][2];
        float inc = slope;
        if (LIMIT) inc = bj_limited(slope, mn[v] - q[v], mxv[v] - q[v]);
        r[v] = q[v] + inc;
      }
    } else {
#pragma unroll
      for (int v = 0; v < 8; ++v) r[v] = q[v];
    }
    if (VISC) mx_viscous(r, tau, g[8], nA, ph, &r[8]);
    (void)side;
    const size_t own = (size_t)k * a.ncp + c;  // this side, slot-major
    st_rec(a.fs + own * 8, make_float4(r[0], r[1], r[2], r[3]),
           VISC ? make_float4(r[4], r[8], r[9], r[10]) : make_float4(r[4], 0.f, 0.f, 0.f));
    if (VISC) a.fsv[own] = r[11];
    if (o[k] == -1) {  // ghost side, as in k_mx_sides
      const size_t gi = (size_t)MCF * a.ncp + (f - a.nf_int);
      const int region = a.fregion[f - a.nf_int];
      const float n[3] = {nA4.x, nA4.y, nA4.z};
      float gq[10];
      mx_ghost(q, region, n, a.pc, ph, gq);
      float vg[4] = {0.f, 0.f, 0.f, 0.f};
      if (VISC) {
        const int type = a.pc.region_type[region];
        float tg[6], gT[3] = {g[8][0], g[8][1], g[8][2]};
#pragma unroll
        for (int j = 0; j < 6; ++j) tg[j] = tau[j];
        if (type == BC_WALL_SLIP || type == BC_SYMMETRY) {
          float gm[12];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            gm[d] = g[1][d]; gm[3 + d] = g[2][d]; gm[6 + d] = g[3][d]; gm[9 + d] = g[8][d];
          }
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const float gn = gm[3 * v] * n[0] + gm[3 * v + 1] * n[1] + gm[3 * v + 2] * n[2];
            gm[3 * v] -= gn * n[0]; gm[3 * v + 1] -= gn * n[1]; gm[3 * v + 2] -= gn * n[2];
          }
          mx_stress(gm, ph, tg);
          gT[0] = gm[9]; gT[1] = gm[10]; gT[2] = gm[11];
        }
        mx_viscous(gq, tg, gT, nA, ph, vg);
        a.fsv[gi] = vg[3];
      }
      st_rec(a.fs + gi * 8, make_float4(gq[0], gq[1], gq[2], gq[3]), make_float4(gq[4], vg[0], vg[1], vg[2]));
    }
  }
}

template <int MCF, int GMODE, bool LINEAR, bool LIMIT, bool VISC, int TL = kTile>
__global__ void __launch_bounds__(TL, FV3D_TMA_MINBLOCKS) k_mx_sides_tma(const __grid_constant__ MxArgs a) {
  static_assert(GMODE != 0, "the staged gradient pass needs gradients");
  using L = SidesTile<MCF, GMODE, TL>;
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x;
  const int c0 = blockIdx.x * TL;
  const uint32_t bar = smem_u32(smem + L::bar);
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(bar, L::bytes);
    const uint32_t s0 = smem_u32(smem);
    bulk_g2s(s0 + L::uf, a.Uf + 8 * (size_t)c0, TL * 32, bar);
    bulk_g2s(s0 + L::cf, a.cface + (size_t)c0 * MCF, TL * MCF * 4, bar);
    bulk_g2s(s0 + L::cn, a.cnbr + (size_t)c0 * MCF, TL * MCF * 4, bar);
    bulk_g2s(s0 + L::cg, a.cgeo + c0, TL * 16, bar);
#pragma unroll
    for (int k = 0; k < MCF; ++k) {
      bulk_g2s(s0 + L::sn + k * TL * 16, a.slotNk + (size_t)k * a.ncp + c0, TL * 16, bar);
      bulk_g2s(s0 + L::sd + k * TL * 16, a.slotDk + (size_t)k * a.ncp + c0, TL * 16, bar);
      if (GMODE == 2) bulk_g2s(s0 + L::sw + k * TL * 16, a.slotWk + (size_t)k * a.ncp + c0, TL * 16, bar);
    }
  }
  if (!mbar_wait_bounded(bar, 0, 500000000ull)) {
    // the copies did not land in 0.5 s: report, give them one more bounded
    // wait so that none is still writing this CTA's shared memory, return
    if (tid == 0) atomicOr(&a.sc->status, kStatusStageTimeout);
    mbar_wait_bounded(bar, 0, 500000000ull);
    return;
  }
  sides_tile<MCF, GMODE, LINEAR, LIMIT, VISC, TL>(a, smem, c0, tid);
}

// ---------------------------------------------------------------------------
// persistent form of the staged gradient pass: each CTA walks the tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... with two tile buffers; the bulk
// copies of its next tile are in flight while it computes the current one.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <int MCF, int GMODE>
__device__ __forceinline__ void sides_issue(const MxArgs& a, uint32_t s0, uint32_t bar, int c0) {
  using L = SidesTile<MCF, GMODE>;
  mbar_expect_tx(bar, L::bytes);
  bulk_g2s(s0 + L::uf, a.Uf + 8 * (size_t)c0, kTile * 32, bar);
  bulk_g2s(s0 + L::cf, a.cface + (size_t)c0 * MCF, kTile * MCF * 4, bar);
  bulk_g2s(s0 + L::cn, a.cnbr + (size_t)c0 * MCF, kTile * MCF * 4, bar);
  bulk_g2s(s0 + L::cg, a.cgeo + c0, kTile * 16, bar);
#pragma unroll
  for (int k = 0; k < MCF; ++k) {
    bulk_g2s(s0 + L::sn + k * kTile * 16, a.slotNk + (size_t)k * a.ncp + c0, kTile * 16, bar);
    bulk_g2s(s0 + L::sd + k * kTile * 16, a.slotDk + (size_t)k * a.ncp + c0, kTile * 16, bar);
    if (GMODE == 2) bulk_g2s(s0 + L::sw + k * kTile * 16, a.slotWk + (size_t)k * a.ncp + c0, kTile * 16, bar);
  }
}

// bytes between the two tile buffers (each ends with its mbarrier)
template <int MCF, int GMODE>
constexpr int sides_buf_stride() {
  return (SidesTile<MCF, GMODE>::total + 127) / 128 * 128;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// persistent staged gradient pass without CTA barriers in the tile loop:
// each buffer has a "full" mbarrier (the bulk copies' transaction count)
// and an "empty" one (one arrival per warp after its last read of the
// tile); only the issuing thread waits for the slowest warp, before it
// refills a buffer.  Every wait is bounded; a thread that gives up records
// kStatusStageTimeout, waits (bounded) for the copies of both buffers and
// leaves.
template <int MCF, int GMODE, bool LINEAR, bool LIMIT, bool VISC>
__global__ void __launch_bounds__(kTile) k_mx_sides_tma2(const __grid_constant__ MxArgs a) {
  static_assert(GMODE != 0, "the staged gradient pass needs gradients");
  using L = SidesTile<MCF, GMODE>;
  constexpr int BUF = sides_buf_stride<MCF, GMODE>();
  constexpr int kWarps = kTile / 32;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long empty_bar[2];
  const int tid = threadIdx.x;
  const int ntiles = a.ncp / kTile;
  int t = blockIdx.x;
  if (t >= ntiles) return;  // whole CTA
  const uint32_t s0 = smem_u32(smem);
  const uint32_t full0 = s0 + L::bar, full1 = s0 + BUF + L::bar;
  const uint32_t empty0 = smem_u32(&empty_bar[0]), empty1 = smem_u32(&empty_bar[1]);
  if (tid == 0) {
    mbar_init(full0, 1);
    mbar_init(full1, 1);
    mbar_init(empty0, kWarps);
    mbar_init(empty1, kWarps);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) sides_issue<MCF, GMODE>(a, s0, full0, t * kTile);
  constexpr unsigned long long kLimit = 500000000ull;
  for (int i = 0; t < ntiles; ++i, t += gridDim.x) {
    const int b = i & 1;
    const int tn = t + gridDim.x;
    const uint32_t full = b ? full1 : full0, full_next = b ? full0 : full1;
    bool ok = true;
    if (tid == 0 && tn < ntiles) {
      // buffer b^1 held tile i - 1: every warp has arrived on its empty
      // barrier after reading it
      if (i >= 1) ok = mbar_wait_bounded(b ? empty0 : empty1, ((i - 1) >> 1) & 1, kLimit);
      if (ok) {
        fence_proxy_async_smem();
        sides_issue<MCF, GMODE>(a, s0 + (b ^ 1) * BUF, full_next, tn * kTile);
      }
    }
    if (ok) ok = mbar_wait_bounded(full, (i >> 1) & 1, kLimit);
    if (!ok) {
      // no copy may outlive the CTA's shared memory: wait (bounded) for this
      // tile's and, when it was due, the next tile's
      atomicOr(&a.sc->status, kStatusStageTimeout);
      mbar_wait_bounded(full, (i >> 1) & 1, kLimit);
      if (tn < ntiles) mbar_wait_bounded(full_next, ((i + 1) >> 1) & 1, kLimit);
      return;
    }
    sides_tile<MCF, GMODE, LINEAR, LIMIT, VISC>(a, smem + b * BUF, t * kTile, tid);
    __syncwarp();
    if ((tid & 31) == 0) mbar_arrive(b ? empty1 : empty0);
  }
}

}  // namespace fv3d
