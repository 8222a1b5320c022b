// Cell-coupling preconditioner of the implicit steady solve (sm_103a).
//
// The Newton system of the pseudo-transient solve is (I/dt - dR/dU) x = R,
// R the second-order viscous residual.  Block Jacobi (one 5x5 block per
// cell) cannot carry information between cells, which is what limits this
// solve; this preconditioner approximates the whole system by the Jacobian of
// the first-order inviscid residual R1 (cell-centre face states, the case's
// own flux: AUSM or Rusanov, flux.c:320-406):
//
//   P_A = I/dt - dR1/dU,   block (c, c) and one block per face slot of c
//
// and applies z = M v as a short inner flexible GMRES on P_A from x = 0 (a
// fixed number of iterations; each direction t_j = M_R v_j is kept and
// z = sum_j y_j t_j), right-preconditioned by damped block-Jacobi sweeps M_R
// of the first-order Rusanov Jacobian with the wave speed frozen,
//
//   P_R = I/dt + (1/V_c) sum_f s_f A_f dF_f/dU,   dF/dU_0 = (A(U_0) + lam I) / 2,
//                                                dF/dU_1 = (A(U_1) - lam I) / 2,
//
// lam = max(|u.n| + c) + 2 mu / (rho d) (A(U) the Euler flux Jacobian along
// n; at a boundary face the ghost's dependence on its cell is included),
// whose sweeps converge where sweeps on P_A diverge.  The outer solve is
// flexible GMRES, so the inner solve may differ from one application to the
// next without changing the answer.
//
// Both operators are applied matrix-free.  P_A x is the exact derivative of
// each face's first-order flux along (x_c, x_o), evaluated in FP32 by
// hand-written forward-mode arithmetic from per-cell FP32 state records and
// per-slot (normal, s A / V); at a boundary face the ghost's tangent is
// G x_c, G = d ghost / d U_c by forward differences of update_boundaries in
// FP64.  P_R's slot blocks are a A(U_o) + b I (per slot the normal and a, b;
// per cell (u, v, w, H)); its diagonal blocks are built in FP64, inverted and
// stored FP32, row-major within a block, element-major over cells ([e][nc]: a
// warp's loads of element e are contiguous).  Every product and sweep is a
// cell gather: no atomics, no face buffers.  The inner Krylov basis, its
// Gram-Schmidt passes, the sweeps and the inner least-squares problem run in
// FP32 on the device, so an application needs no host synchronisation and is
// captured in the outer Arnoldi step's CUDA graph.
#include <algorithm>
#include <cmath>
#include <vector>

#include "context.h"
#include "block5.cuh"
#include "fo_flux.cuh"
#include "implicit.h"

namespace fv3d {

namespace {

inline int nblk(size_t n, int t = 256) { return (int)((n + t - 1) / t); }
constexpr int kHcol = 72;  // per inner column: h [0, 32), |w - V h| and its inverse at 64, 65

// neighbour of each face slot: the other cell (>= 0), -2 - b for boundary
// face b (nf_int + b), -1 for an unused slot
__global__ void k_cpl_nbr(int nc, int mcf, int nf_int, const int* __restrict__ cface, const int* __restrict__ fc0,
                          const int* __restrict__ fc1, int* __restrict__ nbr) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int k = 0; k < mcf; ++k) {
    const int e = cface[(size_t)c * mcf + k];
    int o = -1;
    if (e >= 0) {
      const int f = e >> 1;
      o = (f >= nf_int) ? -2 - (f - nf_int) : ((e & 1) ? fc0[f] : fc1[f]);
    }
    nbr[(size_t)k * nc + c] = o;
  }
}

// Euler flux Jacobian d(F.n)/dU (row-major) of a conserved state, with
// |u.n| + c and rho
__device__ __forceinline__ void euler_jacobian(const double* U, const double* n, double kappa, double* A,
                                               double* lam) {
  const double rho = U[0], ir = 1.0 / rho;
  const double u[3] = {U[1] * ir, U[2] * ir, U[3] * ir};
  const double q2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double p = (kappa - 1.0) * (U[4] - 0.5 * rho * q2);
  const double H = (U[4] + p) * ir;
  const double un = u[0] * n[0] + u[1] * n[1] + u[2] * n[2];
  const double phi = 0.5 * (kappa - 1.0) * q2;
  A[0] = 0.0;
  A[1] = n[0]; A[2] = n[1]; A[3] = n[2];
  A[4] = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    A[(1 + i) * 5] = phi * n[i] - u[i] * un;
#pragma unroll
    for (int j = 0; j < 3; ++j)
      A[(1 + i) * 5 + 1 + j] = u[i] * n[j] - (kappa - 1.0) * u[j] * n[i] + (i == j ? un : 0.0);
    A[(1 + i) * 5 + 4] = (kappa - 1.0) * n[i];
  }
  A[20] = un * (phi - H);
#pragma unroll
  for (int j = 0; j < 3; ++j) A[21 + j] = H * n[j] - (kappa - 1.0) * u[j] * un;
  A[24] = kappa * un;
  *lam = fabs(un) + sqrt(kappa * fmax(p, 1.00E-10) * ir);
}

// |u.n| + c of a conserved state (euler_jacobian's lam, the same arithmetic)
__device__ __forceinline__ double wave_speed(const double* U, const double* n, double kappa) {
  const double rho = U[0], ir = 1.0 / rho;
  const double u[3] = {U[1] * ir, U[2] * ir, U[3] * ir};
  const double q2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double p = (kappa - 1.0) * (U[4] - 0.5 * rho * q2);
  const double un = u[0] * n[0] + u[1] * n[1] + u[2] * n[2];
  return fabs(un) + sqrt(kappa * fmax(p, 1.00E-10) * ir);
}

__device__ __forceinline__ void store_block(float* __restrict__ dst, size_t nc, const double* B) {
#pragma unroll
  for (int e = 0; e < 25; ++e) dst[(size_t)e * nc] = (float)B[e];
}

// the face's geometry for the first-order fluxes: n (cell 0 -> cell 1) and,
// in n[3], the distance |d1| + |d2| (interior) or 2 |d1| (boundary)
__device__ __forceinline__ void face_normal(const double* g, bool bnd, double* n) {
  n[0] = g[G_N]; n[1] = g[G_N + 1]; n[2] = g[G_N + 2];
  const double d1 = sqrt(g[G_D1] * g[G_D1] + g[G_D1 + 1] * g[G_D1 + 1] + g[G_D1 + 2] * g[G_D1 + 2]);
  const double d2 = sqrt(g[G_D2] * g[G_D2] + g[G_D2 + 1] * g[G_D2 + 1] + g[G_D2 + 2] * g[G_D2 + 2]);
  n[3] = bnd ? 2.0 * d1 : d1 + d2;
}

// FP32 state record of a conserved FP64 state: rho, m, E, p, 1/c, 1/rho
// (reciprocals, so that the product's derivatives divide nowhere)
__device__ __forceinline__ void put_state(float* __restrict__ rec, const double* q, double kappa, double km1) {
  const double ir = 1.0 / q[0];
  const double p = fmax(1.00E-10, km1 * (q[4] - 0.5 * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) * ir));
  float4* d = reinterpret_cast<float4*>(rec);
  d[0] = make_float4((float)q[0], (float)q[1], (float)q[2], (float)q[3]);
  d[1] = make_float4((float)q[4], (float)p, (float)(1.0 / sqrt(kappa * p * ir)), (float)ir);
}

// What P_A's matrix-free product reads, per Newton step: each cell's FP32
// state record and 1/dt and each slot's (normal, s A / V); the boundary
// faces' ghost records and derivatives come from k_cpl_build_bnd
template <int MCF>
__global__ void __launch_bounds__(128) k_cpl_build_state(KArgs<double> a, const double* __restrict__ dtl,
                                                         float* __restrict__ cst, float* __restrict__ idt,
                                                         float4* __restrict__ pna) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nc) return;
  const size_t nc = a.nc;
  double qc[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) qc[j] = a.U[(size_t)j * nc + c];
  put_state(cst + 8 * (size_t)c, qc, a.pc.kappa, a.pc.km1);
  idt[c] = (float)(1.0 / dtl[c]);
  const double iv = 1.0 / a.vol[c];
  for (int k = 0; k < MCF; ++k) {
    const size_t sk = (size_t)k * nc + c;
    const int e = a.cface[(size_t)c * MCF + k];
    if (e < 0) { pna[sk] = make_float4(0.f, 0.f, 0.f, 0.f); continue; }
    const int f = e >> 1, side = e & 1;
    const double* g = a.geo + (size_t)f * GEO;
    // the sign of s A / V carries the side (A / V > 0)
    pna[sk] = make_float4((float)g[G_N], (float)g[G_N + 1], (float)g[G_N + 2],
                          (float)((side ? -1.0 : 1.0) * g[G_A] * iv));
  }
}

// ---- forward-mode derivative of the first-order inviscid face flux ---------
// A side's state (from its record) and the derivative of its primitives
// along a tangent x of its conserved state.
struct SideTan {
  float rho, u[3], E, p, c, ic, ir, un, H;
  float dun, dp, dc, dH, du[3];
};

__device__ __forceinline__ void side_tangent(const float4 r0, const float4 r1, const float* x, const float4 n,
                                             float gam, float gm1, SideTan& s) {
  s.rho = r0.x; s.E = r1.x; s.p = r1.y; s.ic = r1.z; s.ir = r1.w;
  s.c = gam * s.p * s.ir * s.ic;  // c^2 / c
  s.u[0] = r0.y * s.ir; s.u[1] = r0.z * s.ir; s.u[2] = r0.w * s.ir;
  s.un = s.u[0] * n.x + s.u[1] * n.y + s.u[2] * n.z;
  s.H = (s.E + s.p) * s.ir;
#pragma unroll
  for (int i = 0; i < 3; ++i) s.du[i] = (x[1 + i] - s.u[i] * x[0]) * s.ir;
  s.dun = s.du[0] * n.x + s.du[1] * n.y + s.du[2] * n.z;
  const float q2 = s.u[0] * s.u[0] + s.u[1] * s.u[1] + s.u[2] * s.u[2];
  const float um = s.u[0] * x[1] + s.u[1] * x[2] + s.u[2] * x[3];
  s.dp = (s.p > 1.00E-10f) ? gm1 * (x[4] - um + 0.5f * q2 * x[0]) : 0.f;
  s.dc = 0.5f * gam * s.ir * s.ic * (s.dp - s.p * s.ir * x[0]);
  s.dH = (x[4] + s.dp - s.H * x[0]) * s.ir;
}

// dF = (dF/dU_L) dl + (dF/dU_R) dr for the first-order flux F(U_L, U_R; n)
// of fo_flux (Rusanov: flux.c:320-336, AUSM: flux.c:344-406), the branch of
// each max / min and of the Mach-number splitting taken at the state (at a
// tie the one a forward difference along the tangent would see)
__device__ void flux_jvp(const float4 l0, const float4 l1, const float4 r0, const float4 r1, const float* dl,
                         const float* dr, const float4 n, int rusanov, float gam, float gm1, float* dF) {
  SideTan L, R;
  side_tangent(l0, l1, dl, n, gam, gm1, L);
  side_tangent(r0, r1, dr, n, gam, gm1, R);
  const float nn[3] = {n.x, n.y, n.z};
  if (rusanov) {
    const float aL = fabsf(L.un) + L.c, aR = fabsf(R.un) + R.c;
    const float sL = (L.un >= 0.f) ? 1.f : -1.f, sR = (R.un >= 0.f) ? 1.f : -1.f;
    const float daL = sL * L.dun + L.dc, daR = sR * R.dun + R.dc;
    const bool left = (aL > aR) || (aL == aR && daL >= daR);
    const float lam = left ? aL : aR, dlam = left ? daL : daR;
    const float uL[5] = {l0.x, l0.y, l0.z, l0.w, l1.x}, uR[5] = {r0.x, r0.y, r0.z, r0.w, r1.x};
    float dfL[5], dfR[5];
    dfL[0] = dl[0] * L.un + L.rho * L.dun;
    dfR[0] = dr[0] * R.un + R.rho * R.dun;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dfL[1 + i] = dl[1 + i] * L.un + uL[1 + i] * L.dun + L.dp * nn[i];
      dfR[1 + i] = dr[1 + i] * R.un + uR[1 + i] * R.dun + R.dp * nn[i];
    }
    dfL[4] = (dl[4] + L.dp) * L.un + (L.E + L.p) * L.dun;
    dfR[4] = (dr[4] + R.dp) * R.un + (R.E + R.p) * R.dun;
#pragma unroll
    for (int j = 0; j < 5; ++j)
      dF[j] = 0.5f * (dfL[j] + dfR[j]) - 0.5f * dlam * (uR[j] - uL[j]) - 0.5f * lam * (dr[j] - dl[j]);
    return;
  }
  const float ML = L.un * L.ic, MR = R.un * R.ic;
  const float dML = (L.dun - ML * L.dc) * L.ic, dMR = (R.dun - MR * R.dc) * R.ic;
  // split Mach numbers and pressures (their values enter only through the
  // mass flux: the pressure flux is linear in them)
  float mp, dmp, dpp, mm, dmm, dpm;
  if (ML <= -1.f) { mp = dmp = dpp = 0.f; }
  else if (ML < 1.f) {
    mp = 0.25f * (ML + 1.f) * (ML + 1.f);
    dmp = 0.5f * (ML + 1.f) * dML;
    dpp = 0.25f * (L.dp * (1.f + ML) * (1.f + ML) * (2.f - ML) + 3.f * L.p * (1.f - ML * ML) * dML);
  } else { mp = ML; dmp = dML; dpp = L.dp; }
  if (MR <= -1.f) { mm = MR; dmm = dMR; dpm = R.dp; }
  else if (MR < 1.f) {
    mm = -0.25f * (MR - 1.f) * (MR - 1.f);
    dmm = -0.5f * (MR - 1.f) * dMR;
    dpm = 0.25f * (R.dp * (1.f - MR) * (1.f - MR) * (2.f + MR) - 3.f * R.p * (1.f - MR * MR) * dMR);
  } else { mm = dmm = dpm = 0.f; }
  const float sm = mp + mm, ds = dmp + dmm;
  float mdl = 0.f, dmdl = 0.f, mdr = 0.f, dmdr = 0.f;
  if (sm > 0.f || (sm == 0.f && ds > 0.f)) {
    mdl = sm * L.c * L.rho;
    dmdl = ds * L.c * L.rho + sm * (L.dc * L.rho + L.c * dl[0]);
  } else {
    mdr = sm * R.c * R.rho;
    dmdr = ds * R.c * R.rho + sm * (R.dc * R.rho + R.c * dr[0]);
  }
  const float dP = dpp + dpm;
  dF[0] = dmdl + dmdr;
#pragma unroll
  for (int i = 0; i < 3; ++i) dF[1 + i] = dmdl * L.u[i] + mdl * L.du[i] + dmdr * R.u[i] + mdr * R.du[i] + dP * nn[i];
  dF[4] = dmdl * L.H + mdl * L.dH + dmdr * R.H + mdr * R.dH;
}

__device__ __forceinline__ void ld_state(const float* __restrict__ rec, float4& r0, float4& r1) {
  r0 = __ldg(reinterpret_cast<const float4*>(rec));
  r1 = __ldg(reinterpret_cast<const float4*>(rec) + 1);
}

// one slot's contribution s A / V dF to (P_A x)_c: xo is the neighbour's x
// (interior) or unused (boundary: the ghost's tangent is G x_c)
__device__ __forceinline__ void slot_jvp(const float4 c0, const float4 c1, const float* xc, int o,
                                         const float* __restrict__ cst, const float* __restrict__ gst,
                                         const float* __restrict__ gjac, const float* xo, const float4 na,
                                         int rusanov, float gam, float gm1, float* acc) {
  float dF[5];
  if (o >= 0) {
    float4 o0, o1;
    ld_state(cst + 8 * (size_t)o, o0, o1);
    if (na.w >= 0.f) flux_jvp(c0, c1, o0, o1, xc, xo, na, rusanov, gam, gm1, dF);
    else flux_jvp(o0, o1, c0, c1, xo, xc, na, rusanov, gam, gm1, dF);
  } else {
    const int b = -2 - o;
    float4 g0, g1;
    ld_state(gst + 8 * (size_t)b, g0, g1);
    float xg[5];
    const float* G = gjac + 25 * (size_t)b;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      float t = 0.f;
#pragma unroll
      for (int j = 0; j < 5; ++j) t = fmaf(__ldg(G + i * 5 + j), xc[j], t);
      xg[i] = t;
    }
    flux_jvp(c0, c1, g0, g1, xc, xg, na, rusanov, gam, gm1, dF);
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) acc[j] = fmaf(na.w, dF[j], acc[j]);
}

// P_R's slot blocks are applied without being stored: the block of slot k
// is a_k A(U_o) + b_k I (the Euler flux Jacobian of the neighbour's state
// along the face normal, a and b from the face's area, volume, wave speed and
// side), so a sweep reads per slot the normal and two scalars plus the
// neighbour's (u, v, w, H) instead of 25 entries.
// A(U; n) x in FP32 from the state's (u, v, w, H):
//   dp = phi x0 - (g-1) u.x_m + (g-1) x4,  phi = (g-1) |u|^2 / 2,
//   (A x)_0 = n.x_m,  (A x)_m = n dp + u (n.x_m - un x0) + un x_m,
//   (A x)_4 = H (n.x_m - un x0) + un (dp + x4)
__device__ __forceinline__ void rus_jx(const float4 st, float gm1, const float4 n, const float* x, float* y) {
  const float un = st.x * n.x + st.y * n.y + st.z * n.z;
  const float nm = n.x * x[1] + n.y * x[2] + n.z * x[3];
  const float um = st.x * x[1] + st.y * x[2] + st.z * x[3];
  const float phi = 0.5f * gm1 * (st.x * st.x + st.y * st.y + st.z * st.z);
  const float dp = phi * x[0] - gm1 * um + gm1 * x[4];
  const float q = nm - un * x[0];
  y[0] = nm;
  y[1] = n.x * dp + st.x * q + un * x[1];
  y[2] = n.y * dp + st.y * q + un * x[2];
  y[3] = n.z * dp + st.z * q + un * x[3];
  y[4] = st.w * q + un * (dp + x[4]);
}

// Per boundary face: the ghost's FP32 record and G = d ghost / d U_c (FP64
// forward differences of update_boundaries, boundary.c:188-320, stored
// FP32) for P_A's product, and P_R's diagonal block per unit weight (s A /
// V), (A(U_c) + lam I) / 2 + (A(U_g) - lam I) / 2 . G, row-major [nb][25]
// FP64.  Apart from the cell passes so that the boundary arithmetic does
// not set their register budgets.
__global__ void __launch_bounds__(128) k_cpl_build_bnd(KArgs<double> a, float* __restrict__ gst,
                                                       float* __restrict__ gjac, double* __restrict__ bpr) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nf - a.nf_int) return;
  const int f = a.nf_int + b, c = a.fc0[f];  // a boundary face's cell is its cell 0
  const size_t nc = a.nc;
  Phys<double> ph;
  ph.load(a.pc);
  const double kappa = a.pc.kappa;
  double qc[10];
#pragma unroll
  for (int j = 0; j < 5; ++j) qc[j] = a.U[(size_t)j * nc + c];
  cons_to_prims(qc, ph);
  const double* g = a.geo + (size_t)f * GEO;
  double n[4];
  face_normal(g, true, n);
  double Ac[25], lc;
  euler_jacobian(qc, n, kappa, Ac, &lc);
  const int region = a.fregion[b];
  double qg[10], Ag[25], lg;
  ghost_state(qc, region, &g[G_N], &g[G_T1], &g[G_T2], a.pc, ph, qg);
  put_state(gst + 8 * (size_t)b, qg, kappa, a.pc.km1);
  euler_jacobian(qg, n, kappa, Ag, &lg);
  const double lam = fmax(lc, lg) + 2.0 * a.pc.mu / (qc[0] * n[3]);
  double* out = bpr + 25 * (size_t)b;
  for (int v = 0; v < 5; ++v) {
    // column v of d ghost / d U_c, then column v of the block
    const double h = 1e-7 * fmax(fabs(qc[v]), 1e-3);
    double qp[10], qh[10], G[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) qp[j] = qc[j];
    qp[v] += h;
    cons_to_prims(qp, ph);
    ghost_state(qp, region, &g[G_N], &g[G_T1], &g[G_T2], a.pc, ph, qh);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      G[i] = (qh[i] - qg[i]) / h;
      gjac[25 * (size_t)b + i * 5 + v] = (float)G[i];
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      double s = 0.5 * (Ac[i * 5 + v] + (i == v ? lam : 0.0));
#pragma unroll
      for (int l = 0; l < 5; ++l) s += 0.5 * (Ag[i * 5 + l] - (i == l ? lam : 0.0)) * G[l];
      out[i * 5 + v] = s;
    }
  }
}

// P_R: the inverted diagonal blocks (FP64 Gauss-Jordan, stored FP32), the
// slot coefficients of the matrix-free off-diagonal blocks and the cell's
// (u, v, w, H)
template <int MCF>
__global__ void __launch_bounds__(128) k_cpl_build_pr(KArgs<double> a, const double* __restrict__ dtl,
                                                      const double* __restrict__ bpr, float* __restrict__ PRi,
                                                      float4* __restrict__ rna, float* __restrict__ rb,
                                                      float4* __restrict__ st4) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nc) return;
  const size_t nc = a.nc;
  Phys<double> ph;
  ph.load(a.pc);
  const double kappa = a.pc.kappa, mu = a.pc.mu;
  double qc[10];
#pragma unroll
  for (int j = 0; j < 5; ++j) qc[j] = a.U[(size_t)j * nc + c];
  cons_to_prims(qc, ph);
  {
    const double ir = 1.0 / qc[0];
    st4[c] = make_float4((float)(qc[1] * ir), (float)(qc[2] * ir), (float)(qc[3] * ir),
                         (float)((qc[4] + qc[PR]) * ir));
  }
  const double iv = 1.0 / a.vol[c];
  double D[25];
#pragma unroll
  for (int e = 0; e < 25; ++e) D[e] = 0.0;
  const double idt = 1.0 / dtl[c];
#pragma unroll
  for (int j = 0; j < 5; ++j) D[j * 5 + j] = idt;
  for (int k = 0; k < MCF; ++k) {
    const size_t sk = (size_t)k * nc + c;
    const int e = a.cface[(size_t)c * MCF + k];
    if (e < 0) { rna[sk] = make_float4(0.f, 0.f, 0.f, 0.f); rb[sk] = 0.f; continue; }
    const int f = e >> 1, side = e & 1;
    const double* g = a.geo + (size_t)f * GEO;
    const bool bnd = f >= a.nf_int;
    double n[4];
    face_normal(g, bnd, n);
    const double w = (side ? -1.0 : 1.0) * g[G_A] * iv;
    if (!bnd) {
      double Ac[25], lc;
      euler_jacobian(qc, n, kappa, Ac, &lc);
      const int o = side ? a.fc0[f] : a.fc1[f];
      double qo[5];
#pragma unroll
      for (int j = 0; j < 5; ++j) qo[j] = a.U[(size_t)j * nc + o];
      const double lo = wave_speed(qo, n, kappa);
      const double lam = fmax(lc, lo) + 2.0 * mu / (0.5 * (qc[0] + qo[0]) * n[3]);
      // own: cell 0 -> (A + lam I) / 2, cell 1 -> (A - lam I) / 2; the other the opposite
      const double so = side ? -lam : lam;
#pragma unroll
      for (int e2 = 0; e2 < 25; ++e2) D[e2] += w * 0.5 * (Ac[e2] + ((e2 % 6 == 0) ? so : 0.0));
      rna[sk] = make_float4((float)n[0], (float)n[1], (float)n[2], (float)(0.5 * w));
      rb[sk] = (float)(-0.5 * w * so);
    } else {
      // the face's block per unit weight, formed by k_cpl_build_bnd
      const double* sb = bpr + 25 * (size_t)(f - a.nf_int);
#pragma unroll
      for (int e2 = 0; e2 < 25; ++e2) D[e2] += w * sb[e2];
      rna[sk] = make_float4(0.f, 0.f, 0.f, 0.f);
      rb[sk] = 0.f;
    }
  }
  double X[25];
  if (!invert5(D, X)) {
#pragma unroll
    for (int e = 0; e < 25; ++e) X[e] = (e % 6 == 0) ? 1.0 / D[e] : 0.0;
  }
  store_block(PRi + c, nc, X);
}

// P_R's slot blocks written out (for the block export): column j of slot k
// is a A(U_o) e_j + b e_j, by the sweep's own arithmetic
template <int MCF>
__global__ void k_cpl_expand_pr(int nc, const int* __restrict__ nbr, const float4* __restrict__ rna,
                                const float* __restrict__ rb, const float4* __restrict__ st4, float gm1,
                                float* __restrict__ O) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int k = 0; k < MCF; ++k) {
    const size_t sk = (size_t)k * nc + c;
    float* Ok = O + (size_t)k * 25 * nc + c;
    const int o = nbr[sk];
    for (int j = 0; j < 5; ++j) {
      float x[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, y[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      x[j] = 1.f;
      if (o >= 0) {
        rus_jx(st4[o], gm1, rna[sk], x, y);
#pragma unroll
        for (int i = 0; i < 5; ++i) y[i] = rna[sk].w * y[i] + rb[sk] * x[i];
      }
#pragma unroll
      for (int i = 0; i < 5; ++i) Ok[(size_t)(i * 5 + j) * nc] = y[i];
    }
  }
}

__device__ __forceinline__ void ld5(const float* __restrict__ x, size_t nc, int c, float* v) {
#pragma unroll
  for (int j = 0; j < 5; ++j) v[j] = __ldg(x + (size_t)j * nc + c);
}

__device__ __forceinline__ void block_mul_add(const float* __restrict__ B, size_t nc, const float* x, float* y) {
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    float s = y[i];
#pragma unroll
    for (int j = 0; j < 5; ++j) s = fmaf(__ldg(B + (size_t)(i * 5 + j) * nc), x[j], s);
    y[i] = s;
  }
}

// y = P_A x = x / dt - dR1/dU x, matrix-free: per slot the exact
// derivative of the face's first-order flux along (x_c, x_o) in FP32
template <int MCF>
__global__ void __launch_bounds__(256, 4) k_cpl_product(int nc, const float* __restrict__ cst,
                                                     const float* __restrict__ idt, const float4* __restrict__ pna,
                                                     const int* __restrict__ nbr, const float* __restrict__ gst,
                                                     const float* __restrict__ gjac, int rusanov, float gam,
                                                     float gm1, const float* __restrict__ x, float* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  float xc[5], acc[5];
  ld5(x, nc, c, xc);
  const float id = __ldg(idt + c);
#pragma unroll
  for (int j = 0; j < 5; ++j) acc[j] = id * xc[j];
  float4 c0, c1;
  ld_state(cst + 8 * (size_t)c, c0, c1);
#pragma unroll
  for (int k = 0; k < MCF; ++k) {
    const size_t sk = (size_t)k * nc + c;
    const int o = __ldg(nbr + sk);
    if (o == -1) continue;
    float xo[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (o >= 0) ld5(x, nc, o, xo);
    slot_jvp(c0, c1, xc, o, cst, gst, gjac, xo, __ldg(pna + sk), rusanov, gam, gm1, acc);
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) y[(size_t)j * nc + c] = acc[j];
}

// the first damped sweep of P_R from zero for cell c: y = omega Dinv b
// (k_cpl_sweep's arithmetic at x = 0)
__device__ __forceinline__ void first_sweep(const float* __restrict__ Di, int nc, int c, float omega,
                                            const float* b, float* __restrict__ y) {
  float r[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  block_mul_add(Di + c, nc, b, r);
#pragma unroll
  for (int j = 0; j < 5; ++j) y[(size_t)j * nc + c] = 0.f + omega * r[j];
}

// the update pass of the inner Gram-Schmidt, per cell: v = (w - sum_i h_i
// V_i) * s, s = 1 / |w - sum_i h_i V_i| (k_gs's PASS 3 arithmetic: the same
// FP32 products and order, so the same values); with y0 set, the first
// sweep of P_R on the new vector too
__global__ void __launch_bounds__(256, 4) k_cpl_next(int nc, size_t ldb, const float* __restrict__ w,
                                                  const float* __restrict__ V, int k, const double* __restrict__ h,
                                                  const double* __restrict__ scale_p, float* __restrict__ vout,
                                                  const float* __restrict__ Di, float omega,
                                                  float* __restrict__ y0) {
  __shared__ float hs[32];
  if (threadIdx.x < 32) hs[threadIdx.x] = (threadIdx.x < (unsigned)k) ? (float)h[threadIdx.x] : 0.f;
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  float sum[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int i = 0; i < k; ++i) {
    float a[5];
    ld5(V + (size_t)i * ldb, nc, c, a);
#pragma unroll
    for (int j = 0; j < 5; ++j) sum[j] = fmaf(hs[i], a[j], sum[j]);
  }
  const float scale = (float)*scale_p;
  float v[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    const size_t e = (size_t)j * nc + c;
    v[j] = (__ldg(w + e) - sum[j]) * scale;
    vout[e] = v[j];
  }
  if (y0 != nullptr) first_sweep(Di, nc, c, omega, v, y0);
}

// P_A written out as blocks (for the block export), by the product's own
// arithmetic: column j of the diagonal block is the response to x_c = e_j,
// of slot k's block the response of that slot to x_o = e_j
template <int MCF>
__global__ void k_cpl_expand_pa(int nc, const float* __restrict__ cst, const float* __restrict__ idt,
                                const float4* __restrict__ pna, const int* __restrict__ nbr,
                                const float* __restrict__ gst, const float* __restrict__ gjac, int rusanov, float gam,
                                float gm1, float* __restrict__ Dg, float* __restrict__ O) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  float4 c0, c1;
  ld_state(cst + 8 * (size_t)c, c0, c1);
  for (int j = 0; j < 5; ++j) {
    float e[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, zero[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    e[j] = 1.f;
    float d[5];
    for (int i = 0; i < 5; ++i) d[i] = idt[c] * e[i];
    for (int k = 0; k < MCF; ++k) {
      const size_t sk = (size_t)k * nc + c;
      const int o = nbr[sk];
      float* Ok = O + (size_t)k * 25 * nc + c;
      float col[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      if (o != -1) {
        slot_jvp(c0, c1, e, o, cst, gst, gjac, zero, pna[sk], rusanov, gam, gm1, d);
        if (o >= 0) slot_jvp(c0, c1, zero, o, cst, gst, gjac, e, pna[sk], rusanov, gam, gm1, col);
      }
      for (int i = 0; i < 5; ++i) Ok[(size_t)(i * 5 + j) * nc] = col[i];
    }
    for (int i = 0; i < 5; ++i) Dg[(size_t)(i * 5 + j) * nc + c] = d[i];
  }
}

// one damped block-Jacobi sweep of P_R after the first, y = x + omega (Dinv
// (b - O x) - x), the slot blocks O applied matrix-free (the first sweep,
// from x = 0, is first_sweep in the pass that forms b).  Undamped sweeps
// overshoot on this operator (at CFL 1e4 the error after four of them is
// about 1.4 times that after four with omega = 0.7)
template <int MCF, class TO>
__global__ void __launch_bounds__(256) k_cpl_sweep(int nc, const float* __restrict__ Di, const int* __restrict__ nbr,
                                                   const float4* __restrict__ rna, const float* __restrict__ rb,
                                                   const float4* __restrict__ st4, float gm1, float omega,
                                                   const float* __restrict__ b, const float* __restrict__ x,
                                                   TO* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  float t[5], r[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, xc[5];
  ld5(b, nc, c, t);
  ld5(x, nc, c, xc);
#pragma unroll
  for (int k = 0; k < MCF; ++k) {
    const size_t sk = (size_t)k * nc + c;
    const int o = __ldg(nbr + sk);
    if (o < 0) continue;
    float xo[5], jx[5];
    ld5(x, nc, o, xo);
    const float4 na = __ldg(rna + sk);
    const float bk = __ldg(rb + sk);
    rus_jx(__ldg(st4 + o), gm1, na, xo, jx);
#pragma unroll
    for (int j = 0; j < 5; ++j) t[j] -= na.w * jx[j] + bk * xo[j];
  }
  block_mul_add(Di + c, nc, t, r);
#pragma unroll
  for (int j = 0; j < 5; ++j) y[(size_t)j * nc + c] = (TO)(xc[j] + omega * (r[j] - xc[j]));
}

// V_0 = v / |v| (the inverse norm from a device slot), stored FP32, per
// cell, and the first sweep of P_R on it into y0
template <class T>
__global__ void __launch_bounds__(256) k_cpl_start(int nc, const T* __restrict__ v, const double* __restrict__ inv,
                                                   float* __restrict__ V0, const float* __restrict__ Di, float omega,
                                                   float* __restrict__ y0) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double s = *inv;
  float b[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    const size_t e = (size_t)j * nc + c;
    b[j] = (float)((double)v[e] * s);
    V0[e] = b[j];
  }
  first_sweep(Di, nc, c, omega, b, y0);
}

// the inner least-squares problem min |beta e_1 - H y| by Givens rotations
// (FP32, H in shared memory): H from the Gram-Schmidt passes' columns, y [m]
// into hin + m * kHcol + 8; the columns past a breakdown (a zero
// subdiagonal or a zero or non-finite rotation) get y = 0.  One thread per
// column, in rounds: round r forms rotation r from column r (which has had
// rotations 0 .. r-1) and the columns past r apply it, so each column sees
// its rotations in the serial order; the back substitution is serial.
// Launched with at least m * 31 threads (one load each), a multiple of 32.
__global__ void k_cpl_lsq(int m, double* __restrict__ hin) {
  __shared__ float H[30][31];
  __shared__ float cs[30], sn[30], g[31], y[30];
  __shared__ int kk_s, stop;
  const int t = threadIdx.x;
  // the columns (one Gram-Schmidt pass: h at [0, 32), the norm at 64)
  for (int q = t; q < m * 31; q += blockDim.x) {
    const int j = q / 31, i = q % 31;
    const double* hc = hin + (size_t)j * kHcol;
    H[j][i] = (i <= j) ? (float)hc[i] : (i == j + 1 ? (float)hc[64] : 0.f);
  }
  if (t <= m) g[t] = (t == 0) ? (float)hin[(size_t)m * kHcol] : 0.f;  // |v| from the norm pass
  if (t == 0) {
    kk_s = 0;
    stop = 0;
  }
  __syncthreads();
  for (int r = 0; r < m; ++r) {
    if (t == r) {
      const float hn = H[r][r + 1];
      const float a0 = H[r][r], b0 = H[r][r + 1];
      const float rr = sqrtf(a0 * a0 + b0 * b0);
      if (!(rr > 0.f) || !isfinite(rr)) {
        stop = 1;
      } else {
        cs[r] = a0 / rr;
        sn[r] = b0 / rr;
        H[r][r] = rr;
        g[r + 1] = -sn[r] * g[r];
        g[r] = cs[r] * g[r];
        kk_s = r + 1;
        if (!(hn > 0.f)) stop = 1;  // the Krylov space is invariant: exact solution
      }
    }
    __syncthreads();
    if (stop) break;  // the same value in every thread
    if (t > r && t < m) {
      const float a0 = H[t][r], b0 = H[t][r + 1];
      H[t][r] = cs[r] * a0 + sn[r] * b0;
      H[t][r + 1] = -sn[r] * a0 + cs[r] * b0;
    }
    __syncthreads();
  }
  const int kk = kk_s;
  if (t == 0) {
    for (int i = kk - 1; i >= 0; --i) {
      float s = g[i];
      for (int j = i + 1; j < kk; ++j) s -= H[j][i] * y[j];
      y[i] = s / H[i][i];
    }
  }
  __syncthreads();
  if (t < m) hin[(size_t)m * kHcol + 8 + t] = (t < kk) ? (double)y[t] : 0.0;
}

// u = sum_j y_j T_j (FP32 directions, ldb apart: 16-byte aligned), four
// consecutive elements per thread with 16-byte loads, then the n % 4 tail
template <class TO>
__global__ void k_cpl_combine(size_t n, size_t ldb, const float* __restrict__ V, const double* __restrict__ y, int m,
                              TO* __restrict__ u) {
  __shared__ float ys[32];
  if (threadIdx.x < 32) ys[threadIdx.x] = (threadIdx.x < (unsigned)m) ? (float)y[threadIdx.x] : 0.f;
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * blockDim.x, gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t nq = n / 4;
  for (size_t q = gid; q < nq; q += stride) {
    float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int j = 0; j < m; ++j) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(V + (size_t)j * ldb) + q);
      s[0] = fmaf(ys[j], v.x, s[0]);
      s[1] = fmaf(ys[j], v.y, s[1]);
      s[2] = fmaf(ys[j], v.z, s[2]);
      s[3] = fmaf(ys[j], v.w, s[3]);
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) u[4 * q + l] = (TO)s[l];
  }
  for (size_t i = 4 * nq + gid; i < n; i += stride) {
    float s = 0.f;
    for (int j = 0; j < m; ++j) s = fmaf(ys[j], __ldg(V + (size_t)j * ldb + i), s);
    u[i] = (TO)s;
  }
}

}  // namespace

#define CCK(expr)                                               \
  do {                                                          \
    fv3d_status st__ = ctx.cuda((expr), #expr);                 \
    if (st__ != FV3D_OK) return st__;                           \
  } while (0)

fv3d_status Coupled::setup(Ctx& ctx, Implicit& im, int m_inner, int n_sweeps, float damping) {
  // captured Arnoldi steps hold the buffers, the inner iteration counts and the damping
  if (m_inner != m_in || n_sweeps != sweep_count || damping != omega) im.release_graphs();
  m_in = m_inner;
  sweep_count = n_sweeps;
  omega = damping;
  if (nc == ctx.nc && mcf == ctx.mcf && nb == ctx.nb && ldb == im.ldb && m_cap >= m_inner) return FV3D_OK;
  im.release_graphs();
  nc = ctx.nc;
  mcf = ctx.mcf;
  n = im.n;
  ldb = im.ldb;
  m_cap = m_inner;
  if (mcf != 4 && mcf != 6 && mcf != 8) return ctx.fail(FV3D_ERR_UNSUPPORTED, "coupled preconditioner: %d face slots", mcf);
  nb = ctx.nb;
  cudaError_t e = nbr.alloc((size_t)mcf * nc);
  if (e == cudaSuccess) e = cst.alloc(8 * (size_t)nc);
  if (e == cudaSuccess) e = idt.alloc(nc);
  if (e == cudaSuccess) e = pna.alloc((size_t)mcf * nc);
  if (e == cudaSuccess) e = gst.alloc(8 * (size_t)nb);
  if (e == cudaSuccess) e = gjac.alloc(25 * (size_t)nb);
  if (e == cudaSuccess) e = bpr.alloc(25 * (size_t)std::max(nb, 1));
  if (e == cudaSuccess) e = PRi.alloc(25 * (size_t)nc);
  if (e == cudaSuccess) e = rna.alloc((size_t)mcf * nc);
  if (e == cudaSuccess) e = rb.alloc((size_t)mcf * nc);
  if (e == cudaSuccess) e = st4.alloc(nc);
  if (e == cudaSuccess) e = Vi.alloc((size_t)(m_cap + 1) * ldb);
  if (e == cudaSuccess) e = wi.alloc(ldb);
  if (e == cudaSuccess) e = ti.alloc(ldb);
  if (e == cudaSuccess) e = Ti.alloc((size_t)m_cap * ldb);
  if (e == cudaSuccess) e = hin.alloc((size_t)(m_cap + 1) * kHcol);
  CCK(e);
  // the tails past n of the FP32 vectors are never written: zero them once
  CCK(cudaMemsetAsync(Vi.p, 0, sizeof(float) * Vi.n, ctx.stream));
  CCK(cudaMemsetAsync(Ti.p, 0, sizeof(float) * Ti.n, ctx.stream));
  CCK(cudaMemsetAsync(hin.p, 0, sizeof(double) * hin.n, ctx.stream));
  KArgs<double> a = ctx.args<double>();
  k_cpl_nbr<<<nblk(nc), 256, 0, ctx.stream>>>(nc, mcf, ctx.nf_int, a.cface, a.fc0, a.fc1, nbr.p);
  CCK(cudaGetLastError());
  return FV3D_OK;
}

fv3d_status Coupled::build(Ctx& ctx, Implicit& im) {
  KArgs<double> a = ctx.args<double>();
  const int g = nblk(nc, 128);
  if (nb > 0) k_cpl_build_bnd<<<nblk(nb, 128), 128, 0, ctx.stream>>>(a, gst.p, gjac.p, bpr.p);
#define CPL_BUILD(M)                                                                           \
  k_cpl_build_state<M><<<g, 128, 0, ctx.stream>>>(a, im.dtl.p, cst.p, idt.p, pna.p);             \
  k_cpl_build_pr<M><<<g, 128, 0, ctx.stream>>>(a, im.dtl.p, bpr.p, PRi.p, rna.p, rb.p, st4.p)
  if (mcf == 4) { CPL_BUILD(4); }
  else if (mcf == 6) { CPL_BUILD(6); }
  else { CPL_BUILD(8); }
#undef CPL_BUILD
  CCK(cudaGetLastError());
  return FV3D_OK;
}

// out = M_R b: `count` damped block-Jacobi sweeps of P_R from zero, the
// first of them (omega Dinv b) already in x0, written by the pass that
// formed b (x0 is out itself for one sweep)
template <class TO>
fv3d_status Coupled::sweeps(Ctx& ctx, int count, const float* b, const float* x0, TO* out) {
  const int g = nblk(nc);
  const float gm1 = (float)ctx.phys.km1;
  // the sweeps alternate between ti and wi, the last one writes out; b is never overwritten
  const float* x = x0;
  for (int s = 1; s < count; ++s) {
    const bool last = (s == count - 1);
    float* tmp = (s % 2 == 0) ? ti.p : wi.p;
#define CPL_SWEEP(M)                                                                                     \
  if (last) k_cpl_sweep<M, TO><<<g, 256, 0, ctx.stream>>>(nc, PRi.p, nbr.p, rna.p, rb.p, st4.p, gm1, omega, b, x, out); \
  else k_cpl_sweep<M, float><<<g, 256, 0, ctx.stream>>>(nc, PRi.p, nbr.p, rna.p, rb.p, st4.p, gm1, omega, b, x, tmp)
    if (mcf == 4) { CPL_SWEEP(4); }
    else if (mcf == 6) { CPL_SWEEP(6); }
    else { CPL_SWEEP(8); }
#undef CPL_SWEEP
    x = tmp;
  }
  CCK(cudaGetLastError());
  return FV3D_OK;
}

template <class T>
fv3d_status Coupled::apply(Ctx& ctx, Implicit& im, const T* v, T* z) {
  const int m = m_in, sw = sweep_count;
  const int rusanov = ctx.phys.flux == 1 ? 1 : 0;
  const float gam = (float)ctx.phys.kappa, gm1 = (float)ctx.phys.km1;
  double* hb = hin.p + (size_t)m * kHcol;  // |v| and its inverse, then y at +8
  // |v| (FP64 for a FP64 input, FP32 otherwise) and V_0 = v / |v|
  fv3d_status st = im.gs_pass<T>(ctx, 0, const_cast<T*>(v), v, 1, nullptr, hb, 1.0, nullptr);
  if (st != FV3D_OK) return st;
  const int g = nblk(nc);
  // the first sweep of each v_j is made by the pass that forms v_j, into ti
  // (into t_j itself with one sweep)
  auto first = [&](int j) { return sw == 1 ? Ti.p + (size_t)j * ldb : ti.p; };
  k_cpl_start<T><<<g, 256, 0, ctx.stream>>>(nc, v, hb + 1, Vi.p, PRi.p, omega, first(0));
  CCK(cudaGetLastError());
  for (int j = 0; j < m; ++j) {
    float* vj = Vi.p + (size_t)j * ldb;
    double* hc = hin.p + (size_t)j * kHcol;
    // t_j = M_R v_j (kept: the inner solve is flexible), w = P_A t_j
    float* tj = Ti.p + (size_t)j * ldb;
    if ((st = sweeps<float>(ctx, sw, vj, first(j), tj)) != FV3D_OK) return st;
#define CPL_PRODUCT(M)                                                                                      \
  k_cpl_product<M><<<g, 256, 0, ctx.stream>>>(nc, cst.p, idt.p, pna.p, nbr.p, gst.p, gjac.p, rusanov, gam, gm1, \
                                              tj, wi.p)
    if (mcf == 4) CPL_PRODUCT(4);
    else if (mcf == 6) CPL_PRODUCT(6);
    else CPL_PRODUCT(8);
#undef CPL_PRODUCT
    CCK(cudaGetLastError());
    // classical Gram-Schmidt once (dots and |w|^2 in one pass, the norm of
    // the projected w by Pythagoras), FP32: a short inner solve that only
    // preconditions needs no re-orthogonalisation.  (The dots summed inside
    // the product's pass instead made that pass longer than the two apart:
    // 617 against 555 ms for the channel's solve.)
    if ((st = im.gs_pass<float>(ctx, 4, wi.p, Vi.p, j + 1, nullptr, hc, 0.0, nullptr, nullptr, hc + 64)) != FV3D_OK)
      return st;
    // v_{j+1} = (w - sum_i h_i v_i) / its norm, and its first sweep; the
    // last iteration's is never used (the least-squares problem takes only
    // the norm)
    if (j + 1 < m) {
      k_cpl_next<<<g, 256, 0, ctx.stream>>>(nc, ldb, wi.p, Vi.p, j + 1, hc, hc + 65, Vi.p + (size_t)(j + 1) * ldb,
                                            PRi.p, omega, first(j + 1));
      CCK(cudaGetLastError());
    }
  }
  k_cpl_lsq<<<1, (m * 31 + 31) / 32 * 32, 0, ctx.stream>>>(m, hin.p);
  // z = sum_j y_j t_j
  k_cpl_combine<T><<<std::min(4096, nblk((n + 3) / 4)), 256, 0, ctx.stream>>>(n, ldb, Ti.p, hb + 8, m, z);
  CCK(cudaGetLastError());
  return FV3D_OK;
}

template fv3d_status Coupled::apply<float>(Ctx&, Implicit&, const float*, float*);
template fv3d_status Coupled::apply<double>(Ctx&, Implicit&, const double*, double*);

}  // namespace fv3d

// ---------------------------------------------------------------------------
// export of the last build's blocks (reference cell order)
// ---------------------------------------------------------------------------
using namespace fv3d;

extern "C" fv3d_status fv3d_get_coupled_blocks(fv3d_ctx* handle, int which, double* diag, double* slots,
                                               int* neighbour, int* max_slots) {
  if (handle == nullptr || max_slots == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  const Coupled* cp = ctx->implicit ? ctx->implicit->coupled : nullptr;
  if (cp == nullptr || cp->nc != ctx->nc) return ctx->fail(FV3D_ERR_STATE, "no coupled preconditioner built");
  if (which != 0 && which != 1) return ctx->fail(FV3D_ERR_INVALID_ARG, "which must be 0 (P_A) or 1 (P_R)");
  *max_slots = cp->mcf;
  if (diag == nullptr && slots == nullptr && neighbour == nullptr) return FV3D_OK;
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "cudaSetDevice");
  const size_t nc = cp->nc, mcf = cp->mcf;
  std::vector<float> d(25 * nc), o(mcf * 25 * nc);
  std::vector<int> nb(mcf * nc);
  // the slot blocks (and P_A's diagonal blocks) written out by the
  // matrix-free operators' own arithmetic
  DevBuf<float> ex_d, ex_o;
  if (ex_o.alloc(mcf * 25 * nc) != cudaSuccess || (which == 0 && ex_d.alloc(25 * nc) != cudaSuccess))
    return ctx->fail(FV3D_ERR_DEVICE, "allocation");
  const int g = (int)((nc + 255) / 256);
  const float gam = (float)ctx->phys.kappa, gm1 = (float)ctx->phys.km1;
  const int rus = ctx->phys.flux == 1 ? 1 : 0;
  const Coupled& q = *cp;
#define CPL_EXPAND(M)                                                                                          \
  if (which) k_cpl_expand_pr<M><<<g, 256, 0, ctx->stream>>>((int)nc, q.nbr.p, q.rna.p, q.rb.p, q.st4.p, gm1, ex_o.p); \
  else k_cpl_expand_pa<M><<<g, 256, 0, ctx->stream>>>((int)nc, q.cst.p, q.idt.p, q.pna.p, q.nbr.p, q.gst.p, q.gjac.p, \
                                                      rus, gam, gm1, ex_d.p, ex_o.p)
  if (mcf == 4) { CPL_EXPAND(4); }
  else if (mcf == 6) { CPL_EXPAND(6); }
  else { CPL_EXPAND(8); }
#undef CPL_EXPAND
  if (cudaGetLastError() != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "expand blocks");
  const float* src_d = which ? cp->PRi.p : ex_d.p;
  const float* src_o = ex_o.p;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
      cudaMemcpy(d.data(), src_d, sizeof(float) * d.size(), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(o.data(), src_o, sizeof(float) * o.size(), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(nb.data(), cp->nbr.p, sizeof(int) * nb.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return ctx->fail(FV3D_ERR_DEVICE, "copy coupled blocks");
  for (size_t c = 0; c < nc; ++c) {
    const size_t r = (size_t)ctx->perm[c];
    for (int e = 0; e < 25; ++e) {
      if (diag) diag[r * 25 + e] = d[(size_t)e * nc + c];
      for (size_t k = 0; k < mcf; ++k)
        if (slots) slots[(r * mcf + k) * 25 + e] = o[(k * 25 + e) * nc + c];
    }
    if (neighbour)
      for (size_t k = 0; k < mcf; ++k) {
        const int x = nb[k * nc + c];
        neighbour[r * mcf + k] = (x < 0) ? -1 : ctx->perm[x];
      }
  }
  return FV3D_OK;
}
