// Residual / explicit-stage kernels for sm_103a.
//
// Per RK stage three launches, all deterministic (no floating-point atomics):
//   k_gradients      cell-gather: own + neighbour states -> Green-Gauss or
//                    least-squares gradients and the Barth-Jespersen neighbour
//                    min/max; one per-cell record  (reconstruction.c:20-93,
//                    limiter.c:60-82, boundary.c:188-412)
//   k_face_flux      face-parallel: limited linear reconstruction of both
//                    sides, Rusanov/AUSM convective + viscous flux, times the
//                    face area (reconstruction.c:142-255, flux.c:23-198)
//   k_gather_update  cell-gather of +-F*A over the cell's faces in ascending
//                    original face id (the summation order of the
//                    reference's face scatter, finite_volume.c:100-123),
//                    -sum/V, fused with the low-storage RK / SSP-RK3 update
//                    (explicit.c:96-140) and the next CFL time step
//                    (navier_stokes.c:171-187).
// R = double: FP64 path.  R = float: mixed path (FP32 faces/gradients/
// limiter with Kahan-compensated per-cell sums; FP64 state and RK register).
#pragma once

#include "physics.cuh"

namespace fv3d {

constexpr int REC = 56;   // per-cell record length (elements of R)
constexpr int GEO = 16;   // per-face geometry record
constexpr int FAS = 8;    // per-face flux slot (5 used): one 32-byte sector in FP32
constexpr int NG = 9;     // gradient variables: 0..7 and T
// record layout
constexpr int R_Q = 0;     // [0..7] rho, rho_u, rho_v, rho_w, rho_e, u, v, w
constexpr int R_P = 8;     // pressure
constexpr int R_T = 9;     // temperature
constexpr int R_G = 10;    // [10..36] gradients, var-major (g*3 + d), g = 0..7, 8 -> T
constexpr int R_MIN = 37;  // [37..44]
constexpr int R_MAX = 45;  // [45..52]
// geometry layout
constexpr int G_N = 0, G_A = 3, G_T1 = 4, G_T2 = 7, G_D1 = 10, G_D2 = 13;

struct DevScalars {
  double t;                     // accumulated time
  double dt;                    // current time step
  unsigned long long lam_bits;  // running min of V / sum (|u|+c) dx (positive double bits)
  int step;
  int status;                   // bit 0: non-finite state/time step
};

template <class R>
struct KArgs {
  int nc, nf, nf_int, mcf;
  const int* __restrict__ fc0;
  const int* __restrict__ fc1;
  const R* __restrict__ geo;       // [nf][GEO]
  const R* __restrict__ lam;       // [nf]
  const R* __restrict__ lsq;       // [nf][6]
  const int* __restrict__ fregion; // [nf - nf_int]
  const int* __restrict__ cface;   // [nc][mcf]: (face << 1) | side, -1 padded
  const R* __restrict__ rvol;      // [nc] 1/V
  const double* __restrict__ vol;  // [nc]
  const double* __restrict__ dx;   // [nc][3]
  double* U;                       // [5][nc] conserved state (FP64)
  double* Pq;                      // [5][nc] its primitives u, v, w, p, T (FP64 path: k_prims)
  double* K;                       // [5][nc] low-storage RK register
  double* U0;                      // [5][nc] SSP-RK3 stage-0 state
  float* Uf;                       // [nc][8] FP32 shadow (rho, m, E, p, T, 1/rho)
  R* rec;                          // [nc][REC]
  R* FA;                           // [nf][FAS]
  double* dphi;                    // [5][nc] residual output
  DevScalars* sc;
  PhysConst pc;
};

// ---------------------------------------------------------------------------
// state access
// ---------------------------------------------------------------------------
template <class R> struct State;

template <> struct State<double> {
  static __device__ __forceinline__ void load(const KArgs<double>& a, int c, double* q,
                                              const Phys<double>& ph) {
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = a.U[(size_t)j * a.nc + c];
    cons_to_prims(q, ph);
  }
};

template <> struct State<float> {
  static __device__ __forceinline__ void load(const KArgs<float>& a, int c, float* q,
                                              const Phys<float>& ph) {
    const float4* s = reinterpret_cast<const float4*>(a.Uf) + 2 * (size_t)c;
    float4 x = __ldg(s), y = __ldg(s + 1);
    q[RHO] = x.x; q[MX] = x.y; q[MY] = x.z; q[MZ] = x.w; q[EN] = y.x;
    q[PR] = y.y; q[TT] = y.z;
    q[VU] = q[MX] / q[RHO];
    q[VV] = q[MY] / q[RHO];
    q[VW] = q[MZ] / q[RHO];
  }
};

// N consecutive elements from p into o; FP64 rows that start on a 16-byte
// boundary (the face geometry, the per-cell records) by 16-byte loads
#ifndef FV3D_F64_VEC
#define FV3D_F64_VEC 1
#endif
template <int N, class R>
__device__ __forceinline__ void load_row(const R* __restrict__ p, R* o) {
  if constexpr (sizeof(R) == 8 && N % 2 == 0 && FV3D_F64_VEC) {
    const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
    for (int j = 0; j < N / 2; ++j) {
      const double2 v = __ldg(q + j);
      o[2 * j] = v.x;
      o[2 * j + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) o[j] = p[j];
  }
}


// ---------------------------------------------------------------------------
// K0 (FP64 path): every cell's primitives (u, v, w, p, T) of the state, once
// per residual, so that the gradient pass reads a neighbour's instead of
// recomputing them per face (four FP64 divisions each, at GB300's FP64
// rate); the same cons_to_prims arithmetic, so the same values
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(256) k_prims(const __grid_constant__ KArgs<R> a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nc) return;
  Phys<R> ph;
  ph.load(a.pc);
  R q[10];
#pragma unroll
  for (int j = 0; j < 5; ++j) q[j] = a.U[(size_t)j * a.nc + c];
  cons_to_prims(q, ph);
#pragma unroll
  for (int j = 0; j < 5; ++j) a.Pq[(size_t)j * a.nc + c] = q[VU + j];
}

// a cell's conserved state and primitives: from k_prims's output on the
// FP64 path, else computed
template <class R>
__device__ __forceinline__ void load_state(const KArgs<R>& a, int c, R* q, const Phys<R>& ph) {
  if constexpr (sizeof(R) == 8) {
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = a.U[(size_t)j * a.nc + c];
#pragma unroll
    for (int j = 0; j < 5; ++j) q[VU + j] = a.Pq[(size_t)j * a.nc + c];
  } else {
    State<R>::load(a, c, q, ph);
  }
}

// ---------------------------------------------------------------------------
// K1: gradients + neighbour min/max
// GMODE 0: no gradients (first order, inviscid); 1 Green-Gauss; 2 least squares
// ---------------------------------------------------------------------------
template <class R, int GMODE, bool LIMIT, bool KAHAN>
__global__ void __launch_bounds__(256) k_gradients(const __grid_constant__ KArgs<R> a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nc) return;
  Phys<R> ph;
  ph.load(a.pc);
  R q[10];
  load_state(a, c, q, ph);
  R* out = a.rec + (size_t)c * REC;
  if (GMODE != 0) {
    Acc<R, KAHAN> g[NG][3];
    R mn[8], mx[8];
#pragma unroll
    for (int v = 0; v < 8; ++v) { mn[v] = q[v]; mx[v] = q[v]; }
    for (int k = 0; k < a.mcf; ++k) {
      const int e = a.cface[(size_t)c * a.mcf + k];
      if (e < 0) break;
      const int f = e >> 1, side = e & 1;
      R go[10];
      load_row<10>(a.geo + (size_t)f * GEO, go);
      R qo[10];
      if (f >= a.nf_int) {
        ghost_state(q, a.fregion[f - a.nf_int], &go[G_N], &go[G_T1], &go[G_T2], a.pc, ph, qo);
      } else {
        const int o = side ? a.fc0[f] : a.fc1[f];
        load_state(a, o, qo, ph);
      }
      if (GMODE == 1) {
        const R lamf = a.lam[f];
        const R A = go[G_A];
        const R* q0 = side ? qo : q;
        const R* q1 = side ? q : qo;
#pragma unroll
        for (int v = 0; v < NG; ++v) {
          const int j = (v < 8) ? v : TT;
          R mean = q0[j] + lamf * (q1[j] - q0[j]);
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            R t = mean * go[G_N + d] * A;
            if (side) g[v][d].sub(t);
            else g[v][d].add(t);
          }
        }
      } else {
        const R* w = a.lsq + (size_t)f * 6 + 3 * side;
        R w0 = w[0], w1 = w[1], w2 = w[2];
#pragma unroll
        for (int v = 0; v < NG; ++v) {
          const int j = (v < 8) ? v : TT;
          R dq = qo[j] - q[j];
          g[v][0].add(w0 * dq);
          g[v][1].add(w1 * dq);
          g[v][2].add(w2 * dq);
        }
      }
      if (LIMIT) {
#pragma unroll
        for (int v = 0; v < 8; ++v) { mn[v] = rmin(mn[v], qo[v]); mx[v] = rmax(mx[v], qo[v]); }
      }
    }
    const R s = (GMODE == 1) ? a.rvol[c] : (R)1;
#pragma unroll
    for (int v = 0; v < NG; ++v)
#pragma unroll
      for (int d = 0; d < 3; ++d) out[R_G + 3 * v + d] = (GMODE == 1) ? g[v][d].value() * s : g[v][d].value();
    if (LIMIT) {
#pragma unroll
      for (int v = 0; v < 8; ++v) { out[R_MIN + v] = mn[v]; out[R_MAX + v] = mx[v]; }
    }
  }
#pragma unroll
  for (int v = 0; v < 8; ++v) out[R_Q + v] = q[v];
  out[R_P] = q[PR];
  out[R_T] = q[TT];
}

// Limited linear reconstruction of variables 0..7 of one side.
// FP64 path: the reference's min(1, y) factor (limiter.c:86-106); FP32 path:
// the algebraically identical division-free clamp of the slope.
template <class R, bool LINEAR, bool LIMIT>
__device__ __forceinline__ void reconstruct(const R* rc, const R* r, R* q) {
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    R val = rc[R_Q + v];
    if (LINEAR) {
      const R* g = rc + R_G + 3 * v;
      R slope = r[0] * g[0] + r[1] * g[1] + r[2] * g[2];
      if (LIMIT) {
        R hi = rc[R_MAX + v], lo = rc[R_MIN + v];
        if (sizeof(R) == 8) {
          R y = (R)1;
          if (slope > (R)0) y = (hi - val) / slope;
          else if (slope < (R)0) y = (lo - val) / slope;
          val = val + rmin((R)1, y) * slope;
        } else {
          R inc = (slope > (R)0) ? rmin(slope, hi - val) : ((slope < (R)0) ? rmax(slope, lo - val) : (R)0);
          val = val + inc;
        }
      } else {
        val = val + slope;
      }
    }
    q[v] = val;
  }
}

// ---------------------------------------------------------------------------
// K2: face fluxes  FA[f] = F(qL, qR) * A
// ---------------------------------------------------------------------------
template <class R, bool LINEAR, bool LIMIT, bool VISCOUS>
__global__ void __launch_bounds__(256) k_face_flux(const __grid_constant__ KArgs<R> a) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.nf) return;
  Phys<R> ph;
  ph.load(a.pc);
  R go[GEO];
  load_row<GEO>(a.geo + (size_t)f * GEO, go);
  const R* n = &go[G_N];
  const R* t1 = &go[G_T1];
  const R* t2 = &go[G_T2];
  const int c0 = a.fc0[f];
  R rl[REC];
  load_row<REC>(a.rec + (size_t)c0 * REC, rl);
  R ql[10], qr[10];
  R gml[12], gmr[12];   // gradients of rho_u, rho_v, rho_w, T for the viscous flux
  reconstruct<R, LINEAR, LIMIT>(rl, &go[G_D1], ql);
  if (VISCOUS) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      gml[0 + d] = rl[R_G + 3 * 1 + d];
      gml[3 + d] = rl[R_G + 3 * 2 + d];
      gml[6 + d] = rl[R_G + 3 * 3 + d];
      gml[9 + d] = rl[R_G + 3 * 8 + d];
    }
  }
  if (f >= a.nf_int) {
    // boundary face: right state = ghost of the cell-centre state, unlimited
    // (reconstruction.c:249-253); ghost gradient = interior gradient
    R qc[10];
#pragma unroll
    for (int j = 0; j < 8; ++j) qc[j] = rl[R_Q + j];
    qc[PR] = rl[R_P];
    qc[TT] = rl[R_T];
    const int region = a.fregion[f - a.nf_int];
    ghost_state(qc, region, n, t1, t2, a.pc, ph, qr);
    if (VISCOUS) {
      const int type = a.pc.region_type[region];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        gmr[3 * v] = gml[3 * v]; gmr[3 * v + 1] = gml[3 * v + 1]; gmr[3 * v + 2] = gml[3 * v + 2];
        ghost_gradient(type, n, t1, t2, &gmr[3 * v], &gmr[3 * v + 1], &gmr[3 * v + 2]);
      }
    }
  } else {
    const int c1 = a.fc1[f];
    R rr[REC];
    load_row<REC>(a.rec + (size_t)c1 * REC, rr);
    reconstruct<R, LINEAR, LIMIT>(rr, &go[G_D2], qr);
    if (VISCOUS) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        gmr[0 + d] = rr[R_G + 3 * 1 + d];
        gmr[3 + d] = rr[R_G + 3 * 2 + d];
        gmr[6 + d] = rr[R_G + 3 * 3 + d];
        gmr[9 + d] = rr[R_G + 3 * 8 + d];
      }
    }
  }
  R lr[10], rrot[10], fc[5];
  rotate_in(ql, n, t1, t2, ph, lr);
  rotate_in(qr, n, t1, t2, ph, rrot);
  if (ph.flux == 1) flux_rusanov(lr, rrot, ph, fc);
  else flux_ausm(lr, rrot, ph, fc);
  R out[5];
  out[0] = fc[0];
  out[1] = fc[1] * n[0] + fc[2] * t1[0] + fc[3] * t2[0];
  out[2] = fc[1] * n[1] + fc[2] * t1[1] + fc[3] * t2[1];
  out[3] = fc[1] * n[2] + fc[2] * t1[2] + fc[3] * t2[2];
  out[4] = fc[4];
  if (VISCOUS) {
    R fl[4], gl[4], hl[4], fr[4], gr[4], hr[4];
    viscous_side(ql, gml, n, ph, fl, gl, hl);
    viscous_side(qr, gmr, n, ph, fr, gr, hr);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      R fv = (R)0.5 * (fl[j] + fr[j]);
      R gv = (R)0.5 * (gl[j] + gr[j]);
      R hv = (R)0.5 * (hl[j] + hr[j]);
      out[j + 1] += fv * n[0] + gv * n[1] + hv * n[2];
    }
  }
  const R A = go[G_A];
  R* dst = a.FA + (size_t)f * FAS;
#pragma unroll
  for (int j = 0; j < 5; ++j) dst[j] = out[j] * A;
}

// ---------------------------------------------------------------------------
// K3: gather + update
// MODE 0: residual only (dphi = -sum/V)
// MODE 1: low-storage RK stage: k = R (+ a k); U += k dt g
// MODE 2: SSP-RK3 stage: U = c0 U0 + c1 (U + dt R)   (stage 0 saves U0)
// DT: also compute the running min of V / sum(|u|+c)dx of the new state
// ---------------------------------------------------------------------------
struct StageCoef {
  double a, g;        // low-storage coefficients
  double c0, c1;      // SSP combination
  int first;          // first stage of the step
  int last;           // last stage of the step
  int store_r;        // also store this stage's time derivative in dphi (the
                      // reference's dphi after a step: that of the last stage)
};

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w < v) ? w : v;
  }
  return v;
}

template <class R, int MODE, bool KAHAN, bool DT>
__global__ void __launch_bounds__(256) k_gather_update(const __grid_constant__ KArgs<R> a,
                                                       StageCoef co) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long lam_bits = 0x7ff0000000000000ull;  // +inf
  bool finite = true;
  if (c < a.nc) {
    Acc<R, KAHAN> s[5];
    for (int k = 0; k < a.mcf; ++k) {
      const int e = a.cface[(size_t)c * a.mcf + k];
      if (e < 0) break;
      const int f = e >> 1, side = e & 1;
      const R* src = a.FA + (size_t)f * FAS;
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        if (side) s[j].sub(src[j]);
        else s[j].add(src[j]);
      }
    }
    double r[5];
    if (sizeof(R) == 8) {
      const double V = a.vol[c];
#pragma unroll
      for (int j = 0; j < 5; ++j) r[j] = -(double)s[j].value() / V;
    } else {
      const R rv = a.rvol[c];
#pragma unroll
      for (int j = 0; j < 5; ++j) r[j] = (double)(-s[j].value() * rv);
    }
    if (MODE == 0 || co.store_r) {
#pragma unroll
      for (int j = 0; j < 5; ++j) a.dphi[(size_t)j * a.nc + c] = r[j];
    }
    if (MODE != 0) {
      const double dt = a.sc->dt;
      double u[5], uold[5];
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const size_t i = (size_t)j * a.nc + c;
        double uj = a.U[i];
        uold[j] = uj;
        if (MODE == 1) {
          double kj = co.first ? r[j] : r[j] + a.K[i] * co.a;
          a.K[i] = kj;
          uj += kj * dt * co.g;
        } else {
          if (co.first) {
            a.U0[i] = uj;
            uj = uj + dt * r[j];
          } else {
            uj = co.c0 * a.U0[i] + co.c1 * (uj + dt * r[j]);
          }
        }
        a.U[i] = uj;
        u[j] = uj;
        finite = finite && isfinite(uj);
      }
      if (sizeof(R) == 4 || DT) {
        // primitive recovery of the new state: FP32 shadow for the next
        // stage (mixed path) and the next CFL time step.  The reference's
        // step loop evaluates calc_ns_timestep on phi_total whose density is
        // already updated while u, v, w, p still hold the values of the last
        // stage's input (timestep_lserkw2 updates only the conserved entries,
        // explicit.c:136-139); the low-storage path reproduces that, SSP-RK3
        // (whose stepper refreshes the primitives) uses the new state.
        const double km1 = a.pc.km1;
        if (sizeof(R) == 4) {
          float4* sh = reinterpret_cast<float4*>(a.Uf) + 2 * (size_t)c;
          float4 o0 = sh[0], o1 = sh[1];  // stage-input shadow (rho, m, E, p, T)
          float rho = (float)u[0], mx = (float)u[1], my = (float)u[2], mz = (float)u[3];
          float vx = mx / rho, vy = my / rho, vz = mz / rho;
          float ke = 0.5f * (mx * vx + my * vy + mz * vz);
          float p = (float)(km1 * (u[4] - (double)ke));
          p = fmaxf(1.00E-10f, p);
          float T = p / (rho * (float)a.pc.R_mix);
          sh[0] = make_float4(rho, mx, my, mz);
          sh[1] = make_float4((float)u[4], p, T, 1.0f / rho);
          if (DT) {
            float pu = vx, pv = vy, pw = vz, pp = p;
            if (MODE == 1) { pu = o0.y / o0.x; pv = o0.z / o0.x; pw = o0.w / o0.x; pp = o1.y; }
            const float c_s = sqrtf((float)a.pc.kappa * pp / rho);
            const double* d = a.dx + 3 * (size_t)c;
            float ds = (fabsf(pu) + c_s) * (float)d[0] + (fabsf(pv) + c_s) * (float)d[1] +
                       (fabsf(pw) + c_s) * (float)d[2];
            double lam = (double)((float)a.vol[c] / ds);
            if (lam > 0.0) lam_bits = (unsigned long long)__double_as_longlong(lam);
          }
        } else if (DT) {
          double q[10];
          Phys<double> ph;
          ph.load(a.pc);
#pragma unroll
          for (int j = 0; j < 5; ++j) q[j] = (MODE == 1) ? uold[j] : u[j];
          cons_to_prims(q, ph);
          double s_rho = 1.0 / u[0];
          double c_s = sqrt(a.pc.kappa * q[PR] * s_rho);
          const double* d = a.dx + 3 * (size_t)c;
          double ds = (fabs(q[VU]) + c_s) * d[0] + (fabs(q[VV]) + c_s) * d[1] + (fabs(q[VW]) + c_s) * d[2];
          double lam = a.vol[c] / ds;
          if (lam > 0.0) lam_bits = (unsigned long long)__double_as_longlong(lam);
        }
      }
    }
  }
  if (MODE != 0) {
    if (!finite) atomicOr(&a.sc->status, 1);
    if (DT) {
      // min is exact and order independent: the result is deterministic
      lam_bits = warp_min_u64(lam_bits);
      if ((threadIdx.x & 31) == 0 && lam_bits != 0x7ff0000000000000ull)
        atomicMin(&a.sc->lam_bits, lam_bits);
    }
  }
}

}  // namespace fv3d
