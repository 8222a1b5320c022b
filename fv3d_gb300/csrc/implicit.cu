// Implicit steady solve on sm_103a: pseudo-transient Newton-Krylov.
//
//   (I/dt_i - dR/dU) dU = R(U),   U <- U + dU,   until ||R||/||R_0|| <= tol
//
// * R(U) is the FP64 residual (finite_volume_time_derivative semantics, the
//   FP64 kernels of kernels.cuh); norms and the Newton update in FP64.
// * Local time steps dt_i = CFL * V_i / sum_d (|u_d| + c) dx_d (the
//   convective formula of calc_ns_timestep, navier_stokes.c:171-187), CFL
//   ramped by switched evolution relaxation CFL = CFL_0 ||R_0|| / ||R||
//   clipped to [CFL_0, CFL_max].
// * Restarted flexible GMRES with FP64 Arnoldi (classical Gram-Schmidt with
//   one re-orthogonalisation, deterministic block reductions) and Givens
//   rotations on the host.  Matrix-free J v = (R(U + eps v) - R(U)) / eps,
//   from the FP32 residual (mixed kernels, eps scaled to FP32) or the FP64
//   residual (eps = 1e-7 relative).
// * Preconditioner: batched 5x5 block Jacobi.  Blocks are the exact
//   diagonal blocks of the first-order (cell-centre) discretisation - central
//   differences of each face's convective flux plus a two-point viscous flux
//   with respect to the cell's own state, ghost states re-derived from the
//   perturbed state - built in FP64, inverted, applied in FP32.  The
//   reference's lumped blocks (implicit.c:61-119: every cell perturbed at
//   once, eps = 1e-4 ||U_v||) are available as an alternative.
// The reference's own implicit step (a block-diagonal linearisation solved
// by basec's GMRES, implicit.c:224-351) is reproduced by the CPU oracle.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
#include "implicit.h"
#include "block5.cuh"
#include "fo_flux.cuh"
#include "gs_reduce.cuh"

namespace fv3d {

namespace {

constexpr int RED_BLOCKS = 608;   // fixed grid for deterministic reductions (4 per SM)
// resident Gram-Schmidt blocks per SM the register budget is cut for (FP32
// basis; an FP64 basis keeps 2 so that its 32-vector passes do not spill)
#ifndef FV3D_GS_MINBLOCKS
#define FV3D_GS_MINBLOCKS 4
#endif
// device coefficient slots: h1 [0, 32), h2 [32, 64), |w| and its derived
// scalars [64, 68), |z|, 1/|z|, eps, 1/eps [68, 72), a host norm [96, 100);
// FGMRES's y for the solution update at [0, k)
constexpr int kHostCoefs = 65;

inline int blocks(size_t n, int t = 256) { return (int)((n + t - 1) / t); }

// ---- vector kernels on N = 5 * nc doubles ---------------------------------
__global__ void k_lincomb(size_t n, double a, const double* __restrict__ x, double b,
                          const double* __restrict__ y, double* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = a * x[i] + b * (y ? y[i] : 0.0);
}

__device__ __forceinline__ float fmadd(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return fma(a, b, c); }

// Krylov vectors are T = double (FP64 Jacobian-vector products) or T =
// float (FP32 ones: basis, Gram-Schmidt and preconditioner in FP32, on the
// FP32 pipe); coefficients, norms and the Newton update stay FP64.

// partial[b][j] = sum over block b's elements of w_i V_j,i, j < k <= KMAX:
// one pass over w and the k vectors; products and sums in T (an FP32 basis
// is reduced in FP32: GB300's FP64 rate is a small fraction of its FP32
// rate), in a fixed order over a fixed grid, so deterministic
template <int KMAX, class T>
__global__ void __launch_bounds__(256) k_dots_partial(size_t n, const T* __restrict__ w, const T* __restrict__ V,
                                                      int k, T* __restrict__ partial) {
  __shared__ T sh[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T acc[KMAX];
#pragma unroll
  for (int j = 0; j < KMAX; ++j) acc[j] = T(0);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const T wi = w[i];
#pragma unroll
    for (int j = 0; j < KMAX; ++j)
      if (j < k) acc[j] = fmadd(wi, V[(size_t)j * n + i], acc[j]);
  }
#pragma unroll
  for (int j = 0; j < KMAX; ++j) {
    if (j >= k) break;
    T v = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32 && (int)threadIdx.x < k) {
    T s = T(0);
#pragma unroll
    for (int wv = 0; wv < 8; ++wv) s += sh[wv][threadIdx.x];
    partial[(size_t)blockIdx.x * 32 + threadIdx.x] = s;
  }
}

// out[j] = sum_b partial[b][j]: 32 warps stride the rows, then a
// fixed-order sum of the 32 warp results.  For a norm (take_sqrt, k = 1)
// out[0] = |w| and, from the one thread, out[1] = 1/|w|, out[2] = c/|w| and
// out[3] = |w|/c (each 0 when |w| = 0), so that no other kernel divides
template <class T>
__global__ void __launch_bounds__(1024) k_dots_final(int nb, int k, const T* __restrict__ partial,
                                                     double* __restrict__ out, int take_sqrt, double c) {
  __shared__ T sh[32][33];
  const int j = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T s = T(0);
  if (j < k)
    for (int b = warp; b < nb; b += 32) s += partial[(size_t)b * 32 + j];
  sh[warp][j] = s;
  __syncthreads();
  if (threadIdx.x < 32 && j < k) {
    T ts = T(0);
#pragma unroll
    for (int wv = 0; wv < 32; ++wv) ts += sh[wv][j];
    const double t = (double)ts;
    if (take_sqrt) {
      const double r = sqrt(t);
      out[0] = r;
      out[1] = (r > 0.0) ? 1.0 / r : 0.0;
      out[2] = (r > 0.0) ? c / r : 0.0;
      out[3] = (r > 0.0) ? r / c : 0.0;
    } else {
      out[j] = t;
    }
  }
}

// ---- 16-byte groups of basis elements ------------------------------------
// G consecutive elements: one 16-byte access when G * sizeof(T) == 16 (the
// address then 16-byte aligned: basis vectors start ldb elements apart, ldb
// a multiple of 64), else G scalar accesses
template <int G, class T>
__device__ __forceinline__ void ldg_group(const T* __restrict__ p, T* x) {
  if constexpr (G * sizeof(T) == 16) {
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
    memcpy(x, &u, 16);
  } else {
#pragma unroll
    for (int l = 0; l < G; ++l) x[l] = __ldg(p + l);
  }
}
template <class T>
__device__ __forceinline__ void ldg16(const T* __restrict__ p, T* x) {
  ldg_group<16 / sizeof(T)>(p, x);
}
// w is read and rewritten by the same thread: plain loads
template <int G, class T>
__device__ __forceinline__ void ld_group(const T* p, T* x) {
  if constexpr (G * sizeof(T) == 16) {
    const uint4 u = *reinterpret_cast<const uint4*>(p);
    memcpy(x, &u, 16);
  } else {
#pragma unroll
    for (int l = 0; l < G; ++l) x[l] = p[l];
  }
}
template <int G, class T>
__device__ __forceinline__ void st_group(T* p, const T* x) {
  if constexpr (G * sizeof(T) == 16) {
    uint4 u;
    memcpy(&u, x, 16);
    *reinterpret_cast<uint4*>(p) = u;
  } else {
#pragma unroll
    for (int l = 0; l < G; ++l) p[l] = x[l];
  }
}

// ---- fused Gram-Schmidt passes -------------------------------------------
// Classical Gram-Schmidt with one re-orthogonalisation in three passes over
// w and the k basis vectors; a pass with sums ends with a fixed-order
// reduction by the grid's last block (an atomic ticket; the block partials
// are summed in block order, so the result does not depend on which block
// is last):
//   PASS 1  h_j = w . V_j
//   PASS 2  w <- w - sum_j h_j V_j, then h'_j = w . V_j and |w|^2 of the
//           new w; the last block also forms |w - sum_j h'_j V_j| =
//           sqrt(|w|^2 - sum_j h'_j^2) (V orthonormal) and its inverse
//   PASS 3  v_{k+1} = (w - sum_j h'_j V_j) / that norm, no sums
//   PASS 0  |w| alone
//   PASS 4  h_j = w . V_j and |w|^2 (one Gram-Schmidt pass, for the inner
//           solves of the coupled preconditioner): the last block forms
//           |w - sum_j h_j V_j| by Pythagoras (the next vector is then
//           formed per cell by the coupled preconditioner's k_cpl_next)
// Products and sums in T (FP32 basis: FP32 pipe), the final sums and the
// coefficients in FP64 (gs_finalize, gs_reduce.cuh).

// w = z / dt_i - (R(U + eps z) - R(U)) / eps (k_jv_combine's arithmetic),
// formed inside the first Gram-Schmidt pass when z is set
template <class T>
struct JvArgs {
  const T* z = nullptr;
  const double* Rp = nullptr;
  const double* Rb = nullptr;
  const double* idt = nullptr;   // per cell
  const double* ieps = nullptr;  // device scalar 1/eps
  size_t nc = 0;
};

// one group of G consecutive elements i.. of a Gram-Schmidt pass: G = 16 /
// sizeof(T) with 16-byte loads (the main loop), G = 1 for the n % G tail.
// PASS 2 reads each V_j twice (for w - sum h_j V_j, then for the new dots):
// the second read finds the group in cache.  acc: PASS 1 / 2 the dots (and
// for PASS 2 |w|^2 at KMAX), PASS 0 the norm; PASS 3 writes vout * scale.
template <int KMAX, int PASS, int G, class T>
__device__ __forceinline__ void gs_group(T* __restrict__ w, const T* __restrict__ V, size_t ldb, size_t i, int k,
                                         const T* hs, T* acc, const JvArgs<T>& jv, T ieps, T* __restrict__ vout,
                                         T scale) {
  T wi[G];
  if (PASS == 1 && jv.z != nullptr) {
    T zi[G];
    ldg_group<G>(jv.z + i, zi);
#pragma unroll
    for (int l = 0; l < G; ++l) {
      const size_t e = i + l;
      const T id = (T)__ldg(jv.idt + e % jv.nc);
      wi[l] = zi[l] * id - (T)(__ldg(jv.Rp + e) - __ldg(jv.Rb + e)) * ieps;
    }
    st_group<G>(w + i, wi);
  } else {
    ld_group<G>(w + i, wi);
  }
  if (PASS == 0) {
#pragma unroll
    for (int l = 0; l < G; ++l) acc[0] = fmadd(wi[l], wi[l], acc[0]);
  } else if (PASS == 1 || PASS == 4) {
#pragma unroll
    for (int j = 0; j < KMAX; ++j)
      if (j < k) {
        T v[G];
        ldg_group<G>(V + (size_t)j * ldb + i, v);
#pragma unroll
        for (int l = 0; l < G; ++l) acc[j] = fmadd(wi[l], v[l], acc[j]);
      }
    if (PASS == 4) {
#pragma unroll
      for (int l = 0; l < G; ++l) acc[KMAX] = fmadd(wi[l], wi[l], acc[KMAX]);
    }
  } else {
    T sum[G];
#pragma unroll
    for (int l = 0; l < G; ++l) sum[l] = T(0);
#pragma unroll
    for (int j = 0; j < KMAX; ++j)
      if (j < k) {
        T v[G];
        ldg_group<G>(V + (size_t)j * ldb + i, v);
#pragma unroll
        for (int l = 0; l < G; ++l) sum[l] = fmadd(hs[j], v[l], sum[l]);
      }
    T wn[G];
#pragma unroll
    for (int l = 0; l < G; ++l) wn[l] = wi[l] - sum[l];
    if (PASS == 2) {
      st_group<G>(w + i, wn);
#pragma unroll
      for (int j = 0; j < KMAX; ++j)
        if (j < k) {
          T v[G];
          ldg_group<G>(V + (size_t)j * ldb + i, v);
#pragma unroll
          for (int l = 0; l < G; ++l) acc[j] = fmadd(wn[l], v[l], acc[j]);
        }
#pragma unroll
      for (int l = 0; l < G; ++l) acc[KMAX] = fmadd(wn[l], wn[l], acc[KMAX]);
    } else {
#pragma unroll
      for (int l = 0; l < G; ++l) wn[l] *= scale;
      st_group<G>(vout + i, wn);
    }
  }
}

template <int KMAX, int PASS, class T>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 2 : FV3D_GS_MINBLOCKS)
    k_gs(size_t n, size_t ldb, T* __restrict__ w, const T* __restrict__ V, int k, const double* __restrict__ h_in,
         T* __restrict__ partial, unsigned int* counter, double* __restrict__ out, double c,
         const double* __restrict__ c_dev, const JvArgs<T> jv, double* __restrict__ out2, T* __restrict__ vout,
         const double* __restrict__ scale_p) {
  static_assert(KMAX <= 32, "at most 32 basis vectors");
  if (c_dev != nullptr) c = *c_dev;  // the finite-difference scale, set per Newton step
  const T ieps = (PASS == 1 && jv.z != nullptr) ? (T)*jv.ieps : T(0);
  const T scale = (PASS == 3) ? (T)*scale_p : T(0);
  __shared__ T hs[32];
  __shared__ T sh[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (PASS >= 2 && threadIdx.x < 32) hs[threadIdx.x] = (threadIdx.x < (unsigned)k) ? (T)h_in[threadIdx.x] : T(0);
  __syncthreads();
  constexpr int NA = (PASS == 0 || PASS == 3) ? 1 : ((PASS == 2 || PASS == 4) ? KMAX + 1 : KMAX);
  constexpr int L = 16 / sizeof(T);
  T acc[NA];
#pragma unroll
  for (int j = 0; j < NA; ++j) acc[j] = T(0);
  const size_t stride = (size_t)gridDim.x * blockDim.x, gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t nq = n / L;
  for (size_t q = gid; q < nq; q += stride)
    gs_group<KMAX, PASS, L>(w, V, ldb, q * L, k, hs, acc, jv, ieps, vout, scale);
  for (size_t i = nq * L + gid; i < n; i += stride)
    gs_group<KMAX, PASS, 1>(w, V, ldb, i, k, hs, acc, jv, ieps, vout, scale);
  if (PASS == 3) return;  // no sums
  const int kk = (PASS == 0) ? 1 : k;
  // PASS 2: |w|^2 goes to column 31 (k <= 31 vectors use columns 0 .. 30)
#pragma unroll
  for (int j = 0; j < NA; ++j) {
    const bool take = ((PASS == 2 || PASS == 4) && j == KMAX) || j < kk;
    if (!take) continue;
    T v = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][((PASS == 2 || PASS == 4) && j == KMAX) ? 31 : j] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32 && ((int)threadIdx.x < kk || ((PASS == 2 || PASS == 4) && threadIdx.x == 31))) {
    T s = T(0);
#pragma unroll
    for (int wv = 0; wv < 8; ++wv) s += sh[wv][threadIdx.x];
    partial[(size_t)blockIdx.x * 32 + threadIdx.x] = s;
  }
  gs_finalize<T>(partial, gridDim.x, kk, out, PASS == 0, c, counter, (PASS == 2 || PASS == 4) ? out2 : nullptr);
}


// out = a x + b y (FP64 inputs) stored as T
template <class T>
__global__ void k_to_basis(size_t n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                           T* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (T)(a * x[i] + b * (y ? y[i] : 0.0));
}

// finite-difference state W = U + eps z (FP64), eps on the device
template <class T>
__global__ void k_fd_state(size_t n, const double* __restrict__ U, const T* __restrict__ z,
                           const double* __restrict__ eps, double* __restrict__ W) {
  const double e = *eps;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    W[i] = U[i] + e * (double)z[i];
}

// x += sum_j h_j Z_j in FP64 (the Newton correction from the basis, vectors
// ldb apart): 16-byte groups of Z per thread, then the n % L tail
template <class T>
__global__ void k_axpy_basis(size_t n, size_t ldb, double* __restrict__ x, const T* __restrict__ Z,
                             const double* __restrict__ h, int k) {
  constexpr int L = 16 / sizeof(T);
  __shared__ double hs[32];
  if (threadIdx.x < 32) hs[threadIdx.x] = (threadIdx.x < (unsigned)k) ? h[threadIdx.x] : 0.0;
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * blockDim.x, gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t nq = n / L;
  for (size_t q = gid; q < nq; q += stride) {
    double s[L];
#pragma unroll
    for (int l = 0; l < L; ++l) s[l] = 0.0;
#pragma unroll 4
    for (int j = 0; j < k; ++j) {
      T z[L];
      ldg16(Z + (size_t)j * ldb + q * L, z);
#pragma unroll
      for (int l = 0; l < L; ++l) s[l] = fma(hs[j], (double)z[l], s[l]);
    }
#pragma unroll
    for (int l = 0; l < L; ++l) x[q * L + l] += s[l];
  }
  for (size_t i = nq * L + gid; i < n; i += stride) {
    double s = 0.0;
    for (int j = 0; j < k; ++j) s = fma(hs[j], (double)Z[(size_t)j * ldb + i], s);
    x[i] += s;
  }
}

// local pseudo-time step per cell (FP64 convective formula)
__global__ void k_local_dt(int nc, const double* __restrict__ U, const double* __restrict__ vol,
                           const double* __restrict__ dx, double kappa, double km1, double cfl,
                           double* __restrict__ dtl, double* __restrict__ idtl) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double q[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) q[j] = U[(size_t)j * nc + c];
  const double ir = 1.0 / q[0];
  const double u = q[1] * ir, v = q[2] * ir, w = q[3] * ir;
  const double p = fmax(1.00E-10, km1 * (q[4] - 0.5 * (q[1] * u + q[2] * v + q[3] * w)));
  const double cs = sqrt(kappa * p * ir);
  const double* d = dx + 3 * (size_t)c;
  const double ds = (fabs(u) + cs) * d[0] + (fabs(v) + cs) * d[1] + (fabs(w) + cs) * d[2];
  dtl[c] = cfl * vol[c] / ds;
  idtl[c] = ds / (cfl * vol[c]);
}

// out = z / dt - (Rp - Rb) / eps per cell and variable; idt = 1/dt per
// cell, ieps = |z| / c = 1/eps on the device (0 for z = 0).  The difference
// of the two residuals is taken in FP64, the rest in T.
template <class T>
__global__ void k_jv_combine(int nc, const T* __restrict__ z, const double* __restrict__ Rp,
                             const double* __restrict__ Rb, const double* __restrict__ idt,
                             const double* __restrict__ ieps_p, T* __restrict__ out) {
  const T ieps = (T)*ieps_p;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const T id = (T)idt[c];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const size_t i = (size_t)j * nc + c;
      out[i] = z[i] * id - (T)(Rp[i] - Rb[i]) * ieps;
    }
  }
}


// FP32 state record (rho, m, E, p, T, 1/rho) of a cell's FP64 state w[5]
__device__ __forceinline__ void put_record(float* __restrict__ Uf, int c, const double* w, float km1, float R) {
  const float rho = (float)w[0], mx = (float)w[1], my = (float)w[2], mz = (float)w[3];
  const double E = w[4];
  const float ir = 1.f / rho;
  const float ke = 0.5f * (mx * mx + my * my + mz * mz) * ir;
  const float p = fmaxf(1.00E-10f, (float)((double)km1 * (E - (double)ke)));
  float4* d = reinterpret_cast<float4*>(Uf) + 2 * (size_t)c;
  d[0] = make_float4(rho, mx, my, mz);
  d[1] = make_float4((float)E, p, p * ir / R, ir);
}

// the records of the finite-difference state W = U + eps z (eps on the
// device), W itself not stored
template <class T>
__global__ void k_fd_record(int nc, const double* __restrict__ U, const T* __restrict__ z,
                            const double* __restrict__ eps, float* __restrict__ Uf, float km1, float R) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double e = *eps;
  double w[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) w[j] = U[(size_t)j * nc + c] + e * (double)z[(size_t)j * nc + c];
  put_record(Uf, c, w, km1, R);
}

// FP32 state record (rho, m, E, p, T, 1/rho) of an FP64 state W (renumbered SoA)
__global__ void k_make_record(int nc, const double* __restrict__ W, float* __restrict__ Uf,
                              float km1, float R) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const float rho = (float)W[c], mx = (float)W[(size_t)nc + c], my = (float)W[2 * (size_t)nc + c];
  const float mz = (float)W[3 * (size_t)nc + c];
  const double E = W[4 * (size_t)nc + c];
  const float ir = 1.f / rho;
  const float ke = 0.5f * (mx * mx + my * my + mz * mz) * ir;
  const float p = fmaxf(1.00E-10f, (float)((double)km1 * (E - (double)ke)));
  float4* d = reinterpret_cast<float4*>(Uf) + 2 * (size_t)c;
  d[0] = make_float4(rho, mx, my, mz);
  d[1] = make_float4((float)E, p, p * ir / R, ir);
}

// ---- first-order FD diagonal blocks ---------------------------------------
// D_c = I/dt_c + (1/V_c) sum_f d(F_f . n_out A_f)/dU_c  (column-major 5x5)
__global__ void k_fo_blocks(KArgs<double> a, const double* __restrict__ dtl,
                            const double* __restrict__ fdist, double* __restrict__ D) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nc) return;
  Phys<double> ph;
  ph.load(a.pc);
  double qc[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) qc[j] = a.U[(size_t)j * a.nc + c];
  double Dc[25];
#pragma unroll
  for (int j = 0; j < 25; ++j) Dc[j] = 0.0;
  for (int k = 0; k < a.mcf; ++k) {
    const int e = a.cface[(size_t)c * a.mcf + k];
    if (e < 0) break;
    const int f = e >> 1, side = e & 1;
    const double* g = a.geo + (size_t)f * GEO;
    const double sg = side ? -1.0 : 1.0;
    const double n[4] = {sg * g[G_N], sg * g[G_N + 1], sg * g[G_N + 2], fdist[f]};
    const double A = g[G_A];
    const bool bnd = f >= a.nf_int;
    double qo[10];
    if (!bnd) {
      const int o = side ? a.fc0[f] : a.fc1[f];
#pragma unroll
      for (int j = 0; j < 5; ++j) qo[j] = a.U[(size_t)j * a.nc + o];
    }
    for (int v = 0; v < 5; ++v) {
      const double h = 1e-7 * fmax(fabs(qc[v]), 1e-3 * fabs(qc[0]) + 1e-12);
      double Fp[5], Fm[5];
      for (int s = 0; s < 2; ++s) {
        double qp[10];
#pragma unroll
        for (int j = 0; j < 5; ++j) qp[j] = qc[j];
        qp[v] += s ? -h : h;
        if (bnd) {
          cons_to_prims(qp, ph);
          ghost_state(qp, a.fregion[f - a.nf_int], &g[G_N], &g[G_T1], &g[G_T2], a.pc, ph, qo);
        }
        fo_flux(qp, qo, n, a.pc, s ? Fm : Fp);
      }
      const double sc = A / (2.0 * h * a.vol[c]);
#pragma unroll
      for (int j = 0; j < 5; ++j) Dc[v * 5 + j] += (Fp[j] - Fm[j]) * sc;
    }
  }
  const double idt = 1.0 / dtl[c];
#pragma unroll
  for (int j = 0; j < 5; ++j) Dc[j * 5 + j] += idt;
#pragma unroll
  for (int j = 0; j < 25; ++j) D[(size_t)c * 25 + j] = Dc[j];
}

// lumped blocks (implicit.c:61-119): column v of -(R(U + e/2) - R(U - e/2)) / e
__global__ void k_perturb_all(int nc, const double* __restrict__ U, int v, double delta,
                              double* __restrict__ W) {
  const size_t n = 5 * (size_t)nc;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    W[i] = U[i] + ((i / nc == (size_t)v) ? delta : 0.0);
}

__global__ void k_lumped_column(int nc, int v, const double* __restrict__ Rp, const double* __restrict__ Rm,
                                double ieps, double* __restrict__ D) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
#pragma unroll
  for (int j = 0; j < 5; ++j)
    D[(size_t)c * 25 + v * 5 + j] = -(Rp[(size_t)j * nc + c] - Rm[(size_t)j * nc + c]) * ieps;
}

__global__ void k_add_diag(int nc, const double* __restrict__ dtl, double* __restrict__ D) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double idt = 1.0 / dtl[c];
#pragma unroll
  for (int j = 0; j < 5; ++j) D[(size_t)c * 25 + j * 5 + j] += idt;
}

// 5x5 inverse by Gauss-Jordan with partial pivoting (FP64, invert5),
// stored FP32; a singular block falls back to the inverse of its diagonal.
// Blocks column-major.
__global__ void __launch_bounds__(128) k_block_invert(int nc, const double* __restrict__ D, float* __restrict__ Dinv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double B[25], X[25];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) B[i * 5 + j] = D[(size_t)c * 25 + j * 5 + i];  // column-major -> row-major
  const bool ok = invert5(B, X);
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const double v = ok ? X[i * 5 + j] : ((i == j) ? 1.0 / B[i * 5 + i] : 0.0);
      Dinv[(size_t)c * 25 + j * 5 + i] = (float)v;  // column-major
    }
}

// z_c = Dinv_c v_c  (FP32 arithmetic)
template <class T>
__global__ void k_block_apply(int nc, const float* __restrict__ Dinv, const T* __restrict__ v,
                              T* __restrict__ z) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  float x[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) x[j] = (float)v[(size_t)j * nc + c];
  const float* M = Dinv + (size_t)c * 25;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 5; ++j) s = fmaf(M[j * 5 + i], x[j], s);
    z[(size_t)i * nc + c] = (T)s;
  }
}

// min density / pressure of a state (positivity check of a Newton update)
__global__ void k_min_rho_p(int nc, const double* __restrict__ U, double km1, unsigned long long* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long b = 0x7ff0000000000000ull;
  if (c < nc) {
    double q[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = U[(size_t)j * nc + c];
    const double p = km1 * (q[4] - 0.5 * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) / q[0]);
    const double m = fmin(q[0], p);
    b = (m > 0.0 && isfinite(m)) ? (unsigned long long)__double_as_longlong(m) : 0ull;
  }
  b = warp_min_u64(b);
  if ((threadIdx.x & 31) == 0) atomicMin(out, b);
}

// ---- the reference's implicit time step ------------------------------------
// f_Y = -(Y - Y_old0) / dt + b dY/dt - sum_s a_s / dt Y_old_s  (the newton
// right-hand side of implicit.c, in its operation order)
__global__ void k_newton_rhs(size_t n, const double* __restrict__ Y, const double* __restrict__ old0,
                             const double* __restrict__ old1, const double* __restrict__ dYdt, double dt, double b,
                             double a0, double a1, int stages, double* __restrict__ fY) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double f = -(Y[i] - old0[i]) / dt + b * dYdt[i];
    f -= a0 / dt * old0[i];
    if (stages > 1) f -= a1 / dt * old1[i];
    fY[i] = f;
  }
}

// column v of the lumped blocks (implicit.c:98-116): (-R(Y + e/2) + R(Y - e/2))
// * b / (eps + 1e-16), plus 1/dt on the diagonal; blocks column-major
__global__ void k_newton_column(int nc, int v, const double* __restrict__ Rp, const double* __restrict__ Rm,
                                double f, double idt, double* __restrict__ D) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    double x = -Rp[(size_t)j * nc + c];
    x += Rm[(size_t)j * nc + c];
    x *= f;
    if (j == v) x += idt;
    D[(size_t)c * 25 + v * 5 + j] = x;
  }
}

// x_c = D_c^{-1} b_c per cell (5x5, column-major, Gaussian elimination with
// partial pivoting in FP64); a singular block gives NaN (reported by the host)
__global__ void k_block_solve(int nc, const double* __restrict__ D, const double* __restrict__ b,
                              double* __restrict__ x) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double M[5][6];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
#pragma unroll
    for (int j = 0; j < 5; ++j) M[i][j] = D[(size_t)c * 25 + j * 5 + i];
    M[i][5] = b[(size_t)i * nc + c];
  }
  bool ok = true;
#pragma unroll
  for (int col = 0; col < 5; ++col) {
    int piv = col;
#pragma unroll
    for (int i = col + 1; i < 5; ++i)
      if (fabs(M[i][col]) > fabs(M[piv][col])) piv = i;
    if (!(fabs(M[piv][col]) > 0.0)) ok = false;
#pragma unroll
    for (int i = 0; i < 5; ++i)
      if (i == piv && piv != col)
#pragma unroll
        for (int j = 0; j < 6; ++j) { const double tmp = M[col][j]; M[col][j] = M[i][j]; M[i][j] = tmp; }
#pragma unroll
    for (int i = col + 1; i < 5; ++i) {
      const double l = M[i][col] / M[col][col];
#pragma unroll
      for (int j = col; j < 6; ++j) M[i][j] -= l * M[col][j];
    }
  }
  double y[5];
#pragma unroll
  for (int i = 4; i >= 0; --i) {
    double s = M[i][5];
#pragma unroll
    for (int j = i + 1; j < 5; ++j) s -= M[i][j] * y[j];
    y[i] = s / M[i][i];
  }
#pragma unroll
  for (int i = 0; i < 5; ++i) x[(size_t)i * nc + c] = ok ? y[i] : NAN;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
#define ICK(expr)                                               \
  do {                                                          \
    fv3d_status st__ = ctx.cuda((expr), #expr);                 \
    if (st__ != FV3D_OK) return st__;                           \
  } while (0)

fv3d_status Implicit::setup(Ctx& ctx, int m) {
  const size_t n = 5 * (size_t)ctx.nc;
  if (this->n == n && this->m >= m) return FV3D_OK;
  release_graphs();  // captured steps hold the old buffers
  this->n = n;
  this->m = m;
  ldb = (n + 63) / 64 * 64;
  auto al = [&](DevBuf<double>& b, size_t cnt) { return ctx.cuda(b.alloc(cnt), "implicit allocation"); };
  fv3d_status st;
  if ((st = al(w, n)) ||
      (st = al(R, n)) || (st = al(Rb, n)) || (st = al(Rp, n)) || (st = al(Wst, n)) || (st = al(x, n)) ||
      (st = al(dtl, (size_t)ctx.nc)) || (st = al(idtl, (size_t)ctx.nc)) || (st = al(D, 25 * (size_t)ctx.nc)) ||
      (st = al(part, (size_t)RED_BLOCKS * 32)) || (st = al(hdev, 128)) || (st = al(fdist, (size_t)ctx.nf)))
    return st;
  if (hpin == nullptr && (st = ctx.cuda(cudaMallocHost((void**)&hpin, sizeof(double) * kHostCoefs),
                                        "implicit host buffer")) != FV3D_OK)
    return st;
  if (hcols == nullptr && (st = ctx.cuda(cudaMallocHost((void**)&hcols, sizeof(double) * 32 * kHostCoefs),
                                         "implicit host buffer")) != FV3D_OK)
    return st;
  if ((st = ctx.cuda(Dinv.alloc(25 * (size_t)ctx.nc), "implicit allocation")) != FV3D_OK) return st;
  if ((st = ctx.cuda(bits.alloc(2), "implicit allocation")) != FV3D_OK) return st;
  // word 0: k_min_rho_p's minimum; word 1: the Gram-Schmidt passes' block ticket
  ICK(cudaMemset(bits.p, 0, 2 * sizeof(unsigned long long)));
  // face centre distances for the two-point viscous term
  std::vector<double> fd(ctx.nf);
  for (int f = 0; f < ctx.nf; ++f) {
    const double* g = &ctx.h_geo[(size_t)f * GEO];
    if (f < ctx.nf_int) {
      double s = 0.0;
      for (int d = 0; d < 3; ++d) s += (g[G_D1 + d] - g[G_D2 + d]) * (g[G_D1 + d] - g[G_D2 + d]);
      fd[f] = sqrt(s);
    } else {
      fd[f] = 2.0 * fabs(g[G_D1] * g[G_N] + g[G_D1 + 1] * g[G_N + 1] + g[G_D1 + 2] * g[G_N + 2]);
    }
  }
  ICK(cudaMemcpy(fdist.p, fd.data(), sizeof(double) * ctx.nf, cudaMemcpyHostToDevice));
  return FV3D_OK;
}

// the FP32 base and stage records of the state U, when the mixed arrays exist
// (the Jacobian-vector products overwrite the stage records)
static fv3d_status refresh_records(Ctx& ctx) {
  if (ctx.d_Uf.p == nullptr) return FV3D_OK;
  k_make_record<<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, ctx.d_U.p, ctx.d_Uf.p, ctx.phys.f32[1],
                                                        ctx.phys.f32[4]);
  ICK(cudaMemcpyAsync(ctx.d_UfN.p, ctx.d_Uf.p, sizeof(float) * 8 * (size_t)ctx.nc, cudaMemcpyDeviceToDevice,
                      ctx.stream));
  return FV3D_OK;
}

// R(state) in FP64 into `out`
static fv3d_status residual64(Ctx& ctx, const double* state, double* out) {
  KArgs<double> a = ctx.args<double>();
  a.U = const_cast<double*>(state);
  a.dphi = out;
  StageCoef co{0, 0, 0, 0, 1, 1};
  const Disc d = ctx.disc();
  ICK(launch_gradients<double>(a, d, ctx.stream));
  ICK(launch_face_flux<double>(a, d, ctx.stream));
  ICK(launch_gather<double>(a, 0, false, co, ctx.stream));
  return FV3D_OK;
}

// R(state) with the FP32 (mixed) kernels into `out`
// the FP32 residual of the state whose records are in Uf
static fv3d_status residual32_records(Ctx& ctx, double* out) {
  MxArgs a = ctx.mx_args();
  a.dphi = out;
  StageCoef co{0, 0, 0, 0, 1, 1};
  const Disc d = ctx.disc();
  ICK(launch_mx_sides(a, d, ctx.stream));
  ICK(launch_mx_flux_update(a, d, 0, false, co, ctx.stream));
  return FV3D_OK;
}

static fv3d_status residual32(Ctx& ctx, const double* state, double* out) {
  k_make_record<<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, state, ctx.d_Uf.p, ctx.phys.f32[1],
                                                        ctx.phys.f32[4]);
  ICK(cudaGetLastError());
  return residual32_records(ctx, out);
}

// k inner products w . V_j (j < k <= 32) into dst on the device, no host
// synchronisation; take_sqrt with V = w, k = 1 gives |w| (and the derived
// scalars of k_dots_final)
template <class T>
fv3d_status Implicit::dots_dev(Ctx& ctx, const T* wv, const T* Vb, int k, double* dst, bool take_sqrt, double c) {
  const int nb = std::min(RED_BLOCKS, blocks(n));
  T* pt = reinterpret_cast<T*>(part.p);  // sized for RED_BLOCKS x 32 doubles
  if (k <= 8) k_dots_partial<8, T><<<nb, 256, 0, ctx.stream>>>(n, wv, Vb, k, pt);
  else if (k <= 16) k_dots_partial<16, T><<<nb, 256, 0, ctx.stream>>>(n, wv, Vb, k, pt);
  else k_dots_partial<32, T><<<nb, 256, 0, ctx.stream>>>(n, wv, Vb, k, pt);
  k_dots_final<T><<<1, 1024, 0, ctx.stream>>>(nb, k, pt, dst, take_sqrt ? 1 : 0, c);
  ICK(cudaGetLastError());
  return FV3D_OK;
}

// one fused Gram-Schmidt pass (k_gs) over a fixed grid of RED_BLOCKS blocks
template <class T>
fv3d_status Implicit::gs_pass(Ctx& ctx, int pass, T* wv, const T* Vb, int k, const double* h_in, double* dst,
                              double c, const double* c_dev, const T* jv_z, double* dst2, T* vout,
                              const double* scale) {
  if ((pass == 2 || pass == 4) && k > 31)
    return ctx.fail(FV3D_ERR_INVALID_ARG, "Gram-Schmidt pass over %d > 31 vectors", k);
  JvArgs<T> jv;
  if (jv_z != nullptr) {
    jv.z = jv_z; jv.Rp = Rp.p; jv.Rb = Rb.p; jv.idt = idtl.p; jv.ieps = jv_ieps; jv.nc = (size_t)ctx.nc;
  }
  const int nb = std::min(RED_BLOCKS, blocks(n));
  T* pt = reinterpret_cast<T*>(part.p);
  unsigned int* ctr = reinterpret_cast<unsigned int*>(bits.p + 1);  // zero between passes
#define GS_LAUNCH(KM, P)                                                                                   \
  k_gs<KM, P, T><<<nb, 256, 0, ctx.stream>>>(n, ldb, wv, Vb, k, h_in, pt, ctr, dst, c, c_dev, jv, dst2, vout, \
                                             scale)
  if (pass == 0) GS_LAUNCH(1, 0);
  else if (pass == 3) { if (k <= 8) GS_LAUNCH(8, 3); else if (k <= 12) GS_LAUNCH(12, 3); else if (k <= 16) GS_LAUNCH(16, 3); else GS_LAUNCH(32, 3); }
  else if (pass == 1) { if (k <= 8) GS_LAUNCH(8, 1); else if (k <= 12) GS_LAUNCH(12, 1); else if (k <= 16) GS_LAUNCH(16, 1); else GS_LAUNCH(32, 1); }
  else if (pass == 4) { if (k <= 8) GS_LAUNCH(8, 4); else if (k <= 12) GS_LAUNCH(12, 4); else if (k <= 16) GS_LAUNCH(16, 4); else GS_LAUNCH(32, 4); }
  else { if (k <= 8) GS_LAUNCH(8, 2); else if (k <= 12) GS_LAUNCH(12, 2); else if (k <= 16) GS_LAUNCH(16, 2); else GS_LAUNCH(32, 2); }
#undef GS_LAUNCH
  ICK(cudaGetLastError());
  return FV3D_OK;
}

// |v| on the host (synchronises)
fv3d_status Implicit::norm(Ctx& ctx, const double* v, double* out) {
  fv3d_status st = dots_dev<double>(ctx, v, v, 1, hdev.p + 96, true, 1.0);
  if (st != FV3D_OK) return st;
  ICK(cudaMemcpyAsync(hpin, hdev.p + 96, sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
  ICK(cudaStreamSynchronize(ctx.stream));
  *out = hpin[0];
  return FV3D_OK;
}

// the cell-coupling preconditioner (coupled.cu) runs its inner Gram-Schmidt
// passes in FP32 and the norm of its input in the input's type
template fv3d_status Implicit::gs_pass<float>(Ctx&, int, float*, const float*, int, const double*, double*, double,
                                              const double*, const float*, double*, float*, const double*);
template fv3d_status Implicit::gs_pass<double>(Ctx&, int, double*, const double*, int, const double*, double*,
                                               double, const double*, const double*, double*, double*,
                                               const double*);

template <class T>
fv3d_status Implicit::precondition(Ctx& ctx, const T* v, T* z) {
  if (opts.preconditioner == FV3D_PC_LEARNED && !use_fallback) return ctx.mlp->apply(ctx, v, z);
  if (opts.preconditioner == FV3D_PC_COUPLED || (opts.preconditioner == FV3D_PC_LEARNED &&
                                                 opts.fallback == FV3D_PC_COUPLED))
    return coupled->apply<T>(ctx, *this, v, z);
  if (opts.preconditioner == FV3D_PC_NONE) {
    if (z != v) ICK(cudaMemcpyAsync(z, v, sizeof(T) * n, cudaMemcpyDeviceToDevice, ctx.stream));
    return FV3D_OK;
  }
  k_block_apply<T><<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, Dinv.p, v, z);
  ICK(cudaGetLastError());
  return FV3D_OK;
}

// w = (I/dt - J) z: the step eps = rel (1 + |U|) / |z| is formed on the
// device, so a Jacobian-vector product needs no host synchronisation
// R(U + eps z) into Rp with eps = c/|z|, c = rel (1 + |U|) from its device
// slot (set each Newton step), so captured iterations stay valid; a unit z
// (an unpreconditioned basis vector, |v_k| = 1) takes eps = c without a
// norm pass.  Sets jv_ieps to the device slot holding 1/eps.
template <class T>
fv3d_status Implicit::fd_residual(Ctx& ctx, const T* z, bool unit) {
  const double* eps = hdev.p + 100;
  jv_ieps = hdev.p + 101;
  if (!unit) {
    fv3d_status st = gs_pass<T>(ctx, 0, const_cast<T*>(z), z, 1, nullptr, hdev.p + 68, 0.0, hdev.p + 100);
    if (st != FV3D_OK) return st;
    eps = hdev.p + 70;
    jv_ieps = hdev.p + 71;
  }
  if (opts.jv_precision >= 1) {
    k_fd_record<T><<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, ctx.d_U.p, z, eps, ctx.d_Uf.p, ctx.phys.f32[1],
                                                          ctx.phys.f32[4]);
    ICK(cudaGetLastError());
    return residual32_records(ctx, Rp.p);
  }
  k_fd_state<T><<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(n, ctx.d_U.p, z, eps, Wst.p);
  ICK(cudaGetLastError());
  return residual64(ctx, Wst.p, Rp.p);
}

// w = (I/dt - J) z: the step eps is formed on the device, so a
// Jacobian-vector product needs no host synchronisation
template <class T>
fv3d_status Implicit::apply_A(Ctx& ctx, const T* z, T* out) {
  fv3d_status st = fd_residual<T>(ctx, z, false);
  if (st != FV3D_OK) return st;
  k_jv_combine<T><<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, z, Rp.p, Rb.p, idtl.p, jv_ieps, out);
  ICK(cudaGetLastError());
  return FV3D_OK;
}

fv3d_status Implicit::build_blocks(Ctx& ctx) {
  // no preconditioner: no blocks, unless a harvest wants them as features
  const bool harvesting = ctx.mlp && ctx.mlp->ready && ctx.mlp->harvest_per_step > 0;
  if (opts.preconditioner == FV3D_PC_NONE && !harvesting) return FV3D_OK;
  if (opts.preconditioner == FV3D_PC_COUPLED ||
      (opts.preconditioner == FV3D_PC_LEARNED && opts.fallback == FV3D_PC_COUPLED)) {
    if (coupled == nullptr) coupled = new Coupled();
    fv3d_status st = coupled->setup(ctx, *this, opts.inner_dim, opts.inner_sweeps, (float)opts.inner_omega);
    if (st == FV3D_OK) st = coupled->build(ctx, *this);
    if (st != FV3D_OK || opts.preconditioner == FV3D_PC_COUPLED) return st;
  }
  if (opts.preconditioner == FV3D_PC_LUMPED) {
    // every cell perturbed at once by +-eps/2, eps = 1e-4 ||U_v||_2 (implicit.c:65-117)
    std::vector<double> slice(ctx.nc);
    for (int v = 0; v < 5; ++v) {
      ICK(cudaMemcpyAsync(slice.data(), ctx.d_U.p + (size_t)v * ctx.nc, sizeof(double) * ctx.nc,
                          cudaMemcpyDeviceToHost, ctx.stream));
      ICK(cudaStreamSynchronize(ctx.stream));
      double s = 0.0;
      for (int c = 0; c < ctx.nc; ++c) s += slice[c] * slice[c];
      const double eps = sqrt(s) * 1e-4;
      k_perturb_all<<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(ctx.nc, ctx.d_U.p, v, 0.5 * eps, Wst.p);
      fv3d_status st = residual64(ctx, Wst.p, Rp.p);
      if (st != FV3D_OK) return st;
      k_perturb_all<<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(ctx.nc, ctx.d_U.p, v, -0.5 * eps, Wst.p);
      st = residual64(ctx, Wst.p, w.p);
      if (st != FV3D_OK) return st;
      k_lumped_column<<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, v, Rp.p, w.p, 1.0 / (eps + 1e-16), D.p);
    }
    k_add_diag<<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, dtl.p, D.p);
  } else {
    k_fo_blocks<<<blocks(ctx.nc, 128), 128, 0, ctx.stream>>>(ctx.args<double>(), dtl.p, fdist.p, D.p);
  }
  ICK(cudaGetLastError());
  k_block_invert<<<blocks(ctx.nc, 128), 128, 0, ctx.stream>>>(ctx.nc, D.p, Dinv.p);
  ICK(cudaGetLastError());
  if (ctx.mlp && ctx.mlp->ready && (opts.preconditioner == FV3D_PC_LEARNED || ctx.mlp->harvest_per_step > 0))
    return ctx.mlp->build_features(ctx, *this);
  return FV3D_OK;
}

// restarted FGMRES(m) for (I/dt - J) x = R, x0 = 0; returns iterations
// one Arnoldi step k: z_k = M v_k, w = A z_k, classical Gram-Schmidt twice,
// |w| and v_{k+1} = w / |w| on the device, the Hessenberg column copied to
// the pinned host buffer.  Replayed from a CUDA graph per (k, preconditioner
// kind) once captured: every scalar it needs lives in device memory.
template <class T>
fv3d_status Implicit::enqueue_arnoldi(Ctx& ctx, T* Vt, T* Zt, T* wt, int k) {
  T* vk = Vt + (size_t)k * ldb;
  T* zk = (opts.preconditioner == FV3D_PC_NONE) ? vk : Zt + (size_t)k * ldb;  // unpreconditioned: z_k = v_k
  fv3d_status st = precondition<T>(ctx, vk, zk);
  if (st != FV3D_OK) return st;
  // w = A z_k formed inside the first Gram-Schmidt pass
  if ((st = fd_residual<T>(ctx, zk, opts.preconditioner == FV3D_PC_NONE)) != FV3D_OK) return st;
  if ((st = gs_pass<T>(ctx, 1, wt, Vt, k + 1, nullptr, hdev.p, 0.0, nullptr, zk)) != FV3D_OK) return st;
  // h' into slots 32.., |w - V h'| and its inverse into 64, 65
  if ((st = gs_pass<T>(ctx, 2, wt, Vt, k + 1, hdev.p, hdev.p + 32, 0.0, nullptr, nullptr, hdev.p + 64)) != FV3D_OK)
    return st;
  // v_{k+1} = (w - V h') / |w - V h'|
  if ((st = gs_pass<T>(ctx, 3, wt, Vt, k + 1, hdev.p + 32, nullptr, 0.0, nullptr, nullptr, nullptr,
                       Vt + (size_t)(k + 1) * ldb, hdev.p + 65)) != FV3D_OK)
    return st;
  ICK(cudaMemcpyAsync(hcols + (size_t)k * kHostCoefs, hdev.p, sizeof(double) * kHostCoefs, cudaMemcpyDeviceToHost,
                      ctx.stream));
  return FV3D_OK;
}

template <class T>
fv3d_status Implicit::arnoldi_step(Ctx& ctx, T* Vt, T* Zt, T* wt, int k) {
  const int pc = (opts.preconditioner == FV3D_PC_LEARNED && use_fallback) ? opts.fallback : opts.preconditioner;
  const long long key = (((long long)k * 8 + pc) * 2 + (sizeof(T) == 4 ? 1 : 0)) * 3 + opts.jv_precision;
  auto it = arnoldi_graphs.find(key);
  if (it == arnoldi_graphs.end()) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    ICK(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
    fv3d_status st = enqueue_arnoldi<T>(ctx, Vt, Zt, wt, k);
    cudaError_t ce = cudaStreamEndCapture(ctx.stream, &g);
    if (st != FV3D_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    ICK(ce);
    ce = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    ICK(ce);
    it = arnoldi_graphs.emplace(key, exec).first;
  }
  ICK(cudaGraphLaunch(it->second, ctx.stream));
  jv_count += 1;
  return FV3D_OK;
}

void Implicit::release_graphs() {
  for (auto& kv : arnoldi_graphs) cudaGraphExecDestroy(kv.second);
  arnoldi_graphs.clear();
}

// restarted flexible GMRES on the Newton system with basis V, Z and work
// vector wt of type T (FP32 for FP32 Jacobian-vector products)
template <class T>
fv3d_status Implicit::fgmres_t(Ctx& ctx, T* Vt, T* Zt, T* wt, double rnorm, int* iters, double* rel_res) {
  const int m = opts.krylov_dim;
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  ICK(cudaMemsetAsync(x.p, 0, sizeof(double) * n, ctx.stream));
  int total = 0;
  double res = rnorm;
  for (int cyc = 0; cyc <= std::max(0, opts.max_restarts); ++cyc) {
    double beta = rnorm;
    if (cyc == 0) {
      k_to_basis<T><<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(n, 1.0 / rnorm, R.p, 0.0, nullptr, Vt);
    } else {
      // true residual of the current iterate: R - A x (in FP64)
      fv3d_status st = apply_A<double>(ctx, x.p, w.p);
      if (st != FV3D_OK) return st;
      jv_count += 1;
      k_lincomb<<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(n, 1.0, R.p, -1.0, w.p, Rp.p);
      if ((st = norm(ctx, Rp.p, &beta)) != FV3D_OK) return st;
      if (!(beta > opts.eta * rnorm)) { res = beta; break; }
      k_to_basis<T><<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(n, 1.0 / beta, Rp.p, 0.0, nullptr, Vt);
    }
    ICK(cudaGetLastError());
    std::fill(H.begin(), H.end(), 0.0);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    bool done = false;
    // chunks of Arnoldi steps run back to back on the device, their
    // coefficients processed after one synchronisation
    // 0: 3 Arnoldi steps a chunk with the coupled preconditioner (each step
    // costs about 0.8 ms, so unused ones at the end of a cycle are dear), 10 otherwise
    const int chunk = opts.sync_every > 0 ? opts.sync_every : (opts.preconditioner == FV3D_PC_COUPLED ? 3 : 10);
    for (int k1 = 0; k < m && !done;) {
      k1 = std::min(m, k + chunk);
      for (int j = k; j < k1; ++j) {
        fv3d_status st = arnoldi_step<T>(ctx, Vt, Zt, wt, j);
        if (st != FV3D_OK) return st;
      }
      ICK(cudaStreamSynchronize(ctx.stream));
      for (; k < k1; ++k) {
        const double* hc = hcols + (size_t)k * kHostCoefs;
        const double hn = hc[64];
        for (int j = 0; j <= k; ++j) H[(size_t)k * (m + 1) + j] = hc[j] + hc[32 + j];
        H[(size_t)k * (m + 1) + k + 1] = hn;
        // Givens rotations on the new column
        for (int j = 0; j < k; ++j) {
          const double a = H[(size_t)k * (m + 1) + j], b = H[(size_t)k * (m + 1) + j + 1];
          H[(size_t)k * (m + 1) + j] = cs[j] * a + sn[j] * b;
          H[(size_t)k * (m + 1) + j + 1] = -sn[j] * a + cs[j] * b;
        }
        const double a = H[(size_t)k * (m + 1) + k], b = H[(size_t)k * (m + 1) + k + 1];
        const double r = sqrt(a * a + b * b);
        // a preconditioned direction with no component (a zero or non-finite
        // preconditioner output): stop without it, leaving the residual unreduced
        if (!(r > 0.0) || !std::isfinite(r)) { res = fabs(g[k]); done = true; break; }
        cs[k] = (r > 0.0) ? a / r : 1.0;
        sn[k] = (r > 0.0) ? b / r : 0.0;
        H[(size_t)k * (m + 1) + k] = r;
        H[(size_t)k * (m + 1) + k + 1] = 0.0;
        g[k + 1] = -sn[k] * g[k];
        g[k] = cs[k] * g[k];
        res = fabs(g[k + 1]);
        if (res <= opts.eta * rnorm || !(hn > 0.0)) { ++k; done = true; break; }
      }
    }
    for (int i = k - 1; i >= 0; --i) {
      double s = g[i];
      for (int j = i + 1; j < k; ++j) s -= H[(size_t)j * (m + 1) + i] * y[j];
      y[i] = s / H[(size_t)i * (m + 1) + i];
    }
    // x += Z y
    ICK(cudaMemcpyAsync(hdev.p, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, ctx.stream));
    k_axpy_basis<T><<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(
        n, ldb, x.p, opts.preconditioner == FV3D_PC_NONE ? Vt : Zt, hdev.p, k);
    ICK(cudaGetLastError());
    total += k;
    if (done) break;
  }
  *iters = total;
  *rel_res = res / rnorm;
  return FV3D_OK;
}

fv3d_status Implicit::fgmres(Ctx& ctx, double rnorm, int* iters, double* rel_res) {
  if (opts.jv_precision == 1) return fgmres_t<float>(ctx, V32.p, Z32.p, w32.p, rnorm, iters, rel_res);
  return fgmres_t<double>(ctx, V.p, Z.p, w.p, rnorm, iters, rel_res);
}

fv3d_status Implicit::solve(Ctx& ctx, const fv3d_implicit_opts& o, fv3d_implicit_stats* stats) {
  opts = o;
  if (opts.krylov_dim < 1 || opts.krylov_dim > 31) return ctx.fail(FV3D_ERR_INVALID_ARG, "krylov_dim must be 1..31");
  // the coupled preconditioner keeps its quality over a few Newton steps: on
  // the 96x48x48 channel rebuilt every 1 / 2 / 3 / 4 / 6 steps it takes 680 /
  // 681 / 681 / 711 / 741 Krylov iterations (530 / 519 / 516 / 542 / 559 ms)
  if (opts.pc_refresh <= 0) opts.pc_refresh = (opts.preconditioner == FV3D_PC_COUPLED) ? 3 : 1;
  if (opts.preconditioner == FV3D_PC_LEARNED && opts.fallback != FV3D_PC_COUPLED)
    opts.fallback = FV3D_PC_BLOCK_JACOBI;
  if (opts.preconditioner == FV3D_PC_COUPLED ||
      (opts.preconditioner == FV3D_PC_LEARNED && opts.fallback == FV3D_PC_COUPLED)) {
    if (opts.inner_dim == 0) opts.inner_dim = 10;
    if (opts.inner_sweeps == 0) opts.inner_sweeps = 2;
    if (opts.inner_omega == 0.0) opts.inner_omega = 0.7;
    if (opts.inner_dim < 1 || opts.inner_dim > 30 || opts.inner_sweeps < 1 || opts.inner_sweeps > 8 ||
        !(opts.inner_omega > 0.0 && opts.inner_omega <= 2.0))
      return ctx.fail(FV3D_ERR_INVALID_ARG, "inner_dim must be 1..30, inner_sweeps 1..8, inner_omega in (0, 2]");
  }
  if (opts.preconditioner == FV3D_PC_LEARNED && !(ctx.mlp && ctx.mlp->ready))
    return ctx.fail(FV3D_ERR_STATE, "learned preconditioner requested but no MLP initialised");
  fv3d_status st = ensure_fp64_path(ctx);
  if (st == FV3D_OK && opts.jv_precision >= 1) st = ensure_mixed_path(ctx);
  if (st == FV3D_OK) st = setup(ctx, opts.krylov_dim);
  if (st != FV3D_OK) return st;
  // Krylov basis: FP32 with jv_precision 1, FP64 otherwise (2: FP32 products, FP64 Arnoldi)
  {
    const size_t nv = (size_t)(opts.krylov_dim + 1) * ldb, nz = (size_t)opts.krylov_dim * ldb;
    cudaError_t e = cudaSuccess;
    if ((opts.jv_precision == 1 && (V32.n < nv || Z32.n < nz || w32.n < n)) ||
        (opts.jv_precision != 1 && (V.n < nv || Z.n < nz)))
      release_graphs();  // captured steps hold the old basis
    if (opts.jv_precision == 1) {
      if (V32.n < nv) e = V32.alloc(nv);
      if (e == cudaSuccess && Z32.n < nz) e = Z32.alloc(nz);
      if (e == cudaSuccess && w32.n < n) e = w32.alloc(n);
    } else {
      if (V.n < nv) e = V.alloc(nv);
      if (e == cudaSuccess && Z.n < nz) e = Z.alloc(nz);
    }
    if ((st = ctx.cuda(e, "Krylov basis allocation")) != FV3D_OK) return st;
  }
  history.clear();
  jv_count = 0;
  const auto t0 = std::chrono::steady_clock::now();
  double res0 = 0.0, res = 0.0, cfl = opts.cfl_start;
  int newton = 0, gmres_total = 0, rejected = 0, fallbacks = 0;
  bool converged = false;
  for (newton = 0; newton <= opts.max_newton; ++newton) {
    if ((st = residual64(ctx, ctx.d_U.p, R.p)) != FV3D_OK) return st;
    if ((st = norm(ctx, R.p, &res)) != FV3D_OK) return st;
    if (!std::isfinite(res)) return ctx.fail(FV3D_ERR_NONFINITE, "non-finite residual at Newton step %d", newton);
    if (newton == 0) res0 = res;
    history.push_back(res);
    if (res <= opts.tol_rel * res0 || res == 0.0) { converged = true; break; }
    if (newton == opts.max_newton) break;
    if (newton > 0) cfl = std::min(opts.cfl_max, std::max(opts.cfl_start, opts.cfl_start * res0 / res));
    if ((st = norm(ctx, ctx.d_U.p, &unorm)) != FV3D_OK) return st;
    {
      // c = rel (1 + |U|) for the finite-difference steps of this Newton step
      const double rel = (opts.jv_precision >= 1) ? 5e-4 : opts.fd_eps;
      hpin[0] = rel * (1.0 + unorm);
      hpin[1] = 1.0 / hpin[0];
      ICK(cudaMemcpyAsync(hdev.p + 100, hpin, 2 * sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
      ICK(cudaStreamSynchronize(ctx.stream));
    }
    // Newton step with a CFL back-off on failure
    for (int attempt = 0; attempt < 6; ++attempt) {
      k_local_dt<<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, ctx.d_U.p, ctx.d_vol.p, ctx.d_dx.p,
                                                        ctx.cfg.kappa, ctx.phys.km1, cfl, dtl.p, idtl.p);
      ICK(cudaGetLastError());
      if (newton % std::max(1, opts.pc_refresh) == 0 || attempt > 0) {
        if ((st = build_blocks(ctx)) != FV3D_OK) return st;
      }
      if (opts.jv_precision >= 1) st = residual32(ctx, ctx.d_U.p, Rb.p);
      else st = ICK_copy(ctx, Rb.p, R.p);
      if (st != FV3D_OK) return st;
      int it = 0;
      double rr = 0.0;
      use_fallback = false;
      if ((st = fgmres(ctx, res, &it, &rr)) != FV3D_OK) return st;
      gmres_total += it;
      if (opts.preconditioner == FV3D_PC_LEARNED && !(rr <= 0.5)) {
        // stagnation with the learned preconditioner: redo with block Jacobi
        use_fallback = true;
        fallbacks += 1;
        if ((st = fgmres(ctx, res, &it, &rr)) != FV3D_OK) return st;
        gmres_total += it;
      }
      if (ctx.mlp && ctx.mlp->ready && ctx.mlp->harvest_per_step > 0 && attempt == 0) {
        if ((st = ctx.mlp->harvest(ctx, *this)) != FV3D_OK) return st;
      }
      // trial state
      k_lincomb<<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(n, 1.0, ctx.d_U.p, 1.0, x.p, Wst.p);
      ICK(cudaMemsetAsync(bits.p, 0xff, sizeof(unsigned long long), ctx.stream));
      k_min_rho_p<<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, Wst.p, ctx.phys.km1, bits.p);
      ICK(cudaGetLastError());
      unsigned long long mb = 0;
      ICK(cudaMemcpyAsync(&mb, bits.p, sizeof(mb), cudaMemcpyDeviceToHost, ctx.stream));
      ICK(cudaStreamSynchronize(ctx.stream));
      if (mb != 0ull) {
        ICK(cudaMemcpyAsync(ctx.d_U.p, Wst.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx.stream));
        break;
      }
      rejected += 1;
      cfl = std::max(1.0, cfl * 0.1);
      if (attempt == 5) return ctx.fail(FV3D_ERR_NOT_CONVERGED, "Newton update not admissible at step %d", newton);
    }
  }
  if ((st = refresh_records(ctx)) != FV3D_OK) return st;
  ICK(cudaStreamSynchronize(ctx.stream));
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats != nullptr) {
    stats->newton_steps = newton;
    stats->gmres_iterations = gmres_total;
    stats->jv_evaluations = jv_count;
    stats->rejected_steps = rejected;
    stats->fallbacks = fallbacks;
    stats->res0 = res0;
    stats->res_final = res;
    stats->rel_res = (res0 > 0.0) ? res / res0 : 0.0;
    stats->wall_ms = ms;
    stats->cfl_final = cfl;
    stats->converged = converged ? 1 : 0;
  }
  ctx.state_ready = true;
  ctx.residual_valid = false;
  if (!converged) return ctx.fail(FV3D_ERR_NOT_CONVERGED, "relative residual %.3e after %d Newton steps", res / res0, newton);
  return FV3D_OK;
}

fv3d_status Implicit::newton_buffers(Ctx& ctx) {
  fv3d_status st = ensure_fp64_path(ctx);
  if (st == FV3D_OK) st = setup(ctx, 1);
  if (st != FV3D_OK) return st;
  cudaError_t e = cudaSuccess;
  for (DevBuf<double>* b : {&old0, &old1, &dYdt, &fY})
    if (e == cudaSuccess && b->n < n) e = b->alloc(n);
  return ctx.cuda(e, "implicit step allocation");
}

// read_restart_data's phi_old (restart.c:50-178) and the time derivative of
// the restart state (the file's phi_dt)
fv3d_status Implicit::set_history(Ctx& ctx, int scheme, int n_stages, const double* rows) {
  const int want = (scheme == FV3D_NEWTON_EULER) ? 1 : 2;
  if (n_stages != want)
    return ctx.fail(FV3D_ERR_INVALID_ARG, "%d history stages for a scheme that keeps %d", n_stages, want);
  fv3d_status st = newton_buffers(ctx);
  if (st != FV3D_OK) return st;
  ICK(cudaMemsetAsync(old1.p, 0, sizeof(double) * n, ctx.stream));
  if ((st = import_rows(ctx, rows, old0.p)) != FV3D_OK) return st;
  if (n_stages > 1 && (st = import_rows(ctx, rows + 5 * (size_t)ctx.nc, old1.p)) != FV3D_OK) return st;
  if ((st = residual64(ctx, ctx.d_U.p, dYdt.p)) != FV3D_OK) return st;
  ICK(cudaStreamSynchronize(ctx.stream));
  n_bdf = want;
  newton_ready = true;
  return FV3D_OK;
}

// timestep_newton (implicit.c:224-351): U is the state Y; R(U) the FP64
// time derivative; ten perturbed residuals build the lumped blocks each
// Newton iteration; the block-diagonal system is solved cell by cell
fv3d_status Implicit::step_newton(Ctx& ctx, const fv3d_newton_opts& o, int iter, double t, double dt,
                                  fv3d_newton_stats* stats) {
  (void)t;  // the implemented boundary conditions do not depend on time
  if (!newton_ready && iter >= 1 && o.scheme == FV3D_NEWTON_BDF2)
    return ctx.fail(FV3D_ERR_STATE, "BDF2 step at iteration %d without the history of the steps before it", iter);
  fv3d_status st = newton_buffers(ctx);
  if (st != FV3D_OK) return st;
  const int grid = std::min(4096, blocks(n));
  double* U = ctx.d_U.p;
  if (!newton_ready || iter == 0) {
    n_bdf = (o.scheme == FV3D_NEWTON_EULER) ? 1 : 2;
    ICK(cudaMemsetAsync(old0.p, 0, sizeof(double) * n, ctx.stream));
    ICK(cudaMemsetAsync(old1.p, 0, sizeof(double) * n, ctx.stream));
    if ((st = residual64(ctx, U, dYdt.p)) != FV3D_OK) return st;  // time derivative at t
    newton_ready = true;
  }
  const bool start = iter < n_bdf;
  const int stages = start ? 1 : n_bdf;
  const double a0 = (start || o.scheme == FV3D_NEWTON_EULER) ? 0.0 : -1. / 3.;
  const double a1 = (start || o.scheme == FV3D_NEWTON_EULER) ? 0.0 : 1 / 3.;
  const double bb = (start || o.scheme == FV3D_NEWTON_EULER) ? 1.0 : 2. / 3.;
  if (stages > 1) ICK(cudaMemcpyAsync(old1.p, old0.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx.stream));
  ICK(cudaMemcpyAsync(old0.p, U, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx.stream));
  k_newton_rhs<<<grid, 256, 0, ctx.stream>>>(n, U, old0.p, old1.p, dYdt.p, dt, bb, a0, a1, stages, fY.p);
  ICK(cudaGetLastError());
  double err0 = 0.0, err = 0.0;
  if ((st = norm(ctx, fY.p, &err0)) != FV3D_OK) return st;
  err = err0;
  std::vector<double> slice(ctx.nc);
  int it;
  for (it = 1; it <= o.max_iter_inner; ++it) {
    // lumped Jacobian (implicit.c:65-117); eps from the variable's norm in
    // reference cell order
    for (int v = 0; v < 5; ++v) {
      ICK(cudaMemcpyAsync(slice.data(), U + (size_t)v * ctx.nc, sizeof(double) * ctx.nc, cudaMemcpyDeviceToHost,
                          ctx.stream));
      ICK(cudaStreamSynchronize(ctx.stream));
      double s2 = 0.0;
      for (int i = 0; i < ctx.nc; ++i) s2 += slice[ctx.iperm[i]] * slice[ctx.iperm[i]];
      const double eps = sqrt(s2) * 1e-4;
      k_perturb_all<<<grid, 256, 0, ctx.stream>>>(ctx.nc, U, v, 0.5 * eps, Wst.p);
      if ((st = residual64(ctx, Wst.p, Rp.p)) != FV3D_OK) return st;
      k_perturb_all<<<grid, 256, 0, ctx.stream>>>(ctx.nc, U, v, -0.5 * eps, Wst.p);
      if ((st = residual64(ctx, Wst.p, w.p)) != FV3D_OK) return st;
      k_newton_column<<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, v, Rp.p, w.p, bb / (eps + 1e-16), 1.0 / dt,
                                                              D.p);
    }
    ICK(cudaGetLastError());
    if (err >= err0) {
      k_block_solve<<<blocks(ctx.nc, 128), 128, 0, ctx.stream>>>(ctx.nc, D.p, fY.p, x.p);
      k_lincomb<<<grid, 256, 0, ctx.stream>>>(n, 1.0, U, 1.0, x.p, Wst.p);
      ICK(cudaMemcpyAsync(U, Wst.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx.stream));
      ICK(cudaGetLastError());
      if ((st = residual64(ctx, U, dYdt.p)) != FV3D_OK) return st;
      k_newton_rhs<<<grid, 256, 0, ctx.stream>>>(n, U, old0.p, old1.p, dYdt.p, dt, bb, a0, a1, stages, fY.p);
      ICK(cudaGetLastError());
      if ((st = norm(ctx, fY.p, &err)) != FV3D_OK) return st;
      if (!std::isfinite(err)) return ctx.fail(FV3D_ERR_NONFINITE, "implicit step: non-finite residual");
    } else {
      if ((st = residual64(ctx, U, dYdt.p)) != FV3D_OK) return st;
    }
    if (err < err0) break;
    if (!o.is_transient) break;
  }
  ICK(cudaMemcpyAsync(ctx.d_dphi.p, dYdt.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx.stream));
  if ((st = refresh_records(ctx)) != FV3D_OK) return st;
  ICK(cudaStreamSynchronize(ctx.stream));
  ctx.residual_valid = true;
  if (stats) {
    stats->n_inner = it;
    stats->err0 = err0;
    stats->err = err;
  }
  if (it >= o.max_iter_inner)
    return ctx.fail(FV3D_ERR_NOT_CONVERGED, "implicit step: no convergence in %d iterations", o.max_iter_inner);
  return FV3D_OK;
}

fv3d_status Implicit::ICK_copy(Ctx& ctx, double* dst, const double* src) {
  ICK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx.stream));
  return FV3D_OK;
}

// J z = (R(U + eps z) - R(U)) / eps at the current state, with the solve's
// steps: FP32 residuals and eps = 5e-4 (1 + |U|) / |z|, or FP64 residuals
// and eps = fd_eps (1 + |U|) / |z|
fv3d_status Implicit::jacobian_vector(Ctx& ctx, int prec, double fd_eps, const double* z_rows, double* out_rows) {
  fv3d_status st = ensure_fp64_path(ctx);
  if (st == FV3D_OK && prec == 1) st = ensure_mixed_path(ctx);
  if (st == FV3D_OK) st = setup(ctx, 1);
  if (st == FV3D_OK) st = import_rows(ctx, z_rows, x.p);
  if (st != FV3D_OK) return st;
  opts.jv_precision = prec;
  st = (prec == 1) ? residual32(ctx, ctx.d_U.p, Rb.p) : residual64(ctx, ctx.d_U.p, Rb.p);
  if (st == FV3D_OK) st = norm(ctx, ctx.d_U.p, &unorm);
  if (st != FV3D_OK) return st;
  hpin[0] = ((prec == 1) ? 5e-4 : fd_eps) * (1.0 + unorm);
  hpin[1] = 1.0 / hpin[0];
  ICK(cudaMemcpyAsync(hdev.p + 100, hpin, 2 * sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
  if ((st = fd_residual<double>(ctx, x.p, false)) != FV3D_OK) return st;
  // w = 0 * z - (Rp - Rb) / eps = -J z (idtl zeroed first)
  ICK(cudaMemsetAsync(idtl.p, 0, sizeof(double) * ctx.nc, ctx.stream));
  k_jv_combine<double><<<blocks(ctx.nc), 256, 0, ctx.stream>>>(ctx.nc, x.p, Rp.p, Rb.p, idtl.p, jv_ieps, w.p);
  ICK(cudaGetLastError());
  k_lincomb<<<std::min(4096, blocks(n)), 256, 0, ctx.stream>>>(n, -1.0, w.p, 0.0, nullptr, Wst.p);
  ICK(cudaGetLastError());
  if ((st = refresh_records(ctx)) != FV3D_OK) return st;  // the perturbed records overwrote the state's
  return export_rows(ctx, Wst.p, out_rows);
}

}  // namespace fv3d

using namespace fv3d;

extern "C" fv3d_status fv3d_implicit_default_opts(fv3d_implicit_opts* o) {
  if (o == nullptr) return FV3D_ERR_INVALID_ARG;
  o->cfl_start = 100.0;
  o->cfl_max = 1e4;
  o->tol_rel = 1e-8;
  o->max_newton = 500;
  o->krylov_dim = 30;
  o->eta = 1e-2;
  o->fd_eps = 1e-7;
  o->jv_precision = 1;
  o->preconditioner = FV3D_PC_BLOCK_JACOBI;
  o->pc_refresh = 0;
  o->max_restarts = 0;
  o->sync_every = 0;
  o->inner_dim = 10;
  o->inner_sweeps = 2;
  o->inner_omega = 0.7;
  o->fallback = FV3D_PC_BLOCK_JACOBI;
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_solve_implicit(fv3d_ctx* handle, const fv3d_implicit_opts* opts,
                                           fv3d_implicit_stats* stats) {
  if (handle == nullptr || opts == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mesh_ready || !ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "mesh and state required");
  for (int b = 0; b < ctx->nb; ++b)
    if (!(ctx->region_set & (1u << ctx->h_fregion[b])))
      return ctx->fail(FV3D_ERR_STATE, "boundary region %d has no condition", ctx->h_fregion[b]);
  if (opts->preconditioner < 0 || opts->preconditioner > FV3D_PC_COUPLED || opts->jv_precision < 0 ||
      opts->jv_precision > 2 || !(opts->tol_rel > 0.0) || !(opts->cfl_start > 0.0) || opts->max_newton < 0)
    return ctx->fail(FV3D_ERR_INVALID_ARG, "bad implicit options");
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "cudaSetDevice");
  if (!ctx->implicit) ctx->implicit = new Implicit();
  return ctx->implicit->solve(*ctx, *opts, stats);
}

extern "C" fv3d_status fv3d_jacobian_vector(fv3d_ctx* handle, int jv_precision, double fd_eps, const double* z,
                                            double* jz) {
  if (handle == nullptr || z == nullptr || jz == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mesh_ready || !ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "mesh and state required");
  for (int b = 0; b < ctx->nb; ++b)
    if (!(ctx->region_set & (1u << ctx->h_fregion[b])))
      return ctx->fail(FV3D_ERR_STATE, "boundary region %d has no condition", ctx->h_fregion[b]);
  if ((jv_precision != 0 && jv_precision != 1) || !(fd_eps > 0.0))
    return ctx->fail(FV3D_ERR_INVALID_ARG, "bad Jacobian-vector arguments");
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "cudaSetDevice");
  if (!ctx->implicit) ctx->implicit = new Implicit();
  return ctx->implicit->jacobian_vector(*ctx, jv_precision, fd_eps, z, jz);
}

extern "C" fv3d_status fv3d_implicit_history(const fv3d_ctx* handle, double* res, int max, int* count) {
  if (handle == nullptr || count == nullptr) return FV3D_ERR_INVALID_ARG;
  const Ctx* ctx = reinterpret_cast<const Ctx*>(handle);
  if (!ctx->implicit) { *count = 0; return FV3D_OK; }
  const std::vector<double>& h = ctx->implicit->history;
  *count = (int)h.size();
  if (res != nullptr)
    for (int i = 0; i < std::min(max, (int)h.size()); ++i) res[i] = h[i];
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_get_blocks(fv3d_ctx* handle, double* blocks_out) {
  // diagonal blocks of the last preconditioner build, [n_cells][25]
  // column-major, reference cell order
  if (handle == nullptr || blocks_out == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->implicit || ctx->implicit->D.p == nullptr) return ctx->fail(FV3D_ERR_STATE, "no blocks built");
  std::vector<double> tmp(25 * (size_t)ctx->nc);
  if (cudaMemcpy(tmp.data(), ctx->implicit->D.p, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return ctx->fail(FV3D_ERR_DEVICE, "copy blocks");
  for (int c = 0; c < ctx->nc; ++c)
    memcpy(blocks_out + 25 * (size_t)ctx->perm[c], &tmp[25 * (size_t)c], sizeof(double) * 25);
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_step_newton(fv3d_ctx* handle, const fv3d_newton_opts* opts, int iter, double t,
                                        double dt, fv3d_newton_stats* stats) {
  if (handle == nullptr || opts == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mesh_ready || !ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "mesh and state required");
  if ((opts->scheme != FV3D_NEWTON_EULER && opts->scheme != FV3D_NEWTON_BDF2) || opts->max_iter_inner < 1 ||
      !(dt > 0.0) || iter < 0)
    return ctx->fail(FV3D_ERR_INVALID_ARG, "bad implicit step arguments");
  for (int b = 0; b < ctx->nb; ++b)
    if (!(ctx->region_set & (1u << ctx->h_fregion[b])))
      return ctx->fail(FV3D_ERR_STATE, "boundary region %d has no condition", ctx->h_fregion[b]);
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "cudaSetDevice");
  if (!ctx->implicit) ctx->implicit = new Implicit();
  return ctx->implicit->step_newton(*ctx, *opts, iter, t, dt, stats);
}

extern "C" fv3d_status fv3d_get_bdf_history(fv3d_ctx* handle, int stage, double* phi_old, int* n_stages) {
  if (handle == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  const Implicit* im = ctx->implicit;
  const int ns = (im != nullptr && im->newton_ready) ? im->n_bdf : 0;
  if (n_stages != nullptr) *n_stages = ns;
  if (phi_old == nullptr) return FV3D_OK;
  if (stage < 0 || stage >= ns) return ctx->fail(FV3D_ERR_INVALID_ARG, "history stage %d of %d", stage, ns);
  return export_rows(*ctx, stage == 0 ? im->old0.p : im->old1.p, phi_old);
}

extern "C" fv3d_status fv3d_set_bdf_history(fv3d_ctx* handle, int scheme, int n_stages, const double* phi_old) {
  if (handle == nullptr || phi_old == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mesh_ready || !ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "mesh and state required");
  if (scheme != FV3D_NEWTON_EULER && scheme != FV3D_NEWTON_BDF2)
    return ctx->fail(FV3D_ERR_INVALID_ARG, "bad implicit scheme %d", scheme);
  for (int b = 0; b < ctx->nb; ++b)
    if (!(ctx->region_set & (1u << ctx->h_fregion[b])))
      return ctx->fail(FV3D_ERR_STATE, "boundary region %d has no condition", ctx->h_fregion[b]);
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "cudaSetDevice");
  if (!ctx->implicit) ctx->implicit = new Implicit();
  return ctx->implicit->set_history(*ctx, scheme, n_stages, phi_old);
}
