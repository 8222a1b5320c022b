// The last-block reduction of the Gram-Schmidt passes (k_gs): each block has
// written its partial sums to partial[block][32]; the block that takes the
// last ticket sums them in block order (the result does not depend on
// which block is last) and resets the ticket.
#pragma once

namespace fv3d {

// eight consecutive partials of a row, with 16-byte loads past L1 (the
// other blocks wrote them)
__device__ __forceinline__ void ldcg8(const float* p, float* v) {
  const float4 a = __ldcg(reinterpret_cast<const float4*>(p)), b = __ldcg(reinterpret_cast<const float4*>(p + 4));
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void ldcg8(const double* p, double* v) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double2 a = __ldcg(reinterpret_cast<const double2*>(p) + q);
    v[2 * q] = a.x;
    v[2 * q + 1] = a.y;
  }
}

// columns j < k of the block partials summed into out[j] (FP64), or with
// norm the square root of column 0 and its derived scalars (r, 1/r, c/r,
// r/c); with out2, column 31 holds |w|^2 and out2 receives
// |w - sum_j out_j V_j| = sqrt(|w|^2 - sum_j out_j^2) (V orthonormal) and
// its inverse.  Blocks of 256 threads; partial 16-byte aligned.
template <class T>
__device__ void gs_finalize(const T* __restrict__ partial, int nb, int k, double* __restrict__ out, bool norm,
                            double c, unsigned int* counter, double* __restrict__ out2 = nullptr) {
  __shared__ bool last;
  __shared__ T red[8][32];
  __shared__ double tot[32];
  // the threads that wrote this block's partials make them visible, then
  // one thread takes the ticket
  if (threadIdx.x < 32) __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // every thread sums the rows b = t, t + 256, ... of the columns needed, 8
  // columns at a time (independent 16-byte loads: a few round trips to L2
  // in all), then a fixed xor tree per warp and the 8 warps in order
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j0 = 0; j0 < 32; j0 += 8) {
    if (!(j0 < k || (out2 != nullptr && j0 == 24))) continue;
    T a[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) a[l] = T(0);
    for (int b = threadIdx.x; b < nb; b += 256) {
      T v[8];
      ldcg8(partial + (size_t)b * 32 + j0, v);
#pragma unroll
      for (int l = 0; l < 8; ++l) a[l] += v[l];
    }
#pragma unroll
    for (int l = 0; l < 8; ++l) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a[l] += __shfl_xor_sync(0xffffffffu, a[l], o);
    }
    if (lane == 0) {
#pragma unroll
      for (int l = 0; l < 8; ++l) red[warp][j0 + l] = a[l];
    }
  }
  __syncthreads();
  const int j = threadIdx.x;
  if (j < 32 && (j < k || (out2 != nullptr && j == 31))) {
    T s = T(0);
#pragma unroll
    for (int wv = 0; wv < 8; ++wv) s += red[wv][j];
    tot[j] = (double)s;
    if (!norm && j < k) out[j] = (double)s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (norm) {
      const double r = sqrt(tot[0]);
      out[0] = r;
      out[1] = (r > 0.0) ? 1.0 / r : 0.0;
      out[2] = (r > 0.0) ? c / r : 0.0;
      out[3] = (r > 0.0) ? r / c : 0.0;
    }
    if (out2 != nullptr) {
      // column 31: |w|^2; the norm of w - sum_j out_j V_j by Pythagoras
      double hh = 0.0;
      for (int i = 0; i < k; ++i) hh += tot[i] * tot[i];
      const double b2 = tot[31] - hh;
      const double r = (b2 > 0.0) ? sqrt(b2) : 0.0;
      out2[0] = r;
      out2[1] = (r > 0.0) ? 1.0 / r : 0.0;
    }
    *counter = 0u;  // ready for the next pass
  }
}

}  // namespace fv3d
