// Template dispatch of the explicit-stage kernels; included once per
// precision by kernels_f64.cu / kernels_f32.cu.
#pragma once

#include "launch.h"

namespace fv3d {

static inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

// FP64 kernels in blocks of 64: at 140-170 registers a 256-thread block
// fits once per multiprocessor (8 warps); 64-thread blocks fit 6-7 times
// (measured, FP64 RK3 steps: tets +14 %, jittered hexes +9 %, the channel
// +10 %).  Every cell's and face's arithmetic is its own, so the results
// do not depend on the block size.
#ifndef FV3D_F64_THREADS
#define FV3D_F64_THREADS 64
#endif

template <class R>
cudaError_t launch_gradients(const KArgs<R>& a, const Disc& d, cudaStream_t s) {
  constexpr bool K = sizeof(R) == 4;
  const int T = sizeof(R) == 8 ? FV3D_F64_THREADS : 256, B = blocks_for(a.nc, T);
  const bool lim = d.linear && d.limit;
  if (sizeof(R) == 8) k_prims<R><<<B, T, 0, s>>>(a);
  if (d.gmode == 0) k_gradients<R, 0, false, K><<<B, T, 0, s>>>(a);
  else if (d.gmode == 1) {
    if (lim) k_gradients<R, 1, true, K><<<B, T, 0, s>>>(a);
    else k_gradients<R, 1, false, K><<<B, T, 0, s>>>(a);
  } else {
    if (lim) k_gradients<R, 2, true, K><<<B, T, 0, s>>>(a);
    else k_gradients<R, 2, false, K><<<B, T, 0, s>>>(a);
  }
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_face_flux(const KArgs<R>& a, const Disc& d, cudaStream_t s) {
  const int T = sizeof(R) == 8 ? FV3D_F64_THREADS : 256, B = blocks_for(a.nf, T);
  const bool lim = d.linear && d.limit;
  if (d.linear) {
    if (lim) {
      if (d.viscous) k_face_flux<R, true, true, true><<<B, T, 0, s>>>(a);
      else k_face_flux<R, true, true, false><<<B, T, 0, s>>>(a);
    } else {
      if (d.viscous) k_face_flux<R, true, false, true><<<B, T, 0, s>>>(a);
      else k_face_flux<R, true, false, false><<<B, T, 0, s>>>(a);
    }
  } else {
    if (d.viscous) k_face_flux<R, false, false, true><<<B, T, 0, s>>>(a);
    else k_face_flux<R, false, false, false><<<B, T, 0, s>>>(a);
  }
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_gather(const KArgs<R>& a, int mode, bool dt, const StageCoef& co, cudaStream_t s) {
  constexpr bool K = sizeof(R) == 4;
  const int T = sizeof(R) == 8 ? FV3D_F64_THREADS : 256, B = blocks_for(a.nc, T);
  if (mode == 0) k_gather_update<R, 0, K, false><<<B, T, 0, s>>>(a, co);
  else if (mode == 1) {
    if (dt) k_gather_update<R, 1, K, true><<<B, T, 0, s>>>(a, co);
    else k_gather_update<R, 1, K, false><<<B, T, 0, s>>>(a, co);
  } else {
    if (dt) k_gather_update<R, 2, K, true><<<B, T, 0, s>>>(a, co);
    else k_gather_update<R, 2, K, false><<<B, T, 0, s>>>(a, co);
  }
  return cudaGetLastError();
}

}  // namespace fv3d
