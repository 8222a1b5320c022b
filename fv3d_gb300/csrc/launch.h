// Host-side launch entry points of the explicit-stage kernels: the FP64 path
// (kernels_f64.cu, three launches per stage) and the mixed path
// (kernels_mixed.cu, two launches per stage).
#pragma once

#include <cuda_runtime.h>
#include "kernels.cuh"

namespace fv3d {

struct Disc {
  int gmode;     // 0 none, 1 Green-Gauss, 2 least squares
  bool linear;   // linear reconstruction
  bool limit;    // Barth-Jespersen
  bool viscous;  // mu != 0
};

struct MxArgs;
cudaError_t launch_mx_sides(const MxArgs& a, const Disc& d, cudaStream_t s);
cudaError_t setup_mx_sides();
cudaError_t launch_bounded_wait_probe(unsigned long long limit_ns, int* flag, cudaStream_t s);
cudaError_t launch_mx_flux_update(const MxArgs& a, const Disc& d, int mode, bool dt,
                                  const StageCoef& co, cudaStream_t s);

template <class R> cudaError_t launch_gradients(const KArgs<R>& a, const Disc& d, cudaStream_t s);
template <class R> cudaError_t launch_face_flux(const KArgs<R>& a, const Disc& d, cudaStream_t s);
template <class R>
cudaError_t launch_gather(const KArgs<R>& a, int mode, bool dt, const StageCoef& co, cudaStream_t s);

}  // namespace fv3d
