// Mixed-precision path instantiations (FP32 faces, FP64 state).
#include "kernels_impl.cuh"
namespace fv3d {
template cudaError_t launch_gradients<float>(const KArgs<float>&, const Disc&, cudaStream_t);
template cudaError_t launch_face_flux<float>(const KArgs<float>&, const Disc&, cudaStream_t);
template cudaError_t launch_gather<float>(const KArgs<float>&, int, bool, const StageCoef&, cudaStream_t);
}  // namespace fv3d
