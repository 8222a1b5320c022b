// FP64 path instantiations.
#include "kernels_impl.cuh"
namespace fv3d {
template cudaError_t launch_gradients<double>(const KArgs<double>&, const Disc&, cudaStream_t);
template cudaError_t launch_face_flux<double>(const KArgs<double>&, const Disc&, cudaStream_t);
template cudaError_t launch_gather<double>(const KArgs<double>&, int, bool, const StageCoef&, cudaStream_t);
}  // namespace fv3d
