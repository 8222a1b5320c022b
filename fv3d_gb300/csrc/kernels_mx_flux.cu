// Mixed-precision explicit-stage launchers (flux + update pass).
#include "kernels_mixed.cuh"
#include "launch.h"

namespace fv3d {

#ifndef FV3D_FLUX_WIDE_THREADS
#define FV3D_FLUX_WIDE_THREADS 64
#endif

template <int MCF>
static void flux_mcf(const MxArgs& a, const Disc& d, int mode, bool dt, const StageCoef& co,
                     cudaStream_t s, int B, int T = 256) {
#define MX_FU(M, D, V)                                                   \
  do {                                                                  \
    if (M != 0 && co.store_r) k_mx_flux_update<MCF, M, D, V, true><<<B, T, 0, s>>>(a, co); \
    else k_mx_flux_update<MCF, M, D, V><<<B, T, 0, s>>>(a, co);        \
  } while (0)
  if (mode == 0) { if (d.viscous) MX_FU(0, false, true); else MX_FU(0, false, false); }
  else if (mode == 1) {
    if (dt) { if (d.viscous) MX_FU(1, true, true); else MX_FU(1, true, false); }
    else { if (d.viscous) MX_FU(1, false, true); else MX_FU(1, false, false); }
  } else {
    if (dt) { if (d.viscous) MX_FU(2, true, true); else MX_FU(2, true, false); }
    else { if (d.viscous) MX_FU(2, false, true); else MX_FU(2, false, false); }
  }
#undef MX_FU
}

cudaError_t launch_mx_flux_update(const MxArgs& a, const Disc& d, int mode, bool dt,
                                  const StageCoef& co, cudaStream_t s) {
  const int B = (a.nc + 255) / 256;
  // 6- and 8-slot cells: blocks of FV3D_FLUX_WIDE_THREADS (their kernels keep
  // 64+ registers, so 256-thread blocks fit 3 per multiprocessor and leave
  // a ragged last wave on meshes of a few hundred thousand cells: the
  // 262 k jittered hexes +13 % per stage with 64-thread blocks)
  const int BW = (a.nc + FV3D_FLUX_WIDE_THREADS - 1) / FV3D_FLUX_WIDE_THREADS;
  if (a.mcf == 4) flux_mcf<4>(a, d, mode, dt, co, s, B);
  else if (a.mcf == 6) flux_mcf<6>(a, d, mode, dt, co, s, BW, FV3D_FLUX_WIDE_THREADS);
  else if (a.mcf == 8) flux_mcf<8>(a, d, mode, dt, co, s, BW, FV3D_FLUX_WIDE_THREADS);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace fv3d
