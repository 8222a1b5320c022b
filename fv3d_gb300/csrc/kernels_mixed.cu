// Mixed-precision explicit-stage launchers.
#include "kernels_mixed.cuh"
#include "launch.h"

namespace fv3d {

static inline int nblocks(int n) { return (n + 255) / 256; }

cudaError_t launch_mx_sides(const MxArgs& a, const Disc& d, cudaStream_t s) {
  const int B = nblocks(a.nc);
  const bool lim = d.linear && d.limit;
#define MX_SIDES(G, L, M, V) k_mx_sides<G, L, M, V><<<B, 256, 0, s>>>(a)
  if (d.gmode == 0) {
    if (d.viscous) MX_SIDES(0, false, false, true);
    else MX_SIDES(0, false, false, false);
  } else if (d.gmode == 1) {
    if (!d.linear) { if (d.viscous) MX_SIDES(1, false, false, true); else MX_SIDES(1, false, false, false); }
    else if (lim) { if (d.viscous) MX_SIDES(1, true, true, true); else MX_SIDES(1, true, true, false); }
    else { if (d.viscous) MX_SIDES(1, true, false, true); else MX_SIDES(1, true, false, false); }
  } else {
    if (!d.linear) { if (d.viscous) MX_SIDES(2, false, false, true); else MX_SIDES(2, false, false, false); }
    else if (lim) { if (d.viscous) MX_SIDES(2, true, true, true); else MX_SIDES(2, true, true, false); }
    else { if (d.viscous) MX_SIDES(2, true, false, true); else MX_SIDES(2, true, false, false); }
  }
#undef MX_SIDES
  return cudaGetLastError();
}

cudaError_t launch_mx_flux_update(const MxArgs& a, const Disc& d, int mode, bool dt,
                                  const StageCoef& co, cudaStream_t s) {
  const int B = nblocks(a.nc);
#define MX_FU(M, D, V) k_mx_flux_update<M, D, V><<<B, 256, 0, s>>>(a, co)
  if (mode == 0) { if (d.viscous) MX_FU(0, false, true); else MX_FU(0, false, false); }
  else if (mode == 1) {
    if (dt) { if (d.viscous) MX_FU(1, true, true); else MX_FU(1, true, false); }
    else { if (d.viscous) MX_FU(1, false, true); else MX_FU(1, false, false); }
  } else {
    if (dt) { if (d.viscous) MX_FU(2, true, true); else MX_FU(2, true, false); }
    else { if (d.viscous) MX_FU(2, false, true); else MX_FU(2, false, false); }
  }
#undef MX_FU
  return cudaGetLastError();
}

}  // namespace fv3d
