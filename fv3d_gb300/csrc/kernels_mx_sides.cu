// Mixed-precision explicit-stage launchers (gradient pass).
#include "kernels_mixed.cuh"
#include "launch.h"

namespace fv3d {

template <int MCF>
static void sides_mcf(const MxArgs& a, const Disc& d, cudaStream_t s, int B) {
  const bool lim = d.linear && d.limit;
#define MX_SIDES(G, L, M, V) k_mx_sides<MCF, G, L, M, V><<<B, 256, 0, s>>>(a)
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
}

cudaError_t launch_mx_sides(const MxArgs& a, const Disc& d, cudaStream_t s) {
  const int B = (a.nc + 255) / 256;
  if (a.mcf == 4) sides_mcf<4>(a, d, s, B);
  else if (a.mcf == 6) sides_mcf<6>(a, d, s, B);
  else if (a.mcf == 8) sides_mcf<8>(a, d, s, B);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace fv3d
