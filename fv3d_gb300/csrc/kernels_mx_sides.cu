// Mixed-precision explicit-stage launchers (gradient pass).
#include "kernels_mixed.cuh"
#include "launch.h"

namespace fv3d {

#if FV3D_SIDES_TMA
// second-order passes: the tile-staged kernel, one CTA of kTile threads per tile
template <int MCF, int G, bool L, bool M, bool V>
static void launch_staged(const MxArgs& a, cudaStream_t s) {
  k_mx_sides_tma<MCF, G, L, M, V><<<a.ncp / kTile, kTile, SidesTile<MCF, G>::total, s>>>(a);
}
#define MX_SIDES(G, L, M, V)                                              \
  do {                                                                   \
    if (G != 0) launch_staged<MCF, (G != 0 ? G : 1), L, M, V>(a, s);      \
    else k_mx_sides<MCF, G, L, M, V><<<B, 256, 0, s>>>(a);                \
  } while (0)
#else
#define MX_SIDES(G, L, M, V) k_mx_sides<MCF, G, L, M, V><<<B, 256, 0, s>>>(a)
#endif

template <int MCF>
static void sides_mcf(const MxArgs& a, const Disc& d, cudaStream_t s, int B) {
  const bool lim = d.linear && d.limit;
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

// tiles above 48 KB (6 or 8 face slots with least squares) need the opt-in
// shared-memory size; set once per context setup, outside any stream capture
cudaError_t setup_mx_sides() {
#if FV3D_SIDES_TMA
  cudaError_t e = cudaSuccess;
#define MX_ATTR(MCF, L, M, V)                                                                   \
  if (e == cudaSuccess)                                                                        \
    e = cudaFuncSetAttribute(k_mx_sides_tma<MCF, 2, L, M, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             SidesTile<MCF, 2>::total);
#define MX_ATTR_ALL(MCF)                                                                        \
  MX_ATTR(MCF, false, false, false) MX_ATTR(MCF, false, false, true) MX_ATTR(MCF, true, false, false) \
  MX_ATTR(MCF, true, false, true) MX_ATTR(MCF, true, true, false) MX_ATTR(MCF, true, true, true)
  static_assert(SidesTile<4, 2>::total <= 48 * 1024 && SidesTile<8, 1>::total <= 48 * 1024,
                "only the least-squares tiles of 6 and 8 slots exceed 48 KB");
  MX_ATTR_ALL(6)
  MX_ATTR_ALL(8)
#undef MX_ATTR_ALL
#undef MX_ATTR
  return e;
#else
  return cudaSuccess;
#endif
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
