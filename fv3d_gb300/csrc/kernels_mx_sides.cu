// Mixed-precision explicit-stage launchers (gradient pass).
#include <algorithm>

#include "kernels_mixed.cuh"
#include "launch.h"

namespace fv3d {

#if FV3D_SIDES_TMA
static int g_sm_count = 0;  // multiprocessors of the device, read in setup_mx_sides

// the persistent two-buffer form while both buffers fit in this many bytes
// (4 CTAs per SM); larger tiles (6 or 8 face slots with least squares, 8
// with Green-Gauss) run one tile per CTA with one buffer, so that 4 CTAs
// still fit on an SM
#ifndef FV3D_PERSIST_MAX_SMEM
#define FV3D_PERSIST_MAX_SMEM (64 * 1024)
#endif
// cells per tile of the one-tile-per-CTA staged pass: 6- and 8-slot cells
// take tiles of FV3D_WIDE_TILE (more, smaller CTAs per multiprocessor than
// their 128-cell tiles allow; measured: the 577 k-cell mixed-element box
// +0.8 %, the 262 k jittered hexes unchanged at 32, 64 or 128)
#ifndef FV3D_WIDE_TILE
#define FV3D_WIDE_TILE 64
#endif
template <int MCF>
constexpr int wide_tile() {
  return MCF >= 6 ? FV3D_WIDE_TILE : kTile;
}

template <int MCF, int G>
constexpr bool sides_persistent() {
  return 2 * sides_buf_stride<MCF, G>() <= FV3D_PERSIST_MAX_SMEM;
}

// second-order passes: the tile-staged kernel
template <int MCF, int G, bool L, bool M, bool V>
static void launch_staged(const MxArgs& a, cudaStream_t s) {
  if constexpr (sides_persistent<MCF, G>()) {
    const int ntiles = a.ncp / kTile;
    const int grid = std::min(ntiles, std::max(1, g_sm_count) * 4);
    k_mx_sides_tma2<MCF, G, L, M, V><<<grid, kTile, 2 * sides_buf_stride<MCF, G>(), s>>>(a);
  } else {
    constexpr int TL = wide_tile<MCF>();
    k_mx_sides_tma<MCF, G, L, M, V, TL><<<a.ncp / TL, TL, SidesTile<MCF, G, TL>::total, s>>>(a);
  }
}

template <int MCF, int G, bool L, bool M, bool V>
static cudaError_t staged_attr() {
  if constexpr (sides_persistent<MCF, G>())
    return cudaFuncSetAttribute(k_mx_sides_tma2<MCF, G, L, M, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                2 * sides_buf_stride<MCF, G>());
  else
    return cudaFuncSetAttribute(k_mx_sides_tma<MCF, G, L, M, V, wide_tile<MCF>()>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, SidesTile<MCF, G, wide_tile<MCF>()>::total);
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

// dynamic shared memory above 48 KB needs the opt-in size per kernel; set
// once per context setup, outside any stream capture
cudaError_t setup_mx_sides() {
#if FV3D_SIDES_TMA
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
#define MX_ATTR(MCF, G, L, M, V) \
  if (e == cudaSuccess) e = staged_attr<MCF, G, L, M, V>();
#define MX_ATTR_ALL(MCF, G)                                                                          \
  MX_ATTR(MCF, G, false, false, false) MX_ATTR(MCF, G, false, false, true)                           \
  MX_ATTR(MCF, G, true, false, false) MX_ATTR(MCF, G, true, false, true)                             \
  MX_ATTR(MCF, G, true, true, false) MX_ATTR(MCF, G, true, true, true)
  MX_ATTR_ALL(4, 1) MX_ATTR_ALL(4, 2) MX_ATTR_ALL(6, 1) MX_ATTR_ALL(6, 2) MX_ATTR_ALL(8, 1) MX_ATTR_ALL(8, 2)
#undef MX_ATTR_ALL
#undef MX_ATTR
  return e;
#else
  return cudaSuccess;
#endif
}

// self-test of the bounded mbarrier wait the staged gradient pass uses: a
// phase that expects 16 bytes no copy will deliver; the wait gives up after
// limit_ns and the kernel records that in *flag (1 = gave up)
__global__ void k_bounded_wait_probe(unsigned long long limit_ns, int* flag) {
  __shared__ __align__(8) unsigned long long bar;
  const uint32_t b = smem_u32(&bar);
  if (threadIdx.x == 0) {
    mbar_init(b, 1);
    fence_mbar_init();
    mbar_expect_tx(b, 16);  // arrives, leaving 16 bytes outstanding
    *flag = mbar_wait_bounded(b, 0, limit_ns) ? 0 : 1;
  }
}

cudaError_t launch_bounded_wait_probe(unsigned long long limit_ns, int* flag, cudaStream_t s) {
  k_bounded_wait_probe<<<1, 32, 0, s>>>(limit_ns, flag);
  return cudaGetLastError();
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
