// Context object behind the fv3d_ctx handle.
#pragma once

#include <cuda_runtime.h>
#include <map>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/fv3d_gpu.h"
#include "kernels_mixed.cuh"
#include "launch.h"

namespace fv3d {

struct Implicit;
struct Mlp;

// owning device allocation
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    release();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * count);
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DevBuf() { release(); }
};

struct Ctx {
  fv3d_config cfg;
  std::string err;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  DevScalars* h_sc = nullptr;  // page-locked copy of the device scalars (asynchronous reads)
  PhysConst phys;
  double kappa_pr = 0.0;
  unsigned region_set = 0;
  bool mesh_ready = false, state_ready = false, residual_valid = false;

  // sizes (renumbered mesh): interior faces first, then boundary faces
  int nc = 0, nf = 0, nf_int = 0, nb = 0, mcf = 0, n_regions = 0;
  int ncp = 0;  // nc rounded up to whole gradient-pass tiles (kTile cells): row count of the staged arrays
  double vol_total = 0.0;

  // host-side maps
  std::vector<int> perm;      // perm[new cell] = reference cell
  std::vector<int> iperm;     // iperm[reference cell] = new cell
  std::vector<int> fperm;     // fperm[new face] = reference face
  std::vector<int> h_fregion; // region of each boundary face (new order)
  std::vector<int> h_fc0, h_fc1, h_cface;
  std::vector<double> h_geo;  // [nf][GEO] FP64 geometry (new order)
  std::vector<double> h_lam, h_lsq, h_vol, h_dx;
  std::vector<double> h_cell_x;  // cell centres in reference order (for exact-function initial states)

  // device mesh
  DevBuf<int> d_iperm, d_perm, d_fc0, d_fc1, d_fregion, d_cface, d_cnbr, d_cother;
  DevBuf<char> d_geo, d_lam, d_lsq, d_rvol;  // FP64-path geometry (double)
  DevBuf<double> d_vol, d_dx;
  // device solution data
  DevBuf<double> d_U, d_K, d_U0, d_dphi, d_stage, d_part;
  DevBuf<double> d_Pq;  // FP64 path: the state's primitives [5][nc] (k_prims)
  DevBuf<float> d_Uf;
  DevBuf<char> d_rec, d_FA;
  // mixed path
  DevBuf<int2> d_fcell;
  DevBuf<float4> d_slotN, d_slotD, d_slotW, d_slotNk, d_slotDk, d_slotWk, d_cgeo, d_cdx;
  DevBuf<float> d_fs, d_fsv, d_UfN, d_kf, d_dU;
  DevBuf<DevScalars> d_sc;
  DevBuf<unsigned long long> d_bits;

  std::map<std::tuple<int, double, int>, cudaGraphExec_t> graphs;  // (scheme, cfl, store_r)
  Implicit* implicit = nullptr;  // Newton-Krylov work space, created on first use
  Mlp* mlp = nullptr;            // learned preconditioner, created on first use

  bool fp64() const { return cfg.precision == FV3D_PRECISION_FP64; }
  size_t rsize() const { return fp64() ? sizeof(double) : sizeof(float); }
  fv3d_status fail(fv3d_status st, const char* fmt, ...);
  fv3d_status cuda(cudaError_t e, const char* what);
  void release_graphs();
  void free_device() {
    d_cnbr.release(); d_perm.release(); d_iperm.release(); d_fc0.release(); d_fc1.release(); d_fregion.release(); d_cface.release();
    d_geo.release(); d_lam.release(); d_lsq.release(); d_rvol.release(); d_vol.release(); d_dx.release();
    d_U.release(); d_K.release(); d_U0.release(); d_dphi.release(); d_stage.release(); d_part.release();
    d_Uf.release(); d_rec.release(); d_FA.release(); d_sc.release(); d_bits.release();
    d_fcell.release(); d_slotN.release(); d_slotD.release(); d_slotW.release(); d_slotNk.release(); d_slotDk.release(); d_slotWk.release(); d_fs.release();
    d_fsv.release(); d_cother.release();
    d_cgeo.release(); d_cdx.release(); d_UfN.release(); d_kf.release(); d_dU.release();
  }
  template <class R> KArgs<R> args() const;
  MxArgs mx_args() const;
  Disc disc() const;
  cudaError_t launch_stage_kernels(int mode, bool dt, const StageCoef& co, int which);
};

fv3d_status prepare_mesh(Ctx& ctx, const fv3d_mesh_arrays& m);
fv3d_status upload_mesh(Ctx& ctx);
fv3d_status ensure_fp64_path(Ctx& ctx);
fv3d_status ensure_mixed_path(Ctx& ctx);
// a [5][nc] FP64 device array from / to n_cells rows of 5 in reference order
// (host memory; synchronous)
fv3d_status import_rows(Ctx& ctx, const double* rows, double* dst);
fv3d_status export_rows(Ctx& ctx, const double* src, double* rows);

}  // namespace fv3d
