// Implicit Newton-Krylov solver state (see implicit.cu).
#pragma once

#include <vector>

#include <map>

#include "context.h"

namespace fv3d {

struct Implicit;

// learned preconditioner state (mlp.cu)
struct Mlp {
  bool ready = false;
  DevBuf<float> P, m, v, grad;      // FP32 master parameters, Adam moments, gradient
  DevBuf<float> part, loss_part;    // per-CTA partial gradients / losses
  DevBuf<int> bidx;
  DevBuf<float> feat;               // [nc][32] per-cell feature record
  DevBuf<float> X, T, Wt;           // harvested training pairs and their loss weights
  int n_samples = 0, max_samples = 0, harvest_per_step = 0, harvest_calls = 0;
  int adam_t = 0;

  fv3d_status init(Ctx& ctx, unsigned long long seed);
  fv3d_status ensure_scratch(Ctx& ctx, int nbatch);
  fv3d_status forward_host(Ctx& ctx, const float* X, int n, float* Y);
  fv3d_status grad_host(Ctx& ctx, const float* X, const float* T, int n, double* loss, float* g);
  fv3d_status train(Ctx& ctx, const fv3d_mlp_train_opts& o, fv3d_mlp_train_stats* stats);
  fv3d_status adam_step(Ctx& ctx, float lr);
  fv3d_status build_features(Ctx& ctx, const Implicit& im);
  fv3d_status apply(Ctx& ctx, const double* v, double* z);
  fv3d_status apply(Ctx& ctx, const float* v, float* z);
  fv3d_status harvest(Ctx& ctx, const Implicit& im);
  // the tcgen05 (TMEM-accumulator) forward (mlp_tc.cu); the inference
  // kernels used: tcgen05 (default) or the warp-level mma.sync ones
  bool use_tc = true, tc_ready = false;
  DevBuf<int> tc_status;            // nonzero: a bounded wait of the tcgen05 kernel ran out
  DevBuf<unsigned char> tc_img;     // the weights as BF16 tiles in the kernel's shared-memory layout
  fv3d_status tc_setup(Ctx& ctx);
  fv3d_status forward_tc(Ctx& ctx, const float* dX, int n, float* dY);
  template <class VT>
  fv3d_status apply_tc(Ctx& ctx, const VT* v, VT* z);
};

// cell-coupling preconditioner (coupled.cu): z = M v, M an inner GMRES on
// P_A = I/dt - dR1/dU right-preconditioned by block-Jacobi sweeps of the
// first-order Rusanov Jacobian P_R
struct Coupled {
  int nc = 0, mcf = 0, m_cap = 0;  // sizes the buffers are allocated for
  int m_in = 0, sweep_count = 0;   // inner GMRES iterations and sweeps of the current solve
  float omega = 0.f;               // damping of the sweeps
  size_t n = 0, ldb = 0;
  DevBuf<int> nbr;                 // [mcf][nc] neighbour of each face slot, -2 - b boundary face b, -1 none
  int nb = 0;
  // P_A, matrix-free: FP32 state records [nc][8] (rho, m, E, p, 1/c, 1/rho), 1/dt [nc], per slot
  // (normal, s A / V) [mcf][nc], per boundary face the ghost's record [nb][8] and d ghost / d U [nb][25]
  DevBuf<float> cst, idt, gst, gjac;
  DevBuf<float4> pna;
  DevBuf<float> PRi;               // P_R: inverted diagonal blocks [25][nc]; its slot blocks are applied
  DevBuf<double> bpr;              // P_R: each boundary face's diagonal block per unit weight [nb][25]
  DevBuf<float4> rna, st4;         // matrix-free: per slot (normal, a) [mcf][nc], per cell (u, v, w, H)
  DevBuf<float> rb;                // per slot b [mcf][nc]
  DevBuf<float> Vi, Ti, wi, ti;    // inner basis [(m_in + 1)][ldb], directions [m_in][ldb], work [ldb]
  DevBuf<double> hin;              // inner Hessenberg columns [m_in + 1][72] and y
  fv3d_status setup(Ctx& ctx, Implicit& im, int m_inner, int n_sweeps, float damping);
  fv3d_status build(Ctx& ctx, Implicit& im);
  template <class T>
  fv3d_status apply(Ctx& ctx, Implicit& im, const T* v, T* z);
  template <class TO>
  fv3d_status sweeps(Ctx& ctx, int count, const float* b, const float* x0, TO* out);
};

struct Implicit {
  fv3d_implicit_opts opts;
  size_t n = 0;   // 5 * cells
  size_t ldb = 0; // Krylov basis vectors' stride: n rounded up to 64 (16-byte aligned vectors)
  int m = 0;      // Krylov dimension allocated
  DevBuf<double> V, Z, w, R, Rb, Rp, Wst, x, dtl, idtl, D, part, hdev, fdist;
  DevBuf<float> V32, Z32, w32;    // Krylov basis for FP32 Jacobian-vector products
  DevBuf<float> Dinv;
  DevBuf<unsigned long long> bits;
  std::vector<double> history;  // ||R||_2 per Newton step
  int jv_count = 0;
  double unorm = 0.0;
  bool use_fallback = false;      // learned preconditioner fell back this step
  double* hpin = nullptr;         // pinned host scalars (kHostCoefs doubles)
  double* hcols = nullptr;        // pinned: each Arnoldi step's coefficients, [32][kHostCoefs]

  std::map<long long, cudaGraphExec_t> arnoldi_graphs;  // captured Arnoldi steps
  Coupled* coupled = nullptr;     // FV3D_PC_COUPLED work space, created on first use

  ~Implicit() {
    release_graphs();
    delete coupled;
    if (hpin) cudaFreeHost(hpin);
    if (hcols) cudaFreeHost(hcols);
  }
  void release_graphs();
  template <class T>
  fv3d_status enqueue_arnoldi(Ctx& ctx, T* Vt, T* Zt, T* wt, int k);
  template <class T>
  fv3d_status arnoldi_step(Ctx& ctx, T* Vt, T* Zt, T* wt, int k);

  fv3d_status setup(Ctx& ctx, int m);
  fv3d_status solve(Ctx& ctx, const fv3d_implicit_opts& o, fv3d_implicit_stats* stats);
  fv3d_status fgmres(Ctx& ctx, double rnorm, int* iters, double* rel_res);
  template <class T>
  fv3d_status fgmres_t(Ctx& ctx, T* Vt, T* Zt, T* wt, double rnorm, int* iters, double* rel_res);
  template <class T>
  fv3d_status apply_A(Ctx& ctx, const T* z, T* out);
  template <class T>
  fv3d_status fd_residual(Ctx& ctx, const T* z, bool unit);
  const double* jv_ieps = nullptr;  // device slot of 1/eps of the last fd_residual
  template <class T>
  fv3d_status precondition(Ctx& ctx, const T* v, T* z);
  fv3d_status build_blocks(Ctx& ctx);
  template <class T>
  fv3d_status dots_dev(Ctx& ctx, const T* w, const T* V, int k, double* dst, bool take_sqrt, double c);
  template <class T>
  fv3d_status gs_pass(Ctx& ctx, int pass, T* w, const T* V, int k, const double* h_in, double* dst, double c,
                      const double* c_dev, const T* jv_z = nullptr, double* dst2 = nullptr, T* vout = nullptr,
                      const double* scale = nullptr);
  fv3d_status norm(Ctx& ctx, const double* v, double* out);
  fv3d_status ICK_copy(Ctx& ctx, double* dst, const double* src);
  fv3d_status jacobian_vector(Ctx& ctx, int prec, double fd_eps, const double* z_rows, double* out_rows);

  // the reference's implicit time step (timestep_newton)
  DevBuf<double> old0, old1, dYdt, fY;
  int n_bdf = 0;
  bool newton_ready = false;
  fv3d_status step_newton(Ctx& ctx, const fv3d_newton_opts& o, int iter, double t, double dt,
                          fv3d_newton_stats* stats);
  fv3d_status newton_buffers(Ctx& ctx);
  fv3d_status set_history(Ctx& ctx, int scheme, int n_stages, const double* rows);
};

}  // namespace fv3d
