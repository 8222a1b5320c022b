// C ABI implementation (include/fv3d_gpu.h): context, mesh preparation
// (metrics, validation, renumbering, structure-of-arrays upload), state
// import/export, the residual entry point and the graph-captured explicit
// step loop.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cfloat>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/fv3d_gpu.h"
#include "launch.h"
#include "context.h"
#include "implicit.h"

using namespace fv3d;

// ---------------------------------------------------------------------------
// small device kernels owned by the host layer
// ---------------------------------------------------------------------------
namespace {

// reference AoS [n][5] (reference order) -> SoA [5][n] (renumbered) + FP32 shadow
__global__ void k_import(int nc, const int* __restrict__ perm, const double* __restrict__ in,
                         double* __restrict__ U, float* __restrict__ Uf, float* __restrict__ UfN,
                         double km1, double R) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double* s = in + 5 * (size_t)perm[c];
  double u[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) { u[j] = s[j]; U[(size_t)j * nc + c] = u[j]; }
  if (Uf != nullptr) {
    float rho = (float)u[0], mx = (float)u[1], my = (float)u[2], mz = (float)u[3];
    float ke = 0.5f * (mx * (mx / rho) + my * (my / rho) + mz * (mz / rho));
    float p = fmaxf(1.00E-10f, (float)(km1 * (u[4] - (double)ke)));
    float T = p / (rho * (float)R);
    float4* d = reinterpret_cast<float4*>(Uf) + 2 * (size_t)c;
    d[0] = make_float4(rho, mx, my, mz);
    d[1] = make_float4((float)u[4], p, T, 1.0f / rho);
    float4* b = reinterpret_cast<float4*>(UfN) + 2 * (size_t)c;
    b[0] = d[0];
    b[1] = d[1];
  }
}

// SoA [m][n] (renumbered) -> reference AoS [n][m]; with prims: [n][10]
// the same import reading the caller's pinned host rows directly: each CTA
// copies its 128 rows (640 doubles, contiguous) with 16-byte loads over the
// host link into shared memory, then scatters them into the renumbered device
// arrays (the host buffer must be 16-byte aligned; checked by the caller)
constexpr int kIoRows = 128;
// With conv_bits set (mixed path), the kernel also takes the state's
// convective time-step bound, min V / sum_d (|u_d| + c) dx_d, from the FP32
// records it writes - k_timestep_f32's arithmetic, so the same bound - while
// the host link sets its pace.
__global__ void __launch_bounds__(kIoRows) k_import_host(int nc, const int* __restrict__ iperm,
                                                         const double* __restrict__ in, double* __restrict__ U,
                                                         float* __restrict__ Uf, float* __restrict__ UfN,
                                                         double km1, double R, const double* __restrict__ vol,
                                                         const double* __restrict__ dx, float kappa,
                                                         unsigned long long* conv_bits) {
  __shared__ __align__(16) double sm[kIoRows * 5];
  const size_t i0 = (size_t)blockIdx.x * kIoRows;
  const int cnt = (int)min((size_t)kIoRows, (size_t)nc - i0);
  const int nd = cnt * 5;
  const double2* src = reinterpret_cast<const double2*>(in + 5 * i0);
  for (int k = threadIdx.x; k < nd / 2; k += kIoRows) reinterpret_cast<double2*>(sm)[k] = src[k];
  if ((nd & 1) && threadIdx.x == 0) sm[nd - 1] = in[5 * i0 + nd - 1];
  __syncthreads();
  unsigned long long bc = 0x7ff0000000000000ull;
  if ((int)threadIdx.x < cnt) {
    const int c = iperm[i0 + threadIdx.x];
    double u[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) { u[j] = sm[5 * threadIdx.x + j]; U[(size_t)j * nc + c] = u[j]; }
    if (Uf != nullptr) {
      float rho = (float)u[0], mx = (float)u[1], my = (float)u[2], mz = (float)u[3];
      float ke = 0.5f * (mx * (mx / rho) + my * (my / rho) + mz * (mz / rho));
      float p = fmaxf(1.00E-10f, (float)(km1 * (u[4] - (double)ke)));
      float T = p / (rho * (float)R);
      float4* d = reinterpret_cast<float4*>(Uf) + 2 * (size_t)c;
      d[0] = make_float4(rho, mx, my, mz);
      d[1] = make_float4((float)u[4], p, T, 1.0f / rho);
      float4* b = reinterpret_cast<float4*>(UfN) + 2 * (size_t)c;
      b[0] = d[0];
      b[1] = d[1];
      if (conv_bits != nullptr) {
        const float ir = 1.f / rho;
        const float uu = mx * ir, vv = my * ir, ww = mz * ir;
        const float cs = sqrtf(kappa * p * ir);
        const double* dc = dx + 3 * (size_t)c;
        const float ds = (fabsf(uu) + cs) * (float)dc[0] + (fabsf(vv) + cs) * (float)dc[1] +
                         (fabsf(ww) + cs) * (float)dc[2];
        const double lc = (double)((float)vol[c] / ds);
        if (lc > 0.0) bc = (unsigned long long)__double_as_longlong(lc);
        if (!(lc == lc)) bc = 0x7ff8000000000000ull;
      }
    }
  }
  if (conv_bits != nullptr) {
    bc = warp_min_u64(bc);
    if ((threadIdx.x & 31) == 0) atomicMin(conv_bits, bc);
  }
}

// export of the 5 conserved variables straight into the caller's pinned
// host rows: each CTA gathers its 128 rows into shared memory and writes
// them with 16-byte stores over the host link (16-byte aligned buffer)
__global__ void __launch_bounds__(kIoRows) k_export_host(int nc, const int* __restrict__ iperm,
                                                         const double* __restrict__ S, double* __restrict__ out) {
  __shared__ __align__(16) double sm[kIoRows * 5];
  const size_t i0 = (size_t)blockIdx.x * kIoRows;
  const int cnt = (int)min((size_t)kIoRows, (size_t)nc - i0);
  if ((int)threadIdx.x < cnt) {
    const int c = iperm[i0 + threadIdx.x];
#pragma unroll
    for (int j = 0; j < 5; ++j) sm[5 * threadIdx.x + j] = S[(size_t)j * nc + c];
  }
  __syncthreads();
  const int nd = cnt * 5;
  double2* dst = reinterpret_cast<double2*>(out + 5 * i0);
  for (int k = threadIdx.x; k < nd / 2; k += kIoRows) dst[k] = reinterpret_cast<const double2*>(sm)[k];
  if ((nd & 1) && threadIdx.x == 0) out[5 * i0 + nd - 1] = sm[nd - 1];
}

// the convective time-step bound min V / sum_d (|u_d| + c) dx_d of the FP32
// state records (mixed path: the precision of its fused per-step bound)
__global__ void k_timestep_f32(int nc, const float* __restrict__ Uf, const double* __restrict__ vol,
                               const double* __restrict__ dx, float kappa, unsigned long long* conv_bits) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long bc = 0x7ff0000000000000ull;
  if (c < nc) {
    const float4* r = reinterpret_cast<const float4*>(Uf) + 2 * (size_t)c;
    const float4 a = r[0], b = r[1];
    const float ir = 1.f / a.x;
    const float u = a.y * ir, v = a.z * ir, w = a.w * ir;
    const float cs = sqrtf(kappa * b.y * ir);
    const double* d = dx + 3 * (size_t)c;
    const float ds = (fabsf(u) + cs) * (float)d[0] + (fabsf(v) + cs) * (float)d[1] + (fabsf(w) + cs) * (float)d[2];
    const double lc = (double)((float)vol[c] / ds);
    if (lc > 0.0) bc = (unsigned long long)__double_as_longlong(lc);
    if (!(lc == lc)) bc = 0x7ff8000000000000ull;
  }
  bc = warp_min_u64(bc);
  if ((threadIdx.x & 31) == 0) atomicMin(conv_bits, bc);
}

__global__ void k_export(int nc, int m, const int* __restrict__ perm, const double* __restrict__ S,
                         double* __restrict__ out, int with_prims, double km1, double R) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double q[10];
#pragma unroll
  for (int j = 0; j < 5; ++j) q[j] = (j < m) ? S[(size_t)j * nc + c] : 0.0;
  const int w = with_prims ? 10 : m;
  double* d = out + (size_t)w * perm[c];
  if (with_prims) {
    // eos.c:81-92 in FP64
    q[5] = q[1] / q[0];
    q[6] = q[2] / q[0];
    q[7] = q[3] / q[0];
    double ke = q[1] * q[5];
    ke += q[2] * q[6];
    ke += q[3] * q[7];
    q[8] = km1 * (q[4] - 0.5 * ke);
    q[8] = (1.00E-10 > q[8]) ? 1.00E-10 : q[8];
    q[9] = q[8] / (q[0] * R);
  }
  for (int j = 0; j < w; ++j) d[j] = q[j];
}

// calc_ns_timestep (navier_stokes.c:159-193) reduced over cells: min of the
// convective and viscous bounds (exact, order independent)
__global__ void k_timestep(int nc, const double* __restrict__ U, const double* __restrict__ vol,
                           const double* __restrict__ dx, double kappa, double km1,
                           unsigned long long* conv_bits, unsigned long long* visc_bits) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long bc = 0x7ff0000000000000ull, bv = 0x7ff0000000000000ull;
  if (c < nc) {
    double q[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = U[(size_t)j * nc + c];
    double u = q[1] / q[0], v = q[2] / q[0], w = q[3] / q[0];
    double ke = q[1] * u;
    ke += q[2] * v;
    ke += q[3] * w;
    double p = km1 * (q[4] - 0.5 * ke);
    p = (1.00E-10 > p) ? 1.00E-10 : p;
    double s_rho = 1.0 / q[0];
    double cs = sqrt(kappa * p * s_rho);
    const double* d = dx + 3 * (size_t)c;
    double ds1 = (fabs(u) + cs) * d[0] + (fabs(v) + cs) * d[1] + (fabs(w) + cs) * d[2];
    double lc = vol[c] / ds1;
    double ds2 = d[0] * d[0];
    ds2 += d[1] * d[1];
    ds2 += d[2] * d[2];
    double lv = s_rho * ds2 / vol[c];
    if (lc > 0.0) bc = (unsigned long long)__double_as_longlong(lc);
    if (lv > 0.0) bv = (unsigned long long)__double_as_longlong(lv);
    if (!(lc == lc) || !(lv == lv)) { bc = 0x7ff8000000000000ull; }
  }
  bc = warp_min_u64(bc);
  bv = warp_min_u64(bv);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(conv_bits, bc);
    atomicMin(visc_bits, bv);
  }
}

// end of an explicit step: advance time, next dt = cfl * min lambda
__global__ void k_finish_step(DevScalars* sc, double cfl) {
  sc->t += sc->dt;
  sc->step += 1;
  if (cfl > 0.0) {
    double lam = __longlong_as_double((long long)sc->lam_bits);
    sc->dt = lam * cfl;
    sc->lam_bits = 0x7ff0000000000000ull;
    if (!(sc->dt > 0.0) || isinf(sc->dt)) sc->status |= 1;
  }
}

__global__ void k_set_dt(DevScalars* sc, const unsigned long long* lam_bits, double cfl, double dt_fixed) {
  if (cfl > 0.0) sc->dt = __longlong_as_double((long long)lam_bits[0]) * cfl;
  else sc->dt = dt_fixed;
  sc->lam_bits = 0x7ff0000000000000ull;
  if (!(sc->dt > 0.0) || isinf(sc->dt)) sc->status |= 1;
}

// calc_global_residual (analyze.c:37-61): per-block partial sums, then one
// block sums the partials in a fixed order (deterministic)
__global__ void k_residual_partial(int nc, const double* __restrict__ dphi,
                                   const double* __restrict__ vol, double* __restrict__ part) {
  __shared__ double sh[5][256];
  int c = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
  for (int j = 0; j < 5; ++j) sh[j][threadIdx.x] = (c < nc) ? fabs(dphi[(size_t)j * nc + c]) * vol[c] : 0.0;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
#pragma unroll
      for (int j = 0; j < 5; ++j) sh[j][threadIdx.x] += sh[j][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int j = 0; j < 5; ++j) part[(size_t)blockIdx.x * 5 + j] = sh[j][0];
}

__global__ void k_residual_final(int nb, const double* __restrict__ part, double scale, double* out) {
  __shared__ double sh[5][256];
  double acc[5] = {0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
    for (int j = 0; j < 5; ++j) acc[j] += part[(size_t)b * 5 + j];
#pragma unroll
  for (int j = 0; j < 5; ++j) sh[j][threadIdx.x] = acc[j];
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
#pragma unroll
      for (int j = 0; j < 5; ++j) sh[j][threadIdx.x] += sh[j][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int j = 0; j < 5; ++j) out[j] = sh[j][0] * scale;
}

int nblk(int n, int t = 256) { return (n + t - 1) / t; }

}  // namespace

// ---------------------------------------------------------------------------
// context helpers
// ---------------------------------------------------------------------------
namespace fv3d {
fv3d_status Ctx::fail(fv3d_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  err = buf;
  return st;
}

fv3d_status Ctx::cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return FV3D_OK;
  return fail(FV3D_ERR_DEVICE, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr)                                              \
  do {                                                        \
    fv3d_status st__ = ctx->cuda((expr), #expr);              \
    if (st__ != FV3D_OK) return st__;                         \
  } while (0)

#define REQUIRE(cond, st, ...)                                \
  do {                                                        \
    if (!(cond)) return ctx->fail((st), __VA_ARGS__);         \
  } while (0)

void Ctx::release_graphs() {
  for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
  graphs.clear();
  if (implicit) implicit->release_graphs();  // they capture the same buffers and constants
}

template <class R>
KArgs<R> Ctx::args() const {
  KArgs<R> a;
  memset(&a, 0, sizeof(a));
  a.nc = nc; a.nf = nf; a.nf_int = nf_int; a.mcf = mcf;
  a.fc0 = d_fc0.p; a.fc1 = d_fc1.p;
  a.geo = (const R*)d_geo.p; a.lam = (const R*)d_lam.p; a.lsq = (const R*)d_lsq.p;
  a.fregion = d_fregion.p; a.cface = d_cface.p; a.rvol = (const R*)d_rvol.p;
  a.vol = d_vol.p; a.dx = d_dx.p;
  a.U = d_U.p; a.Pq = d_Pq.p; a.K = d_K.p; a.U0 = d_U0.p; a.Uf = d_Uf.p;
  a.rec = (R*)d_rec.p; a.FA = (R*)d_FA.p; a.dphi = d_dphi.p; a.sc = d_sc.p;
  a.pc = phys;
  return a;
}

template KArgs<double> Ctx::args<double>() const;

MxArgs Ctx::mx_args() const {
  MxArgs a;
  memset(&a, 0, sizeof(a));
  a.nc = nc; a.nf = nf; a.nf_int = nf_int; a.mcf = mcf; a.ncp = ncp;
  a.cface = d_cface.p; a.cnbr = d_cnbr.p; a.fcell = d_fcell.p; a.slotN = d_slotN.p;
  a.slotD = d_slotD.p; a.slotW = d_slotW.p; a.slotNk = d_slotNk.p; a.slotDk = d_slotDk.p; a.slotWk = d_slotWk.p; a.fregion = d_fregion.p; a.cgeo = d_cgeo.p; a.cdx = d_cdx.p;
  a.Uf = d_Uf.p; a.UfN = d_UfN.p; a.fs = d_fs.p; a.fsv = d_fsv.p; a.cother = d_cother.p;
  a.U = d_U.p; a.kf = d_kf.p; a.dU = d_dU.p; a.dphi = d_dphi.p; a.sc = d_sc.p;
  a.pc = phys;
  return a;
}

Disc Ctx::disc() const {
  Disc d;
  d.linear = cfg.reconstruction == FV3D_RECON_LINEAR;
  d.limit = cfg.limiter == FV3D_LIMITER_BARTH_JESPERSEN;
  d.viscous = cfg.mu_mix != 0.0;
  d.gmode = (!d.linear && !d.viscous) ? 0 : (cfg.gradient == FV3D_GRADIENT_LEAST_SQUARES ? 2 : 1);
  return d;
}

cudaError_t Ctx::launch_stage_kernels(int mode, bool dt, const StageCoef& co, int which) {
  cudaError_t e = cudaSuccess;
  const Disc d = disc();
  if (fp64()) {
    KArgs<double> a = args<double>();
    if (which & 1) e = launch_gradients<double>(a, d, stream);
    if (e == cudaSuccess && (which & 2)) e = launch_face_flux<double>(a, d, stream);
    if (e == cudaSuccess && (which & 4)) e = launch_gather<double>(a, mode, dt, co, stream);
  } else {
    // mixed path: bit 1 = gradient pass, bit 4 = flux + update pass
    MxArgs a = mx_args();
    if (which & 1) e = launch_mx_sides(a, d, stream);
    if (e == cudaSuccess && (which & 4)) e = launch_mx_flux_update(a, d, mode, dt, co, stream);
  }
  return e;
}
}  // namespace fv3d

// ---------------------------------------------------------------------------
// lifecycle
// ---------------------------------------------------------------------------
extern "C" const char* fv3d_version(void) { return "fv3d_gb300 1.0 (sm_103a)"; }

extern "C" fv3d_status fv3d_create(const fv3d_config* config, fv3d_ctx** out) {
  if (config == nullptr || out == nullptr) return FV3D_ERR_INVALID_ARG;
  *out = nullptr;
  Ctx* ctx = new Ctx();
  ctx->cfg = *config;
  const fv3d_config& c = *config;
  if (!(c.kappa > 1.0) || !(c.R_mix > 0.0) || !(c.mu_mix >= 0.0) || !(c.Pr > 0.0) ||
      c.flux_scheme < 0 || c.flux_scheme > 1 || c.reconstruction < 0 || c.reconstruction > 1 ||
      c.limiter < 0 || c.limiter > 1 || c.gradient < 0 || c.gradient > 1 || c.precision < 0 ||
      c.precision > 1 || c.renumber < 0 || c.renumber > 2) {
    delete ctx;
    return FV3D_ERR_INVALID_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || c.device < 0 || c.device >= ndev) {
    delete ctx;
    return FV3D_ERR_DEVICE;
  }
  if (cudaSetDevice(c.device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
      cudaMallocHost((void**)&ctx->h_sc, sizeof(DevScalars)) != cudaSuccess) {
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
    delete ctx;
    return FV3D_ERR_DEVICE;
  }
  // navier_stokes.c:85-124 derived constants
  PhysConst& p = ctx->phys;
  memset(&p, 0, sizeof(p));
  p.kappa = c.kappa;
  p.km1 = c.kappa - 1.0;
  p.kp1 = c.kappa + 1.0;
  p.s_km1 = 1.0 / p.km1;
  p.s_kp1 = 1.0 / p.kp1;
  p.R_mix = c.R_mix;
  p.mu = c.mu_mix;
  double cv = c.R_mix * p.s_km1;
  double cp = c.kappa * cv;
  p.heat_lambda = c.mu_mix * cp / c.Pr;
  p.flux = c.flux_scheme;
  p.f32[0] = (float)p.kappa; p.f32[1] = (float)p.km1; p.f32[2] = (float)p.s_km1;
  p.f32[3] = (float)p.s_kp1; p.f32[4] = (float)p.R_mix; p.f32[5] = (float)p.mu;
  p.f32[6] = (float)p.heat_lambda; p.f32[7] = 0.f;
  ctx->kappa_pr = c.kappa / c.Pr;
  *out = reinterpret_cast<fv3d_ctx*>(ctx);
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_destroy(fv3d_ctx* handle) {
  if (handle == nullptr) return FV3D_OK;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  cudaSetDevice(ctx->cfg.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->release_graphs();
  delete ctx->implicit;
  ctx->implicit = nullptr;
  delete ctx->mlp;
  ctx->mlp = nullptr;
  ctx->free_device();
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return FV3D_OK;
}

extern "C" const char* fv3d_last_error(const fv3d_ctx* handle) {
  if (handle == nullptr) return "null context";
  return reinterpret_cast<const Ctx*>(handle)->err.c_str();
}

extern "C" fv3d_status fv3d_get_stream(const fv3d_ctx* handle, void** stream) {
  if (handle == nullptr || stream == nullptr) return FV3D_ERR_INVALID_ARG;
  *stream = (void*)reinterpret_cast<const Ctx*>(handle)->stream;
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_selftest_bounded_wait(fv3d_ctx* handle, int limit_us, int* timed_out, double* elapsed_ms) {
  if (handle == nullptr || timed_out == nullptr || limit_us <= 0 || limit_us > 1000000) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  CK(cudaSetDevice(ctx->cfg.device));
  DevBuf<int> flag;
  CK(flag.alloc(1));
  CK(cudaMemsetAsync(flag.p, 0xff, sizeof(int), ctx->stream));
  cudaEvent_t ev[2];
  CK(cudaEventCreate(&ev[0]));
  CK(cudaEventCreate(&ev[1]));
  CK(cudaEventRecord(ev[0], ctx->stream));
  CK(launch_bounded_wait_probe(1000ull * (unsigned long long)limit_us, flag.p, ctx->stream));
  CK(cudaEventRecord(ev[1], ctx->stream));
  int h = -1;
  CK(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  *timed_out = h;
  if (elapsed_ms) *elapsed_ms = ms;
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_device_state(const fv3d_ctx* handle, double** u) {
  if (handle == nullptr || u == nullptr) return FV3D_ERR_INVALID_ARG;
  const Ctx* ctx = reinterpret_cast<const Ctx*>(handle);
  if (!ctx->mesh_ready) return FV3D_ERR_STATE;
  *u = ctx->d_U.p;
  return FV3D_OK;
}

// ---------------------------------------------------------------------------
// mesh
// ---------------------------------------------------------------------------
extern "C" fv3d_status fv3d_mesh_load_h5(fv3d_ctx* handle, const char* path) {
  if (handle == nullptr || path == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  return ctx->fail(FV3D_ERR_UNSUPPORTED,
                   "HDF5 mesh files are not supported by this build (no HDF5 library); "
                   "load the arrays and call fv3d_mesh_from_arrays");
}

extern "C" fv3d_status fv3d_get_permutation(const fv3d_ctx* handle, int* perm) {
  if (handle == nullptr || perm == nullptr) return FV3D_ERR_INVALID_ARG;
  const Ctx* ctx = reinterpret_cast<const Ctx*>(handle);
  if (!ctx->mesh_ready) return FV3D_ERR_STATE;
  std::copy(ctx->perm.begin(), ctx->perm.end(), perm);
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_mesh_from_arrays(fv3d_ctx* handle, const fv3d_mesh_arrays* m) {
  if (handle == nullptr || m == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  CK(cudaSetDevice(ctx->cfg.device));
  fv3d_status st = prepare_mesh(*ctx, *m);
  if (st != FV3D_OK) return st;
  return upload_mesh(*ctx);
}

extern "C" fv3d_status fv3d_set_region(fv3d_ctx* handle, int region, int type, const double prim[5]) {
  if (handle == nullptr || prim == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  REQUIRE(region >= 0 && region < MAX_REGIONS, FV3D_ERR_INVALID_ARG, "region %d out of range", region);
  REQUIRE(type >= FV3D_BC_FLOW && type <= FV3D_BC_PRESSURE_OUTLET && type != FV3D_BC_FUNCTION,
          FV3D_ERR_UNSUPPORTED, "boundary type %d not supported", type);
  PhysConst& p = ctx->phys;
  p.region_type[region] = type;
  double* q = p.region_phi[region];
  for (int j = 0; j < 10; ++j) q[j] = 0.0;
  // parse_primitive_state (boundary.c:144-183) + prim_to_con (eos.c:120-127)
  q[5] = prim[0]; q[6] = prim[1]; q[7] = prim[2]; q[8] = prim[3]; q[9] = prim[4];
  q[0] = q[8] / (ctx->cfg.R_mix * q[9]);
  q[1] = q[5] * q[0];
  q[2] = q[6] * q[0];
  q[3] = q[7] * q[0];
  double ke = q[5] * q[1];
  ke += q[6] * q[2];
  ke += q[7] * q[3];
  q[4] = p.s_km1 * q[8] + 0.5 * ke;
  for (int j = 0; j < 10; ++j) p.region_phi_f[region][j] = (float)q[j];
  p.n_regions = std::max(p.n_regions, region + 1);
  ctx->region_set |= 1u << region;
  ctx->release_graphs();  // physics constants are baked into captured graphs
  return FV3D_OK;
}

// ---------------------------------------------------------------------------
// state
// ---------------------------------------------------------------------------
static fv3d_status check_ready(Ctx* ctx) {
  if (!ctx->mesh_ready) return ctx->fail(FV3D_ERR_STATE, "no mesh loaded");
  for (int b = 0; b < ctx->nb; ++b) {
    int r = ctx->h_fregion[b];
    if (!(ctx->region_set & (1u << r)))
      return ctx->fail(FV3D_ERR_STATE, "boundary region %d has no condition (fv3d_set_region)", r);
  }
  return FV3D_OK;
}

// the device address of a caller buffer in page-locked host memory
// (cudaHostAlloc / cudaHostRegister), or null for pageable memory
static const double* pinned_device_view(const double* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // clear: an unknown pointer is pageable memory
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
  if (reinterpret_cast<uintptr_t>(at.devicePointer) % 16 != 0) return nullptr;  // the kernels use 16-byte accesses
  return static_cast<const double*>(at.devicePointer);
}

// the state from the caller's rows; with want_bound (mixed path, pinned
// rows) the import kernel also reduces the initial time-step bound into
// d_bits and *bound_done says so
static fv3d_status set_state_rows(Ctx* ctx, const double* u, bool want_bound, bool* bound_done) {
  if (bound_done != nullptr) *bound_done = false;
  if (!ctx->mesh_ready) return ctx->fail(FV3D_ERR_STATE, "no mesh loaded");
  CK(cudaSetDevice(ctx->cfg.device));
  const double* hdev = pinned_device_view(u);
  if (hdev != nullptr) {
    // pinned caller memory: one kernel reads it over the host link
    const bool bound = want_bound && !ctx->fp64() && ctx->d_Uf.p != nullptr;
    if (bound) CK(cudaMemsetAsync(ctx->d_bits.p, 0xff, 2 * sizeof(unsigned long long), ctx->stream));
    k_import_host<<<(ctx->nc + kIoRows - 1) / kIoRows, kIoRows, 0, ctx->stream>>>(
        ctx->nc, ctx->d_iperm.p, hdev, ctx->d_U.p, ctx->d_Uf.p, ctx->d_UfN.p, ctx->phys.km1, ctx->cfg.R_mix,
        ctx->d_vol.p, ctx->d_dx.p, (float)ctx->cfg.kappa, bound ? ctx->d_bits.p : nullptr);
    if (bound && bound_done != nullptr) *bound_done = true;
  } else {
    CK(cudaMemcpyAsync(ctx->d_stage.p, u, sizeof(double) * 5 * (size_t)ctx->nc, cudaMemcpyHostToDevice,
                       ctx->stream));
    k_import<<<nblk(ctx->nc), 256, 0, ctx->stream>>>(ctx->nc, ctx->d_perm.p, ctx->d_stage.p, ctx->d_U.p,
                                                    ctx->d_Uf.p, ctx->d_UfN.p, ctx->phys.km1,
                                                    ctx->cfg.R_mix);
  }
  CK(cudaGetLastError());
  ctx->state_ready = true;
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_set_state(fv3d_ctx* handle, const double* u) {
  if (handle == nullptr || u == nullptr) return FV3D_ERR_INVALID_ARG;
  return set_state_rows(reinterpret_cast<Ctx*>(handle), u, false, nullptr);
}

static fv3d_status export_soa(Ctx* ctx, const double* src, int m, int with_prims, double* out) {
  const int w = with_prims ? 10 : m;
  double* hdev = (with_prims || m != 5) ? nullptr : const_cast<double*>(pinned_device_view(out));
  if (hdev != nullptr) {
    // pinned caller memory: one kernel writes it over the host link
    k_export_host<<<(ctx->nc + kIoRows - 1) / kIoRows, kIoRows, 0, ctx->stream>>>(ctx->nc, ctx->d_iperm.p, src,
                                                                                  hdev);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    return FV3D_OK;
  }
  k_export<<<nblk(ctx->nc), 256, 0, ctx->stream>>>(ctx->nc, m, ctx->d_perm.p, src, ctx->d_stage.p,
                                                  with_prims, ctx->phys.km1, ctx->cfg.R_mix);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, ctx->d_stage.p, sizeof(double) * w * (size_t)ctx->nc, cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return FV3D_OK;
}

fv3d_status fv3d::export_rows(Ctx& c, const double* src, double* rows) {
  Ctx* ctx = &c;
  CK(cudaSetDevice(ctx->cfg.device));
  return export_soa(ctx, src, 5, 0, rows);
}

fv3d_status fv3d::import_rows(Ctx& c, const double* rows, double* dst) {
  Ctx* ctx = &c;
  CK(cudaSetDevice(ctx->cfg.device));
  CK(cudaMemcpyAsync(ctx->d_stage.p, rows, sizeof(double) * 5 * (size_t)ctx->nc, cudaMemcpyHostToDevice,
                     ctx->stream));
  k_import<<<nblk(ctx->nc), 256, 0, ctx->stream>>>(ctx->nc, ctx->d_perm.p, ctx->d_stage.p, dst, nullptr, nullptr,
                                                  ctx->phys.km1, ctx->cfg.R_mix);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_set_exact_function(fv3d_ctx* handle, fv3d_exact_fn fn, void* user, int id, double t) {
  if (handle == nullptr || fn == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mesh_ready) return ctx->fail(FV3D_ERR_STATE, "no mesh loaded");
  std::vector<double> u((size_t)ctx->nc * 5);
  double phi[10];
  for (int i = 0; i < ctx->nc; ++i) {
    for (int j = 0; j < 10; ++j) phi[j] = 0.0;
    fn(user, id, t, &ctx->h_cell_x[3 * (size_t)i], phi);
    for (int j = 0; j < 5; ++j) u[5 * (size_t)i + j] = phi[j];
  }
  return fv3d_set_state(handle, u.data());
}

extern "C" fv3d_status fv3d_get_state(fv3d_ctx* handle, double* phi_total) {
  if (handle == nullptr || phi_total == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "no state set");
  CK(cudaSetDevice(ctx->cfg.device));
  return export_soa(ctx, ctx->d_U.p, 5, 1, phi_total);
}

extern "C" fv3d_status fv3d_get_conserved(fv3d_ctx* handle, double* u) {
  if (handle == nullptr || u == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "no state set");
  CK(cudaSetDevice(ctx->cfg.device));
  return export_soa(ctx, ctx->d_U.p, 5, 0, u);
}

extern "C" fv3d_status fv3d_get_time_derivative(fv3d_ctx* handle, double* phi_dt) {
  if (handle == nullptr || phi_dt == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->residual_valid) return ctx->fail(FV3D_ERR_STATE, "no time derivative evaluated");
  CK(cudaSetDevice(ctx->cfg.device));
  return export_soa(ctx, ctx->d_dphi.p, 5, 0, phi_dt);
}

// ---------------------------------------------------------------------------
// hot path
// ---------------------------------------------------------------------------
extern "C" fv3d_status fv3d_time_derivative(fv3d_ctx* handle, double t, double* phi_dt) {
  (void)t;  // the implemented boundary conditions do not depend on time
  if (handle == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  fv3d_status st = check_ready(ctx);
  if (st != FV3D_OK) return st;
  if (!ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "no state set");
  CK(cudaSetDevice(ctx->cfg.device));
  StageCoef co{0, 0, 0, 0, 1, 1};
  CK(ctx->launch_stage_kernels(0, false, co, 7));
  ctx->residual_valid = true;
  if (phi_dt != nullptr) return export_soa(ctx, ctx->d_dphi.p, 5, 0, phi_dt);
  CK(cudaStreamSynchronize(ctx->stream));
  return FV3D_OK;
}

static fv3d_status reduce_timestep(Ctx* ctx, bool with_visc) {
  CK(cudaMemsetAsync(ctx->d_bits.p, 0xff, 2 * sizeof(unsigned long long), ctx->stream));
  // 0xff.. is larger than any positive double's bits; k_timestep mins into it
  k_timestep<<<nblk(ctx->nc), 256, 0, ctx->stream>>>(ctx->nc, ctx->d_U.p, ctx->d_vol.p, ctx->d_dx.p,
                                                    ctx->cfg.kappa, ctx->phys.km1, ctx->d_bits.p,
                                                    ctx->d_bits.p + 1);
  CK(cudaGetLastError());
  (void)with_visc;
  return FV3D_OK;
}

// the initial convective bound of an explicit run: FP32 records on the mixed
// path (as its fused per-step bound), FP64 state otherwise
static fv3d_status reduce_step_bound(Ctx* ctx) {
  if (ctx->fp64()) return reduce_timestep(ctx, false);
  CK(cudaMemsetAsync(ctx->d_bits.p, 0xff, 2 * sizeof(unsigned long long), ctx->stream));
  k_timestep_f32<<<nblk(ctx->nc), 256, 0, ctx->stream>>>(ctx->nc, ctx->d_Uf.p, ctx->d_vol.p, ctx->d_dx.p,
                                                        (float)ctx->cfg.kappa, ctx->d_bits.p);
  CK(cudaGetLastError());
  return FV3D_OK;
}


extern "C" fv3d_status fv3d_timestep(fv3d_ctx* handle, double cfl, double* dt) {
  if (handle == nullptr || dt == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "no state set");
  CK(cudaSetDevice(ctx->cfg.device));
  fv3d_status st = reduce_timestep(ctx, cfl <= 0.0);
  if (st != FV3D_OK) return st;
  unsigned long long bits[2];
  CK(cudaMemcpyAsync(bits, ctx->d_bits.p, sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  double lc, lv;
  memcpy(&lc, &bits[0], 8);
  memcpy(&lv, &bits[1], 8);
  if (bits[0] == ~0ull || !(lc > 0.0) || std::isinf(lc))
    return ctx->fail(FV3D_ERR_NONFINITE, "non-finite state in time step reduction");
  if (cfl > 0.0) {
    *dt = lc * cfl;
  } else {
    // navier_stokes.c:186-192, including its viscous branch as written
    lc *= ctx->cfg.cfl_scale;
    lv *= ctx->cfg.dfl_scale * ctx->cfg.mu_mix * ctx->kappa_pr * lv;
    *dt = (lc < lv) ? lc : lv;
  }
  return FV3D_OK;
}

// Williamson 2N low-storage tables (explicit.c:19-39): forward Euler,
// Williamson RK3, Carpenter-Kennedy RK4(5) - published coefficients.
static const double RK_A[3][5] = {
    {0.0},
    {0., -5. / 9., -153. / 128.},
    {0., -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
     -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0}};
static const double RK_G[3][5] = {
    {1.0},
    {1. / 3., 15. / 16., 8. / 15.},
    {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
     1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
     2277821191437.0 / 14882151754819.0}};
static const int RK_S[3] = {1, 3, 5};

// store_r: the last stage also stores its time derivative in dphi (what
// calc_global_residual reads after a reference step)
static fv3d_status enqueue_step(Ctx* ctx, int scheme, double cfl, bool store_r) {
  const bool dt_dev = cfl > 0.0;
  if (scheme == FV3D_SSP_RK3) {
    const double c0[3] = {0.0, 0.75, 1.0 / 3.0}, c1[3] = {1.0, 0.25, 2.0 / 3.0};
    for (int s = 0; s < 3; ++s) {
      StageCoef co{0, 0, c0[s], c1[s], s == 0, s == 2, store_r && s == 2};
      CK(ctx->launch_stage_kernels(2, dt_dev && s == 2, co, 7));
    }
  } else {
    for (int s = 0; s < RK_S[scheme]; ++s) {
      const bool last = s == RK_S[scheme] - 1;
      StageCoef co{RK_A[scheme][s], RK_G[scheme][s], 0, 0, s == 0, last, store_r && last};
      CK(ctx->launch_stage_kernels(1, dt_dev && last, co, 7));
    }
  }
  k_finish_step<<<1, 1, 0, ctx->stream>>>(ctx->d_sc.p, cfl);
  CK(cudaGetLastError());
  return FV3D_OK;
}

// the captured graph of one explicit step, built on first use
static fv3d_status step_graph(Ctx* ctx, int scheme, double cfl, bool store_r, cudaGraphExec_t* out) {
  const std::tuple<int, double, int> key(scheme, cfl, store_r ? 1 : 0);
  auto it = ctx->graphs.find(key);
  if (it != ctx->graphs.end()) {
    *out = it->second;
    return FV3D_OK;
  }
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  fv3d_status est = enqueue_step(ctx, scheme, cfl, store_r);
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
  if (est != FV3D_OK) {
    if (g) cudaGraphDestroy(g);
    return est;
  }
  CK(ce);
  ce = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  CK(ce);
  ctx->graphs[key] = exec;
  *out = exec;
  return FV3D_OK;
}

// n_steps explicit steps enqueued on the context stream (no synchronisation);
// the caller reads the device scalars afterwards (finish_explicit)
static fv3d_status enqueue_explicit(Ctx* ctx, int scheme, int n_steps, double cfl, double dt_fixed,
                                   bool bound_ready = false) {
  REQUIRE(scheme >= 0 && scheme <= 3, FV3D_ERR_INVALID_ARG, "bad explicit scheme %d", scheme);
  REQUIRE(n_steps >= 0, FV3D_ERR_INVALID_ARG, "negative step count");
  REQUIRE(cfl > 0.0 || dt_fixed > 0.0, FV3D_ERR_INVALID_ARG, "need cfl > 0 or dt_fixed > 0");
  fv3d_status st = check_ready(ctx);
  if (st != FV3D_OK) return st;
  if (!ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "no state set");
  // initial dt from the current state (timedisc.c:163-165 at the first step)
  CK(cudaMemsetAsync(ctx->d_sc.p, 0, sizeof(DevScalars), ctx->stream));
  if (cfl > 0.0 && !bound_ready) {
    st = reduce_step_bound(ctx);
    if (st != FV3D_OK) return st;
  }
  k_set_dt<<<1, 1, 0, ctx->stream>>>(ctx->d_sc.p, ctx->d_bits.p, cfl, dt_fixed);
  CK(cudaGetLastError());
  // one graph per (scheme, cfl) replayed n_steps times
  cudaGraphExec_t exec = nullptr;
  if ((st = step_graph(ctx, scheme, cfl, false, &exec)) != FV3D_OK) return st;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int i = 0; i < n_steps; ++i) CK(cudaGraphLaunch(exec, ctx->stream));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->residual_valid = false;
  return FV3D_OK;
}

// after the enqueued steps (and anything enqueued behind them) completed:
// the step statistics and status from the device scalars read into hs
static fv3d_status finish_explicit(Ctx* ctx, const DevScalars& hs, fv3d_step_stats* stats) {
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  if (stats != nullptr) {
    stats->t = hs.t;
    stats->dt = hs.dt;
    stats->steps = hs.step;
    stats->elapsed_ms = ms;
  }
  if (hs.status & kStatusStageTimeout)
    return ctx->fail(FV3D_ERR_TIMEOUT, "gradient pass: a tile's staged copies did not arrive within 0.5 s");
  if (hs.status & 1) return ctx->fail(FV3D_ERR_NONFINITE, "non-finite state or time step after %d steps", hs.step);
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_step_explicit(fv3d_ctx* handle, int scheme, int n_steps, double cfl,
                                          double dt_fixed, fv3d_step_stats* stats) {
  if (handle == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  CK(cudaSetDevice(ctx->cfg.device));
  fv3d_status st = enqueue_explicit(ctx, scheme, n_steps, cfl, dt_fixed);
  if (st != FV3D_OK) return st;
  DevScalars hs;
  CK(cudaMemcpyAsync(&hs, ctx->d_sc.p, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return finish_explicit(ctx, hs, stats);
}

extern "C" fv3d_status fv3d_step_explicit_io(fv3d_ctx* handle, int scheme, int n_steps, double cfl,
                                             double dt_fixed, const double* u_in, double* u_out,
                                             fv3d_step_stats* stats) {
  if (handle == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  fv3d_status st;
  // the initial time-step bound is taken by the import kernel where it can
  bool bound = false;
  if (u_in != nullptr && (st = set_state_rows(ctx, u_in, cfl > 0.0, &bound)) != FV3D_OK) return st;
  CK(cudaSetDevice(ctx->cfg.device));
  if ((st = enqueue_explicit(ctx, scheme, n_steps, cfl, dt_fixed, bound)) != FV3D_OK) return st;
  // scalars into page-locked memory (asynchronous), then the export, which
  // synchronises the stream once for both
  CK(cudaMemcpyAsync(ctx->h_sc, ctx->d_sc.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
  if (u_out != nullptr) {
    if ((st = export_soa(ctx, ctx->d_U.p, 5, 0, u_out)) != FV3D_OK) return st;
  } else {
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return finish_explicit(ctx, *ctx->h_sc, stats);
}

extern "C" fv3d_status fv3d_global_residual(fv3d_ctx* handle, double dt, double res[5]) {
  if (handle == nullptr || res == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->residual_valid) return ctx->fail(FV3D_ERR_STATE, "no residual evaluated (call fv3d_time_derivative)");
  CK(cudaSetDevice(ctx->cfg.device));
  const int nb = nblk(ctx->nc);
  k_residual_partial<<<nb, 256, 0, ctx->stream>>>(ctx->nc, ctx->d_dphi.p, ctx->d_vol.p, ctx->d_part.p);
  k_residual_final<<<1, 256, 0, ctx->stream>>>(nb, ctx->d_part.p, dt / ctx->vol_total, ctx->d_part.p + 5 * (size_t)nb);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(res, ctx->d_part.p + 5 * (size_t)nb, 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return FV3D_OK;
}

// ---------------------------------------------------------------------------
// calc_global_residual without any device allocation: the block partial sums
// and the five results live in one file-scope static device array of fixed
// size instead of the context's scratch.  Same kernels and grid as
// fv3d_global_residual, so the results are bitwise identical.
// ---------------------------------------------------------------------------
namespace {
constexpr int kNoAllocMaxBlocks = FV3D_NOALLOC_MAX_CELLS / 256;
constexpr int kNoAllocMaxDevices = 64;
// [kNoAllocMaxBlocks][5] block partials, then the 5 results (320 KiB).  Every
// slot a call reads is written earlier in that call, so nothing in it has to
// start at zero.  One array per device: calls that overlap on one device
// (other threads, other contexts' streams) race on it.
static __device__ __align__(256) double g_noalloc_part[5 * kNoAllocMaxBlocks + 5];
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};  // resolved by the first call on each device
}  // namespace

extern "C" fv3d_status fv3d_global_residual_noalloc(fv3d_ctx* handle, double dt, double res[5]) {
  if (handle == nullptr || res == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (ctx->mesh_ready && ctx->nc > FV3D_NOALLOC_MAX_CELLS)
    return ctx->fail(FV3D_ERR_UNSUPPORTED,
                     "fv3d_global_residual_noalloc: %d cells exceed its static scratch (at most %d cells); "
                     "use fv3d_global_residual",
                     ctx->nc, FV3D_NOALLOC_MAX_CELLS);
  if (!ctx->residual_valid) return ctx->fail(FV3D_ERR_STATE, "no residual evaluated (call fv3d_time_derivative)");
  const int dev = ctx->cfg.device;
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return ctx->fail(FV3D_ERR_UNSUPPORTED, "fv3d_global_residual_noalloc: device %d beyond %d", dev,
                     kNoAllocMaxDevices - 1);
  CK(cudaSetDevice(dev));
  double* part = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_part);
      if (e != cudaSuccess || p == nullptr)
        return ctx->fail(FV3D_ERR_DEVICE, "cudaGetSymbolAddress of the static residual scratch: %s",
                         cudaGetErrorString(e));
      g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    part = g_noalloc_ptr[dev];
  }
  const int nb = nblk(ctx->nc);
  k_residual_partial<<<nb, 256, 0, ctx->stream>>>(ctx->nc, ctx->d_dphi.p, ctx->d_vol.p, part);
  k_residual_final<<<1, 256, 0, ctx->stream>>>(nb, part, dt / ctx->vol_total, part + 5 * (size_t)nb);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(res, part + 5 * (size_t)nb, 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_profile_stage(fv3d_ctx* handle, int n_reps, double cfl, double* ms) {
  if (handle == nullptr || ms == nullptr || n_reps <= 0) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  fv3d_status st = check_ready(ctx);
  if (st != FV3D_OK) return st;
  CK(cudaSetDevice(ctx->cfg.device));
  cudaEvent_t ev[4];
  for (int i = 0; i < 4; ++i) CK(cudaEventCreate(&ev[i]));
  double acc[3] = {0, 0, 0};
  // keep the state unchanged: stage of a low-storage Euler step with dt = 0
  CK(cudaMemsetAsync(ctx->d_sc.p, 0, sizeof(DevScalars), ctx->stream));
  StageCoef co{0.0, 0.0, 0, 0, 1, 0};
  // FP64 path: gradients, face flux, gather+update; mixed path: gradient
  // pass, flux+update pass (ms[2] = 0)
  const int masks[3] = {1, ctx->fp64() ? 2 : 0, ctx->fp64() ? 4 : 4};
  for (int r = 0; r < n_reps; ++r) {
    CK(cudaEventRecord(ev[0], ctx->stream));
    CK(ctx->launch_stage_kernels(1, cfl > 0.0, co, masks[0]));
    CK(cudaEventRecord(ev[1], ctx->stream));
    if (ctx->fp64()) CK(ctx->launch_stage_kernels(1, cfl > 0.0, co, masks[1]));
    CK(cudaEventRecord(ev[2], ctx->stream));
    if (ctx->fp64()) CK(ctx->launch_stage_kernels(1, cfl > 0.0, co, masks[2]));
    else CK(ctx->launch_stage_kernels(1, cfl > 0.0, co, 4));
    CK(cudaEventRecord(ev[3], ctx->stream));
    CK(cudaEventSynchronize(ev[3]));
    for (int k = 0; k < 3; ++k) {
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
      acc[k] += t;
    }
  }
  for (int i = 0; i < 4; ++i) cudaEventDestroy(ev[i]);
  for (int k = 0; k < 3; ++k) ms[k] = acc[k] / n_reps;
  if (!ctx->fp64()) { ms[1] = ms[2]; ms[2] = 0.0; }
  return FV3D_OK;
}

// the kernels of n_steps real explicit steps (the launches a step graph
// replays, same coefficients, the dt computed on the device), each launch
// bracketed by CUDA events on the context stream: ms[0] the gradient pass,
// ms[1] the flux + update pass (FP64 path: face flux + gather), averaged
// over every stage, ms[2] the flux pass of the last stage alone.  The
// state advances by n_steps.
extern "C" fv3d_status fv3d_profile_step(fv3d_ctx* handle, int scheme, int n_steps, double cfl, double* ms) {
  if (handle == nullptr || ms == nullptr || n_steps <= 0) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  REQUIRE(scheme >= 0 && scheme <= 3, FV3D_ERR_INVALID_ARG, "bad explicit scheme %d", scheme);
  REQUIRE(cfl > 0.0, FV3D_ERR_INVALID_ARG, "need cfl > 0");
  fv3d_status st = check_ready(ctx);
  if (st != FV3D_OK) return st;
  if (!ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "no state set");
  CK(cudaSetDevice(ctx->cfg.device));
  CK(cudaMemsetAsync(ctx->d_sc.p, 0, sizeof(DevScalars), ctx->stream));
  if ((st = reduce_step_bound(ctx)) != FV3D_OK) return st;
  k_set_dt<<<1, 1, 0, ctx->stream>>>(ctx->d_sc.p, ctx->d_bits.p, cfl, 0.0);
  CK(cudaGetLastError());
  // one step captured as a graph with an event node at every launch
  // boundary (external events, recorded when the graph runs): the kernels
  // run exactly as the step graph runs them; one synchronisation per step
  const int ns = (scheme == FV3D_SSP_RK3) ? 3 : RK_S[scheme];
  cudaEvent_t ev[2 * 5 + 1] = {};
  for (int i = 0; i < 2 * ns + 1; ++i) CK(cudaEventCreate(&ev[i]));
  const int flux_mask = ctx->fp64() ? 6 : 4;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t ce = cudaEventRecordWithFlags(ev[0], ctx->stream, cudaEventRecordExternal);
  for (int s = 0; s < ns && ce == cudaSuccess; ++s) {
    const bool last = s == ns - 1;
    int mode = 1;
    StageCoef co{0, 0, 0, 0, s == 0, last, 0};
    if (scheme == FV3D_SSP_RK3) {
      const double c0[3] = {0.0, 0.75, 1.0 / 3.0}, c1[3] = {1.0, 0.25, 2.0 / 3.0};
      mode = 2;
      co.c0 = c0[s];
      co.c1 = c1[s];
    } else {
      co.a = RK_A[scheme][s];
      co.g = RK_G[scheme][s];
    }
    ce = ctx->launch_stage_kernels(mode, last, co, 1);
    if (ce == cudaSuccess) ce = cudaEventRecordWithFlags(ev[2 * s + 1], ctx->stream, cudaEventRecordExternal);
    if (ce == cudaSuccess) ce = ctx->launch_stage_kernels(mode, last, co, flux_mask);
    if (ce == cudaSuccess) ce = cudaEventRecordWithFlags(ev[2 * s + 2], ctx->stream, cudaEventRecordExternal);
  }
  if (ce == cudaSuccess) {
    k_finish_step<<<1, 1, 0, ctx->stream>>>(ctx->d_sc.p, cfl);
    ce = cudaGetLastError();
  }
  cudaError_t ee = cudaStreamEndCapture(ctx->stream, &g);
  if (ce == cudaSuccess) ce = ee;
  if (ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, g, 0);
  if (g) cudaGraphDestroy(g);
  double acc[3] = {0, 0, 0};
  for (int r = 0; r < n_steps && ce == cudaSuccess; ++r) {
    ce = cudaGraphLaunch(exec, ctx->stream);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(ev[2 * ns]);
    for (int s = 0; s < ns && ce == cudaSuccess; ++s) {
      float t0 = 0.f, t1 = 0.f;
      ce = cudaEventElapsedTime(&t0, ev[2 * s], ev[2 * s + 1]);
      if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t1, ev[2 * s + 1], ev[2 * s + 2]);
      acc[0] += t0;
      acc[1] += t1;
      if (s == ns - 1) acc[2] += t1;
    }
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
  if (exec) cudaGraphExecDestroy(exec);
  for (int i = 0; i < 2 * ns + 1; ++i) cudaEventDestroy(ev[i]);
  CK(ce);
  ms[0] = acc[0] / (n_steps * ns);
  ms[1] = acc[1] / (n_steps * ns);
  ms[2] = acc[2] / n_steps;
  ctx->residual_valid = false;
  return FV3D_OK;
}

// ---------------------------------------------------------------------------
// timedisc (timedisc.c:134-222): the step loop with its stop criteria
// ---------------------------------------------------------------------------
extern "C" fv3d_status fv3d_timedisc(fv3d_ctx* handle, const fv3d_timedisc_opts* o, fv3d_timedisc_stats* stats) {
  if (handle == nullptr || o == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  REQUIRE(o->implicit == 0 || o->implicit == 1, FV3D_ERR_INVALID_ARG, "bad time discretisation %d", o->implicit);
  REQUIRE(o->implicit ? (o->scheme == FV3D_NEWTON_EULER || o->scheme == FV3D_NEWTON_BDF2)
                      : (o->scheme >= 0 && o->scheme <= 3),
          FV3D_ERR_INVALID_ARG, "bad scheme %d", o->scheme);
  REQUIRE(o->max_iter >= 1, FV3D_ERR_INVALID_ARG, "max_iter must be >= 1");
  REQUIRE(o->iter_start >= 0, FV3D_ERR_INVALID_ARG, "iter_start must be >= 0");
  fv3d_status st = check_ready(ctx);
  if (st != FV3D_OK) return st;
  if (!ctx->state_ready) return ctx->fail(FV3D_ERR_STATE, "no state set");
  CK(cudaSetDevice(ctx->cfg.device));
  // steady runs have no end time (init_timedisc sets t_end = BC_DMAX)
  const double t_end = o->is_transient ? o->t_end : DBL_MAX;
  double t = o->t_start, dt = 0.0;
  double res[5] = {0, 0, 0, 0, 0};
  int iter = o->iter_start, reason = 0, n_inner = 0;
  bool finalize = false;
  const bool output = o->on_output != nullptr && o->i_output_data != 0;
  if (output && o->iter_start == 0) {
    // finite_volume_time_derivative(t) then write_output(0, t)
    if ((st = fv3d_time_derivative(handle, t, nullptr)) != FV3D_OK) return st;
    o->on_output(o->user, 0, t);
  }
  const bool dev_dt = !o->implicit && o->cfl > 0.0;
  // calc_ns_timestep as written after a low-storage step sees the reference's
  // phi_total: new density, the last stage's input u, v, w, p
  // (timestep_lserkw2 updates only the conserved entries, explicit.c:136-139).
  // Its convective bound is the one the last stage fuses (the graph runs it
  // with CFL 1); the viscous bound needs only the new density.
  const bool fused_lc = !o->implicit && o->cfl <= 0.0 && o->scheme != FV3D_SSP_RK3;
  cudaGraphExec_t exec = nullptr;
  if (!o->implicit) {
    if ((st = step_graph(ctx, o->scheme, fused_lc ? 1.0 : o->cfl, true, &exec)) != FV3D_OK) return st;
    DevScalars h0{};
    h0.t = t;
    h0.lam_bits = 0x7ff0000000000000ull;  // +inf: the fused bound mins into it
    CK(cudaMemcpyAsync(ctx->d_sc.p, &h0, sizeof(h0), cudaMemcpyHostToDevice, ctx->stream));
    if (dev_dt) {  // first dt from the initial state; later ones from each step's last stage
      if ((st = reduce_step_bound(ctx)) != FV3D_OK) return st;
      k_set_dt<<<1, 1, 0, ctx->stream>>>(ctx->d_sc.p, ctx->d_bits.p, o->cfl, 0.0);
      CK(cudaGetLastError());
    }
  }
  const int nb = nblk(ctx->nc);
  DevScalars hs{};
  while (true) {
    // time step: the device's (fused CFL) or calc_ns_timestep's / the
    // convective formula's from the current state
    if (dev_dt) {
      CK(cudaMemcpyAsync(&hs, ctx->d_sc.p, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      if (hs.status & 1) return ctx->fail(FV3D_ERR_NONFINITE, "non-finite state or time step at iteration %d", iter);
      dt = hs.dt;
    } else if (fused_lc && iter > o->iter_start) {
      CK(cudaMemcpyAsync(&hs, ctx->d_sc.p, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
      if ((st = reduce_timestep(ctx, true)) != FV3D_OK) return st;
      unsigned long long bits[2];
      CK(cudaMemcpyAsync(bits, ctx->d_bits.p, sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      if (hs.status & 1) return ctx->fail(FV3D_ERR_NONFINITE, "non-finite state or time step at iteration %d", iter);
      double lv;
      memcpy(&lv, &bits[1], 8);
      // navier_stokes.c:186-192
      const double lc = hs.dt * ctx->cfg.cfl_scale;
      lv *= ctx->cfg.dfl_scale * ctx->cfg.mu_mix * ctx->kappa_pr * lv;
      dt = (lc < lv) ? lc : lv;
    } else {
      if ((st = fv3d_timestep(handle, o->cfl, &dt)) != FV3D_OK) return st;
    }
    if (!(dt > 0.0) || std::isinf(dt))
      return ctx->fail(FV3D_ERR_NONFINITE, "time step %g at iteration %d", dt, iter);
    bool dt_changed = !dev_dt;
    if (t + dt > t_end) {
      dt = t_end - t;
      finalize = true;
      dt_changed = true;
      reason = 0;
    }
    if (!o->implicit) {
      if (dt_changed)
        CK(cudaMemcpyAsync(reinterpret_cast<char*>(ctx->d_sc.p) + offsetof(DevScalars, dt), &dt, sizeof(double),
                           cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaGraphLaunch(exec, ctx->stream));
      ctx->residual_valid = true;  // the last stage stored its time derivative
    } else {
      if (!ctx->implicit) ctx->implicit = new Implicit();
      fv3d_newton_opts no{o->scheme, o->max_iter_inner, o->is_transient};
      fv3d_newton_stats ns{};
      if ((st = ctx->implicit->step_newton(*ctx, no, iter, t, dt, &ns)) != FV3D_OK) return st;
      n_inner = ns.n_inner;
    }
    // calc_global_residual(dt) of the step's time derivative
    k_residual_partial<<<nb, 256, 0, ctx->stream>>>(ctx->nc, ctx->d_dphi.p, ctx->d_vol.p, ctx->d_part.p);
    k_residual_final<<<1, 256, 0, ctx->stream>>>(nb, ctx->d_part.p, dt / ctx->vol_total, ctx->d_part.p + 5 * (size_t)nb);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(res, ctx->d_part.p + 5 * (size_t)nb, sizeof(res), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int j = 0; j < 5; ++j)
      if (!std::isfinite(res[j])) return ctx->fail(FV3D_ERR_NONFINITE, "non-finite residual at iteration %d", iter);
    t = t + dt;
    iter = iter + 1;
    double rmax = res[0];
    for (int j = 1; j < 5; ++j) rmax = std::max(rmax, res[j]);
    if (!o->is_transient && rmax < o->abort_residual) {
      finalize = true;
      reason = 1;
    }
    const bool cadence = o->i_output_data > 0 && iter % o->i_output_data == 0;
    if (iter >= o->iter_start + o->max_iter && !finalize) {
      finalize = true;
      reason = 2;
    }
    if (o->on_iteration) o->on_iteration(o->user, iter, t, dt, res, n_inner);
    if (output && (finalize || cadence)) o->on_output(o->user, iter, t);
    if (finalize) break;
  }
  if (!o->implicit) {
    CK(cudaMemcpyAsync(&hs, ctx->d_sc.p, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (hs.status & kStatusStageTimeout)
      return ctx->fail(FV3D_ERR_TIMEOUT, "gradient pass: a tile's staged copies did not arrive within 0.5 s");
    if (hs.status & 1) return ctx->fail(FV3D_ERR_NONFINITE, "non-finite state at iteration %d", iter);
  }
  if (stats) {
    stats->iter = iter;
    stats->t = t;
    stats->dt = dt;
    for (int j = 0; j < 5; ++j) stats->res[j] = res[j];
    stats->stop_reason = reason;
  }
  return FV3D_OK;
}
