// The learned preconditioner's network on the fifth-generation tensor cores
// (sm_100 family: tcgen05.mma with the accumulator in tensor memory).
//
// One CTA of 128 threads takes tiles of 128 cells (M = 128: thread r of the
// CTA owns row r of the tile and TMEM lane r).  Per layer one thread issues
// the K/16 MMAs D[128 x N] = A[128 x K] W^T[K x N] (BF16 operands in shared
// memory, FP32 accumulation in TMEM: 64 columns), commits them to an
// mbarrier, and every warp reads its 32 lanes back with tcgen05.ld, adds the
// bias, applies GELU and writes the BF16 activations as the next layer's A
// operand.  The same roundings as the mma.sync kernels: BF16 inputs,
// weights and stored activations, FP32 accumulation and output.
//
// Operand layout: K-major, no swizzle.  A core matrix is 8 rows of 16 bytes
// (8 BF16 along K) stored as 128 contiguous bytes; core matrix (row group i,
// K group j) of a tile with KG K-groups sits at (i KG + j) 128 bytes, so the
// descriptor's leading byte offset (between core matrices along K) is 128
// and its stride byte offset (along M / N) KG 128.  One MMA (K = 16) reads
// two K-groups; the next starts 256 bytes further.
//
// Every wait on the mbarrier is bounded (0.5 s by %globaltimer); a wait that
// runs out sets *status and the CTA stops taking tiles (the host reports
// FV3D_ERR_TIMEOUT).
#include <cstddef>
#include <algorithm>

#include <cuda_bf16.h>

#include "context.h"
#include "implicit.h"
#include "mlp.cuh"

namespace fv3d {

namespace {

using bf16 = __nv_bfloat16;
constexpr int kTcRows = 128;      // M: cells per tile = threads per CTA
constexpr int kTcCols = 64;       // TMEM columns allocated (FP32 accumulator, N <= 64)
constexpr int kKG = 8;            // K-groups of the 64-wide operands
constexpr int kKG0 = 6;           // K-groups of the 48-wide input layer
constexpr unsigned long long kTcWaitNs = 500000000ull;

struct TcSmem {
  alignas(1024) bf16 A[kTcRows * 64];    // activations, core-matrix layout, 8 K-groups
  alignas(128) bf16 W0[64 * 48];         // [N = 64][K = 48]
  alignas(128) bf16 W1[64 * 64];
  alignas(128) bf16 W2[64 * 64];
  alignas(128) bf16 W3[16 * 64];         // [N = 16: 5 outputs, zero rows][K = 64]
  float b0[64], b1[64], b2[64], b3[16];
  alignas(8) unsigned long long bar;
  uint32_t tmem;
};

// byte offset of element (row, k) in a core-matrix tile of kg K-groups
__device__ __forceinline__ int core_off(int row, int k, int kg) {
  return ((row >> 3) * kg + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared memory matrix descriptor: start >> 4 [0,14), leading byte offset
// >> 4 [16,30), stride byte offset >> 4 [32,46), descriptor version 1 at
// bit 46, no swizzle (bits 61-63 zero)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1),
// BF16 A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17,
// M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ bool bar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool bar_wait_bounded(uint32_t bar, uint32_t parity) {
  if (bar_try_wait(bar, parity)) return true;
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  while (!bar_try_wait(bar, parity)) {
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > kTcWaitNs) return false;
  }
  return true;
}

__device__ __forceinline__ float tc_gelu(float x) { return mlp_gelu(x); }

// the FP32 master parameters as BF16 core-matrix tiles (W [out][in]: N x K,
// K-major) and FP32 biases, into the weight part of a TcSmem layout (here
// an image in device memory that each CTA of the network kernels copies)
__device__ void tc_load_weights(const float* __restrict__ P, TcSmem& S) {
  unsigned char* w0 = reinterpret_cast<unsigned char*>(S.W0);
  unsigned char* w1 = reinterpret_cast<unsigned char*>(S.W1);
  unsigned char* w2 = reinterpret_cast<unsigned char*>(S.W2);
  unsigned char* w3 = reinterpret_cast<unsigned char*>(S.W3);
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x, ts = gridDim.x * blockDim.x;
  for (int i = t0; i < 64 * 48; i += ts) {
    const int o = i / 48, k = i % 48;
    *reinterpret_cast<bf16*>(w0 + core_off(o, k, kKG0)) = __float2bfloat16(k < MLP_IN ? P[MLP_W0 + o * MLP_IN + k] : 0.f);
  }
  for (int i = t0; i < 64 * 64; i += ts) {
    const int o = i / 64, k = i % 64;
    *reinterpret_cast<bf16*>(w1 + core_off(o, k, kKG)) = __float2bfloat16(P[MLP_W1 + o * MLP_H + k]);
    *reinterpret_cast<bf16*>(w2 + core_off(o, k, kKG)) = __float2bfloat16(P[MLP_W2 + o * MLP_H + k]);
  }
  for (int i = t0; i < 16 * 64; i += ts) {
    const int o = i / 64, k = i % 64;
    *reinterpret_cast<bf16*>(w3 + core_off(o, k, kKG)) =
        __float2bfloat16(o < MLP_OUT ? P[MLP_W3 + o * MLP_H + k] : 0.f);
  }
  for (int i = t0; i < 64; i += ts) {
    S.b0[i] = P[MLP_B0 + i];
    S.b1[i] = P[MLP_B1 + i];
    S.b2[i] = P[MLP_B2 + i];
  }
  if (t0 < 16) S.b3[t0] = t0 < MLP_OUT ? P[MLP_B3 + t0] : 0.f;
}

// the packing kernel: the weight image in device memory
__global__ void k_mlp_pack_tc(const float* __restrict__ P, TcSmem* img) { tc_load_weights(P, *img); }

// bytes of the weight part of TcSmem (W0 .. b3), copied by one bulk copy
constexpr size_t kTcWeightOff = offsetof(TcSmem, W0);
constexpr size_t kTcWeightBytes = offsetof(TcSmem, bar) - offsetof(TcSmem, W0);
static_assert(kTcWeightOff % 16 == 0 && kTcWeightBytes % 16 == 0, "bulk copies move 16-byte multiples");

// the 8 BF16 of K-group j of this thread's row into the A tile
// (pairs rounded to nearest by one conversion each: the same values as one
// at a time)
__device__ __forceinline__ void put_group(TcSmem& S, int row, int j, const float* x) {
  __align__(16) __nv_bfloat162 h[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) h[l] = __floats2bfloat162_rn(x[2 * l], x[2 * l + 1]);
  *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.A) + core_off(row, 8 * j, kKG)) =
      *reinterpret_cast<const uint4*>(h);
}

// One layer's MMAs (one thread) and their completion.  Returns false when
// the wait ran out.
template <int KG, int N>
__device__ __forceinline__ bool tc_layer(TcSmem& S, const bf16* W, uint32_t tmem, uint32_t bar, uint32_t& phase) {
  if (threadIdx.x == 0) {
    tc_fence_after();
    const uint32_t a0 = smem_addr(S.A), w0 = smem_addr(W);
    constexpr uint32_t idesc = idesc_bf16(kTcRows, N);
#pragma unroll
    for (int s = 0; s < KG / 2; ++s)
      tc_mma(tmem, smem_desc(a0 + 256 * s, 128, kKG * 128), smem_desc(w0 + 256 * s, 128, KG * 128), idesc, s > 0);
    tc_commit(bar);
  }
  const bool ok = bar_wait_bounded(bar, phase);
  phase ^= 1u;
  tc_fence_after();
  return ok;
}

// a hidden layer's epilogue: the accumulator of this thread's row, 16
// columns at a time (few live registers), + bias, GELU, BF16 into A
__device__ __forceinline__ void tc_hidden_epilogue(TcSmem& S, uint32_t tmem, const float* bias) {
  const uint32_t lane_addr = tmem + ((uint32_t)(32 * (threadIdx.x >> 5)) << 16);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float acc[16];
    tc_ld16(lane_addr + 16 * c, acc);
    tc_wait_ld();
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = tc_gelu(acc[q] + bias[16 * c + q]);
    put_group(S, threadIdx.x, 2 * c, acc);
    put_group(S, threadIdx.x, 2 * c + 1, acc + 8);
  }
}

// rows of the tile: src holds `width` floats per row (rows contiguous);
// with width <= 32 the CTA stages the tile's rows through the A buffer (free
// at the start of a tile) with coalesced 16-byte loads, otherwise IN reads
// src itself; IN(row, row's floats, x[48]) fills a row's inputs (false: no
// such row), OUT(row, y[5]) takes its outputs
template <class IN, class OUT>
__device__ void tc_forward(const TcSmem* __restrict__ img, int n, int* status, const float* __restrict__ src,
                           int width, IN in, OUT out) {
  extern __shared__ __align__(1024) unsigned char tc_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(tc_raw + ((1024 - (smem_addr(tc_raw) & 1023)) & 1023));
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t bar = smem_addr(&S.bar);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&S.tmem)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // the packed weights: one bulk copy, completing phase 0 of the barrier
    const uint32_t dst = smem_addr(S.W0);
    const unsigned char* srcw = reinterpret_cast<const unsigned char*>(img) + kTcWeightOff;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"((uint32_t)kTcWeightBytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(srcw), "r"((uint32_t)kTcWeightBytes), "r"(bar)
                 : "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  if (__syncthreads_or(!bar_wait_bounded(bar, 0))) {
    // the weights did not land in time (every thread takes this branch):
    // report, wait once more so that the copy does not outlive the CTA,
    // free the tensor memory
    if (tid == 0) atomicOr(status, 1);
    bar_wait_bounded(bar, 0);
    if (warp == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
    return;
  }
  uint32_t phase = 1;
  const int tiles = (n + kTcRows - 1) / kTcRows;
  for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int row = t * kTcRows + tid;
    {
      const bool staged = width <= 32;   // the tile's rows fit the 16 KB A buffer
      const float* rowp = src + (size_t)row * width;
      if (staged) {
        const int rows = min(kTcRows, n - t * kTcRows);
        const float4* g = reinterpret_cast<const float4*>(src + (size_t)t * kTcRows * width);
        float4* st = reinterpret_cast<float4*>(S.A);
        for (int i = tid; i < rows * width / 4; i += kTcRows) st[i] = __ldg(g + i);
        __syncthreads();
        rowp = reinterpret_cast<const float*>(S.A) + tid * width;
      }
      float x[48];
      if (!in(row, rowp, x))
#pragma unroll
        for (int k = 0; k < 48; ++k) x[k] = 0.f;
      if (staged) __syncthreads();         // every row read before A takes the inputs
#pragma unroll
      for (int j = 0; j < 6; ++j) put_group(S, tid, j, x + 8 * j);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    bool ok = tc_layer<kKG0, 64>(S, S.W0, tmem, bar, phase);
    const float* bias[3] = {S.b0, S.b1, S.b2};
    const bf16* W[3] = {S.W1, S.W2, S.W3};
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      tc_hidden_epilogue(S, tmem, bias[l]);
      fence_async_smem();
      tc_fence_before();
      if (__syncthreads_or(!ok)) break;
      if (l < 2) ok = tc_layer<kKG, 64>(S, W[l], tmem, bar, phase);
      else ok = tc_layer<kKG, 16>(S, W[l], tmem, bar, phase);
    }
    float y[16];
    tc_ld16(tmem + ((uint32_t)(32 * warp) << 16), y);
    tc_wait_ld();
    tc_fence_before();
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(status, 1);
      break;
    }
#pragma unroll
    for (int o = 0; o < MLP_OUT; ++o) y[o] += S.b3[o];
    out(row, y);
  }
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
}

__global__ void __launch_bounds__(kTcRows, 1) k_mlp_forward_tc(const TcSmem* __restrict__ img,
                                                               const float* __restrict__ X, int n,
                                                               float* __restrict__ Y, int* status) {
  tc_forward(
      img, n, status, X, MLP_IN,
      [&](int row, const float* xs, float* x) {
        if (row >= n) return false;
        for (int k = 0; k < 48; ++k) x[k] = (k < MLP_IN) ? xs[k] : 0.f;
        return true;
      },
      [&](int row, const float* y) {
        if (row >= n) return;
        for (int o = 0; o < MLP_OUT; ++o) Y[(size_t)row * MLP_OUT + o] = y[o];
      });
}

// z = M(v) inside FGMRES: the features of k_mlp_apply, rescaled by |v| / ||D||_F
template <class T>
__global__ void __launch_bounds__(kTcRows, 1) k_mlp_apply_tc(const TcSmem* __restrict__ img, int nc,
                                                             const float* __restrict__ feat,
                                                             const T* __restrict__ v, T* __restrict__ z,
                                                             int* status) {
  tc_forward(
      img, nc, status, feat, MLP_FEAT,
      [&](int c, const float* fs, float* x) {
        if (c >= nc) return false;
        float vv[5], s = 0.f;
        for (int j = 0; j < 5; ++j) {
          vv[j] = (float)v[(size_t)j * nc + c];
          s += vv[j] * vv[j];
        }
        const float vn = sqrtf(s), iv = (vn > 0.f) ? 1.f / vn : 0.f;
        for (int k = 0; k < 31; ++k) x[k] = fs[k];
        for (int j = 0; j < 5; ++j) x[31 + j] = vv[j] * iv;
        for (int k = MLP_IN; k < 48; ++k) x[k] = 0.f;
        return true;
      },
      [&](int c, const float* y) {
        if (c >= nc) return;
        float s = 0.f;
        for (int j = 0; j < 5; ++j) {
          const float e = (float)v[(size_t)j * nc + c];
          s += e * e;
        }
        const float sc = sqrtf(s) * feat[(size_t)c * MLP_FEAT + 31];
        for (int o = 0; o < MLP_OUT; ++o) z[(size_t)o * nc + c] = (T)(y[o] * sc);
      });
}

// persistent grid of the network kernels: this many CTAs per
// multiprocessor (5 fit: 43 KB of shared memory, 64 tensor-memory columns
// and 95 registers x 128 threads each; measured on the channel 3 / 4 / 5:
// 41.9 / 39.2 / 36.4 us per application)
#ifndef FV3D_TC_CTAS_PER_SM
#define FV3D_TC_CTAS_PER_SM 5
#endif
int tc_grid(int tiles) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 1;
  }
  return std::max(1, std::min(tiles, FV3D_TC_CTAS_PER_SM * sms));
}

constexpr size_t kTcSmem = sizeof(TcSmem) + 1024;  // + alignment slack
constexpr int kTcPackBlocks = 16;                    // 4,096 threads pack the 11,013 parameters

}  // namespace

#define TCK(expr)                                                  \
  do {                                                             \
    cudaError_t e__ = (expr);                                      \
    if (e__ != cudaSuccess) return ctx.cuda(e__, #expr);           \
  } while (0)

fv3d_status Mlp::tc_setup(Ctx& ctx) {
  if (tc_ready) return FV3D_OK;
  TCK(cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
  TCK(cudaFuncSetAttribute(k_mlp_apply_tc<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
  TCK(cudaFuncSetAttribute(k_mlp_apply_tc<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
  TCK(tc_status.alloc(1));
  TCK(cudaMemset(tc_status.p, 0, sizeof(int)));
  TCK(tc_img.alloc(sizeof(TcSmem)));
  TCK(cudaMemset(tc_img.p, 0, sizeof(TcSmem)));
  tc_ready = true;
  return FV3D_OK;
}

fv3d_status Mlp::forward_tc(Ctx& ctx, const float* dX, int n, float* dY) {
  fv3d_status st = tc_setup(ctx);
  if (st != FV3D_OK) return st;
  TcSmem* img = reinterpret_cast<TcSmem*>(tc_img.p);
  k_mlp_pack_tc<<<kTcPackBlocks, 256, 0, ctx.stream>>>(P.p, img);
  k_mlp_forward_tc<<<tc_grid((n + kTcRows - 1) / kTcRows), kTcRows, kTcSmem, ctx.stream>>>(img, dX, n, dY,
                                                                                         tc_status.p);
  TCK(cudaGetLastError());
  return FV3D_OK;
}

// inside FGMRES: may be captured in a CUDA graph, so no set-up here (Mlp::init did it)
template <class VT>
fv3d_status Mlp::apply_tc(Ctx& ctx, const VT* v, VT* z) {
  if (!tc_ready) return ctx.fail(FV3D_ERR_STATE, "tcgen05 kernels not set up");
  // the weight image from the current parameters (they change between
  // training steps), then the network
  TcSmem* img = reinterpret_cast<TcSmem*>(tc_img.p);
  k_mlp_pack_tc<<<kTcPackBlocks, 256, 0, ctx.stream>>>(P.p, img);
  k_mlp_apply_tc<VT><<<tc_grid((ctx.nc + kTcRows - 1) / kTcRows), kTcRows, kTcSmem, ctx.stream>>>(
      img, ctx.nc, feat.p, v, z, tc_status.p);
  TCK(cudaGetLastError());
  return FV3D_OK;
}

template fv3d_status Mlp::apply_tc<float>(Ctx&, const float*, float*);
template fv3d_status Mlp::apply_tc<double>(Ctx&, const double*, double*);

}  // namespace fv3d
