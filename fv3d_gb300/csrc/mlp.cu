// Learned preconditioner: per-cell MLP forward / backward / Adam kernels
// (hand-written, BF16 tensor-core operands via mma.sync m16n8k16, FP32
// accumulation), feature construction from the block-Jacobi blocks, the
// harvest of (residual, Newton correction) training pairs from the plain
// implicit solver, and the training loop.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "context.h"
#include "implicit.h"
#include "mlp.cuh"

namespace fv3d {

namespace {

using bf16 = __nv_bfloat16;
constexpr int LD_H = 72;  // bf16 leading dim of 64-wide tiles (conflict-free fragment loads)
constexpr int LD_X = 56;  // bf16 leading dim of the 48-wide input tile
constexpr int LD_O = 24;  // bf16 leading dim of 16-wide output tiles
constexpr int LDF = 72;   // float leading dim

__device__ __forceinline__ uint32_t ld2(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t ld2s(const bf16* lo, const bf16* hi) {
  const uint32_t a = *reinterpret_cast<const uint16_t*>(lo), b = *reinterpret_cast<const uint16_t*>(hi);
  return a | (b << 16);
}

__device__ __forceinline__ void mma16816(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu(float x) { return mlp_gelu(x); }
__device__ __forceinline__ float gelu_d(float x) { return mlp_gelu_d(x); }

struct MlpW {  // BF16 weights in the layouts the fragments read
  bf16 W0[MLP_H * LD_X];   // [out][in]
  bf16 W1[MLP_H * LD_H];
  bf16 W2[MLP_H * LD_H];
  bf16 W3[8 * LD_H];
  float b0[MLP_H], b1[MLP_H], b2[MLP_H], b3[8];
};

struct MlpBwdW {  // transposed weights for the delta products
  bf16 W1T[MLP_H * LD_H];  // [in][out]
  bf16 W2T[MLP_H * LD_H];
  bf16 W3T[MLP_H * LD_O];
};

struct MlpAct {
  bf16 x[MLP_TILE * LD_X];
  bf16 a1[MLP_TILE * LD_H], a2[MLP_TILE * LD_H], a3[MLP_TILE * LD_H];
  float h1[MLP_TILE * LDF], h2[MLP_TILE * LDF], h3[MLP_TILE * LDF];
  float y[MLP_TILE * 8];
};

struct MlpTrainSmem {
  MlpW w;
  MlpBwdW wt;
  MlpAct act;
  bf16 dy[MLP_TILE * LD_O];
  bf16 d3[MLP_TILE * LD_H], d2[MLP_TILE * LD_H], d1[MLP_TILE * LD_H];
  float red[4];
};

__device__ void load_weights(const float* __restrict__ P, MlpW& w, MlpBwdW* wt) {
  for (int i = threadIdx.x; i < MLP_H * LD_X; i += blockDim.x) {
    const int o = i / LD_X, k = i % LD_X;
    w.W0[i] = __float2bfloat16(k < MLP_IN ? P[MLP_W0 + o * MLP_IN + k] : 0.f);
  }
  for (int i = threadIdx.x; i < MLP_H * LD_H; i += blockDim.x) {
    const int o = i / LD_H, k = i % LD_H;
    const bool ok = k < MLP_H;
    w.W1[i] = __float2bfloat16(ok ? P[MLP_W1 + o * MLP_H + k] : 0.f);
    w.W2[i] = __float2bfloat16(ok ? P[MLP_W2 + o * MLP_H + k] : 0.f);
    if (wt) {  // W^T[in = o][out = k]
      wt->W1T[i] = __float2bfloat16(ok ? P[MLP_W1 + k * MLP_H + o] : 0.f);
      wt->W2T[i] = __float2bfloat16(ok ? P[MLP_W2 + k * MLP_H + o] : 0.f);
    }
  }
  for (int i = threadIdx.x; i < 8 * LD_H; i += blockDim.x) {
    const int o = i / LD_H, k = i % LD_H;
    w.W3[i] = __float2bfloat16((o < MLP_OUT && k < MLP_H) ? P[MLP_W3 + o * MLP_H + k] : 0.f);
  }
  if (wt)
    for (int i = threadIdx.x; i < MLP_H * LD_O; i += blockDim.x) {
      const int in = i / LD_O, o = i % LD_O;
      wt->W3T[i] = __float2bfloat16(o < MLP_OUT ? P[MLP_W3 + o * MLP_H + in] : 0.f);
    }
  for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
    w.b0[i] = P[MLP_B0 + i];
    w.b1[i] = P[MLP_B1 + i];
    w.b2[i] = P[MLP_B2 + i];
  }
  if (threadIdx.x < 8) w.b3[threadIdx.x] = threadIdx.x < MLP_OUT ? P[MLP_B3 + threadIdx.x] : 0.f;
}

// One warp: C[16 rows of the warp][N] = A[16][K] * B, B in "col" layout
// (element (k, n) at B[n * ldb + k]); epilogue per (row, col, value).
template <class Epi>
__device__ __forceinline__ void warp_gemm(const bf16* A, int lda, const bf16* B, int ldb, int K, int N,
                                          Epi epi) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  for (int nt = 0; nt < N / 8; ++nt) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    for (int kt = 0; kt < K / 16; ++kt) {
      const int k0 = kt * 16 + 2 * t;
      const uint32_t a0 = ld2(A + g * lda + k0), a1 = ld2(A + (g + 8) * lda + k0);
      const uint32_t a2 = ld2(A + g * lda + k0 + 8), a3 = ld2(A + (g + 8) * lda + k0 + 8);
      const bf16* bp = B + (nt * 8 + g) * ldb + k0;
      mma16816(c, a0, a1, a2, a3, ld2(bp), ld2(bp + 8));
    }
    const int col = nt * 8 + 2 * t;
    epi(g, col, c[0]);
    epi(g, col + 1, c[1]);
    epi(g + 8, col, c[2]);
    epi(g + 8, col + 1, c[3]);
  }
}

// forward of the warp's 16 rows; keeps the pre-activations (training) when
// the activation struct has them
__device__ __forceinline__ float* pre_act(MlpAct& s, int l) { return l == 1 ? s.h1 : (l == 2 ? s.h2 : s.h3); }

template <class Act>
__device__ void mlp_forward_warp(const MlpW& w, Act& s, int r0, bool keep) {
  const bf16* x = s.x + r0 * LD_X;
  bf16* a1 = s.a1 + r0 * LD_H;
  bf16* a2 = s.a2 + r0 * LD_H;
  bf16* a3 = s.a3 + r0 * LD_H;
  float* h1 = keep ? pre_act(s, 1) + r0 * LDF : nullptr;
  float* h2 = keep ? pre_act(s, 2) + r0 * LDF : nullptr;
  float* h3 = keep ? pre_act(s, 3) + r0 * LDF : nullptr;
  warp_gemm(x, LD_X, w.W0, LD_X, MLP_INP, MLP_H, [&](int r, int c, float v) {
    v += w.b0[c];
    if (keep) h1[r * LDF + c] = v;
    a1[r * LD_H + c] = __float2bfloat16(gelu(v));
  });
  __syncwarp();
  warp_gemm(a1, LD_H, w.W1, LD_H, MLP_H, MLP_H, [&](int r, int c, float v) {
    v += w.b1[c];
    if (keep) h2[r * LDF + c] = v;
    a2[r * LD_H + c] = __float2bfloat16(gelu(v));
  });
  __syncwarp();
  warp_gemm(a2, LD_H, w.W2, LD_H, MLP_H, MLP_H, [&](int r, int c, float v) {
    v += w.b2[c];
    if (keep) h3[r * LDF + c] = v;
    a3[r * LD_H + c] = __float2bfloat16(gelu(v));
  });
  __syncwarp();
  float* y = s.y + r0 * 8;
  warp_gemm(a3, LD_H, w.W3, LD_H, MLP_H, 8, [&](int r, int c, float v) { y[r * 8 + c] = v + w.b3[c]; });
  __syncwarp();
}

// ---------------------------------------------------------------------------
// training step: forward + backward over one tile of 64 samples per CTA;
// per-CTA partial gradients (deterministic reduction afterwards)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_mlp_train(const float* __restrict__ P, const float* __restrict__ X,
                                                   const float* __restrict__ T, const float* __restrict__ Wt,
                                                   const int* __restrict__ idx, int nbatch, float inv_b,
                                                   float* __restrict__ part, float* __restrict__ loss_part) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpTrainSmem& S = *reinterpret_cast<MlpTrainSmem*>(smem_raw);
  const int base = blockIdx.x * MLP_TILE;
  load_weights(P, S.w, &S.wt);
  for (int i = threadIdx.x; i < MLP_TILE * LD_X; i += blockDim.x) {
    const int r = i / LD_X, k = i % LD_X;
    const int sidx = (base + r < nbatch) ? idx[base + r] : -1;
    S.act.x[i] = __float2bfloat16((sidx >= 0 && k < MLP_IN) ? X[(size_t)sidx * MLP_IN + k] : 0.f);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = warp * 16;
  mlp_forward_warp(S.w, S.act, r0, true);
  // output delta dL/dy = 2 w (y - t) / B  (weighted mean over samples of the
  // sum over outputs; w = 1 without a weight array)
  float lsum = 0.f;
  for (int i = lane; i < 16 * LD_O; i += 32) {
    const int r = r0 + i / LD_O, o = i % LD_O;
    const int sidx = (base + r < nbatch) ? idx[base + r] : -1;
    float d = 0.f;
    if (sidx >= 0 && o < MLP_OUT) {
      const float w = Wt ? Wt[sidx] : 1.f;
      const float e = S.act.y[r * 8 + o] - T[(size_t)sidx * MLP_OUT + o];
      lsum += w * e * e;
      d = 2.f * w * e * inv_b;
    }
    if (o < 8) S.act.y[r * 8 + o] = d;  // keep the FP32 delta for db3
    S.dy[r * LD_O + o] = __float2bfloat16(d);
  }
  __syncwarp();
  // delta3 = (dy W3) * gelu'(h3); FP32 copy in h3, BF16 copy in d3
  warp_gemm(S.dy + r0 * LD_O, LD_O, S.wt.W3T, LD_O, 16, MLP_H, [&](int r, int c, float v) {
    float* h = S.act.h3 + (r0 + r) * LDF + c;
    const float d = v * gelu_d(*h);
    *h = d;
    S.d3[(r0 + r) * LD_H + c] = __float2bfloat16(d);
  });
  __syncwarp();
  warp_gemm(S.d3 + r0 * LD_H, LD_H, S.wt.W2T, LD_H, MLP_H, MLP_H, [&](int r, int c, float v) {
    float* h = S.act.h2 + (r0 + r) * LDF + c;
    const float d = v * gelu_d(*h);
    *h = d;
    S.d2[(r0 + r) * LD_H + c] = __float2bfloat16(d);
  });
  __syncwarp();
  warp_gemm(S.d2 + r0 * LD_H, LD_H, S.wt.W1T, LD_H, MLP_H, MLP_H, [&](int r, int c, float v) {
    float* h = S.act.h1 + (r0 + r) * LDF + c;
    const float d = v * gelu_d(*h);
    *h = d;
    S.d1[(r0 + r) * LD_H + c] = __float2bfloat16(d);
  });
  // loss of the tile
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) S.red[warp] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) loss_part[blockIdx.x] = S.red[0] + S.red[1] + S.red[2] + S.red[3];
  // weight gradients dW[o][i] = sum_s delta[s][o] act[s][i]: the sample index
  // is the reduction dimension, so both operands are read transposed
  float* G = part + (size_t)blockIdx.x * MLP_NPARAM;
  const int g = lane >> 2, t = lane & 3;
  auto dw = [&](const bf16* D, int ldd, const bf16* Aact, int lda, int mt, int N, int n_out, int n_in, int off) {
    for (int nt = 0; nt < N / 8; ++nt) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      for (int kt = 0; kt < MLP_TILE / 16; ++kt) {
        const int s0 = kt * 16 + 2 * t;
        const int o0 = mt * 16 + g;
        const uint32_t a0 = ld2s(D + s0 * ldd + o0, D + (s0 + 1) * ldd + o0);
        const uint32_t a1 = ld2s(D + s0 * ldd + o0 + 8, D + (s0 + 1) * ldd + o0 + 8);
        const uint32_t a2 = ld2s(D + (s0 + 8) * ldd + o0, D + (s0 + 9) * ldd + o0);
        const uint32_t a3 = ld2s(D + (s0 + 8) * ldd + o0 + 8, D + (s0 + 9) * ldd + o0 + 8);
        const int i0 = nt * 8 + g;
        const uint32_t b0 = ld2s(Aact + s0 * lda + i0, Aact + (s0 + 1) * lda + i0);
        const uint32_t b1 = ld2s(Aact + (s0 + 8) * lda + i0, Aact + (s0 + 9) * lda + i0);
        mma16816(c, a0, a1, a2, a3, b0, b1);
      }
      const int o = mt * 16 + g, i = nt * 8 + 2 * t;
      if (o < n_out && i < n_in) G[off + o * n_in + i] = c[0];
      if (o < n_out && i + 1 < n_in) G[off + o * n_in + i + 1] = c[1];
      if (o + 8 < n_out && i < n_in) G[off + (o + 8) * n_in + i] = c[2];
      if (o + 8 < n_out && i + 1 < n_in) G[off + (o + 8) * n_in + i + 1] = c[3];
    }
  };
  // each warp takes one 16-row block of output units
  dw(S.d1, LD_H, S.act.x, LD_X, warp, MLP_INP, MLP_H, MLP_IN, MLP_W0);
  dw(S.d2, LD_H, S.act.a1, LD_H, warp, MLP_H, MLP_H, MLP_H, MLP_W1);
  dw(S.d3, LD_H, S.act.a2, LD_H, warp, MLP_H, MLP_H, MLP_H, MLP_W2);
  if (warp == 0) dw(S.dy, LD_O, S.act.a3, LD_H, 0, MLP_H, MLP_OUT, MLP_H, MLP_W3);
  // bias gradients from the FP32 deltas
  if (threadIdx.x < MLP_H) {
    const int c = threadIdx.x;
    float s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int r = 0; r < MLP_TILE; ++r) {
      s1 += S.act.h1[r * LDF + c];
      s2 += S.act.h2[r * LDF + c];
      s3 += S.act.h3[r * LDF + c];
    }
    G[MLP_B0 + c] = s1;
    G[MLP_B1 + c] = s2;
    G[MLP_B2 + c] = s3;
  } else if (threadIdx.x < MLP_H + MLP_OUT) {
    const int o = threadIdx.x - MLP_H;
    float s = 0.f;
    for (int r = 0; r < MLP_TILE; ++r) s += S.act.y[r * 8 + o];
    G[MLP_B3 + o] = s;
  }
}

__global__ void k_mlp_reduce(int nparts, const float* __restrict__ part, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_NPARAM) return;
  float s = 0.f;
  for (int c = 0; c < nparts; ++c) s += part[(size_t)c * MLP_NPARAM + p];
  grad[p] = s;
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_NPARAM) return;
  const float gi = g[p];
  const float mi = b1 * m[p] + (1.f - b1) * gi;
  const float vi = b2 * v[p] + (1.f - b2) * gi * gi;
  m[p] = mi;
  v[p] = vi;
  P[p] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// forward over host-provided samples (tests): X [n][36] -> Y [n][5]
// ---------------------------------------------------------------------------
// register-resident forward for inference: one warp runs 16 rows through all
// four layers.  The m16n8k16 accumulator fragment of n-tiles 2q and 2q+1
// (rows g, g+8; columns 2t, 2t+1 of each) is exactly the A fragment of the
// next layer's k-chunk q, so activations never leave registers; only the
// weights (B fragments) come from shared memory.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// one hidden layer: h = gelu(A W^T + b), K = 16 * KC input columns, 64 outputs
template <int KC>
__device__ __forceinline__ void fused_layer(const uint32_t (&a)[KC][4], const bf16* W, int ldw, const float* b,
                                            uint32_t (&out)[4][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float h[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kt = 0; kt < KC; ++kt) {
      const bf16* bp = W + (nt * 8 + g) * ldw + kt * 16 + 2 * t;
      mma16816(c, a[kt][0], a[kt][1], a[kt][2], a[kt][3], ld2(bp), ld2(bp + 8));
    }
    const float b0 = b[nt * 8 + 2 * t], b1 = b[nt * 8 + 2 * t + 1];
    h[nt][0] = gelu(c[0] + b0);
    h[nt][1] = gelu(c[1] + b1);
    h[nt][2] = gelu(c[2] + b0);
    h[nt][3] = gelu(c[3] + b1);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    out[q][0] = pack_bf16(h[2 * q][0], h[2 * q][1]);
    out[q][1] = pack_bf16(h[2 * q][2], h[2 * q][3]);
    out[q][2] = pack_bf16(h[2 * q + 1][0], h[2 * q + 1][1]);
    out[q][3] = pack_bf16(h[2 * q + 1][2], h[2 * q + 1][3]);
  }
}

// x (A fragments of the 48-wide input, 3 k-chunks) -> y: this thread's
// outputs (row g: y[0], y[1] for outputs 2t, 2t+1; row g + 8: y[2], y[3])
__device__ __forceinline__ void fused_forward(const MlpW& w, const uint32_t (&x)[3][4], float (&y)[4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t a1[4][4], a2[4][4], a3[4][4];
  fused_layer<3>(x, w.W0, LD_X, w.b0, a1);
  fused_layer<4>(a1, w.W1, LD_H, w.b1, a2);
  fused_layer<4>(a2, w.W2, LD_H, w.b2, a3);
  float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
    const bf16* bp = w.W3 + g * LD_H + kt * 16 + 2 * t;
    mma16816(c, a3[kt][0], a3[kt][1], a3[kt][2], a3[kt][3], ld2(bp), ld2(bp + 8));
  }
  const float b0 = w.b3[2 * t], b1 = w.b3[2 * t + 1];
  y[0] = c[0] + b0;
  y[1] = c[1] + b1;
  y[2] = c[2] + b0;
  y[3] = c[3] + b1;
}

// the input fragments of one row pair from a per-row value function x(row, k)
template <class X>
__device__ __forceinline__ void input_fragments(X xval, uint32_t (&x)[3][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int kt = 0; kt < 3; ++kt) {
    const int k0 = kt * 16 + 2 * t;
    x[kt][0] = pack_bf16(xval(g, k0), xval(g, k0 + 1));
    x[kt][1] = pack_bf16(xval(g + 8, k0), xval(g + 8, k0 + 1));
    x[kt][2] = pack_bf16(xval(g, k0 + 8), xval(g, k0 + 9));
    x[kt][3] = pack_bf16(xval(g + 8, k0 + 8), xval(g + 8, k0 + 9));
  }
}

constexpr int kInfWarps = 8;  // warps per inference CTA

// inference kernels: persistent CTAs of kInfWarps warps; the weights are
// converted into shared memory once per CTA, then every warp takes 16-row
// groups in turn through the register-resident forward
__global__ void __launch_bounds__(32 * kInfWarps) k_mlp_forward(const float* __restrict__ P,
                                                                const float* __restrict__ X, int n,
                                                                float* __restrict__ Y) {
  __shared__ __align__(16) MlpW W;
  load_weights(P, W, nullptr);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int groups = (n + 15) / 16;
  for (int grp = blockIdx.x * kInfWarps + (threadIdx.x >> 5); grp < groups; grp += gridDim.x * kInfWarps) {
    const int r0 = grp * 16;
    uint32_t x[3][4];
    input_fragments(
        [&](int r, int k) {
          return (r0 + r < n && k < MLP_IN) ? X[(size_t)(r0 + r) * MLP_IN + k] : 0.f;
        },
        x);
    float y[4];
    fused_forward(W, x, y);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int row = r0 + g + 8 * h;
      if (row >= n) continue;
      if (2 * t < MLP_OUT) Y[(size_t)row * MLP_OUT + 2 * t] = y[2 * h];
      if (2 * t + 1 < MLP_OUT) Y[(size_t)row * MLP_OUT + 2 * t + 1] = y[2 * h + 1];
    }
  }
}

// preconditioner application z = M(v) (vectors in FP64 or, for the FP32
// Krylov basis, FP32): features of each cell from its block / geometry
// record and its vector, MLP, rescale by |v| / ||D||_F
template <class T>
__global__ void __launch_bounds__(32 * kInfWarps) k_mlp_apply(const float* __restrict__ P, int nc,
                                                              const float* __restrict__ feat,
                                                              const T* __restrict__ v, T* __restrict__ z) {
  __shared__ __align__(16) MlpW W;
  load_weights(P, W, nullptr);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int groups = (nc + 15) / 16;
  for (int grp = blockIdx.x * kInfWarps + (threadIdx.x >> 5); grp < groups; grp += gridDim.x * kInfWarps) {
    const int r0 = grp * 16;
    // |v| of this thread's two rows
    float vn[2], iv[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = r0 + g + 8 * h;
      float s = 0.f;
      if (c < nc)
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          const float e = (float)v[(size_t)j * nc + c];
          s += e * e;
        }
      vn[h] = sqrtf(s);
      iv[h] = (vn[h] > 0.f) ? 1.f / vn[h] : 0.f;
    }
    uint32_t x[3][4];
    input_fragments(
        [&](int r, int k) {
          const int c = r0 + r;
          if (c >= nc || k >= MLP_IN) return 0.f;
          if (k < 31) return feat[(size_t)c * MLP_FEAT + k];
          return (float)v[(size_t)(k - 31) * nc + c] * iv[r >= 8 ? 1 : 0];
        },
        x);
    float y[4];
    fused_forward(W, x, y);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = r0 + g + 8 * h;
      if (c >= nc) continue;
      const float sc = vn[h] * feat[(size_t)c * MLP_FEAT + 31];
      if (2 * t < MLP_OUT) z[(size_t)(2 * t) * nc + c] = (T)(y[2 * h] * sc);
      if (2 * t + 1 < MLP_OUT) z[(size_t)(2 * t + 1) * nc + c] = (T)(y[2 * h + 1] * sc);
    }
  }
}

// per-cell feature record: D / ||D||_F (25), A_k / V^(2/3) (6), 1 / ||D||_F
__global__ void k_mlp_features(int nc, int mcf, const int* __restrict__ cface, const double* __restrict__ geo,
                               const double* __restrict__ vol, const double* __restrict__ D,
                               float* __restrict__ feat) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double s = 0.0;
  for (int j = 0; j < 25; ++j) s += D[(size_t)c * 25 + j] * D[(size_t)c * 25 + j];
  const double inv = (s > 0.0) ? 1.0 / sqrt(s) : 0.0;
  float* f = feat + (size_t)c * MLP_FEAT;
  for (int j = 0; j < 25; ++j) f[j] = (float)(D[(size_t)c * 25 + j] * inv);
  const double v23 = cbrt(vol[c] * vol[c]);
  for (int k = 0; k < 6; ++k) {
    const int e = (k < mcf) ? cface[(size_t)c * mcf + k] : -1;
    f[25 + k] = (e >= 0) ? (float)(geo[(size_t)(e >> 1) * GEO + G_A] / v23) : 0.f;
  }
  f[31] = (float)inv;
}

// training pairs from a Newton step: cells c_j = (j0 + j * stride) mod nc
// with raw weights (|r_c| / ||D_c||_F)^2: the squared size of the cell's
// block-Jacobi output, so that a cell whose local residual is tiny next to its
// Newton correction (a correction carried in from elsewhere) does not dominate
__global__ void k_mlp_harvest(int nc, int count, long long j0, long long stride, const float* __restrict__ feat,
                              const double* __restrict__ r, const double* __restrict__ x,
                              float* __restrict__ X, float* __restrict__ T, float* __restrict__ Wt) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= count) return;
  const int c = (int)((j0 + (long long)j * stride) % nc);
  double rn = 0.0;
  for (int k = 0; k < 5; ++k) rn += r[(size_t)k * nc + c] * r[(size_t)k * nc + c];
  rn = sqrt(rn);
  const float* f = feat + (size_t)c * MLP_FEAT;
  float* Xo = X + (size_t)j * MLP_IN;
  float* To = T + (size_t)j * MLP_OUT;
  for (int k = 0; k < 31; ++k) Xo[k] = f[k];
  const double scale = (rn > 0.0 && f[31] > 0.f) ? 1.0 / (rn * (double)f[31]) : 0.0;
  for (int k = 0; k < 5; ++k) {
    Xo[31 + k] = (rn > 0.0) ? (float)(r[(size_t)k * nc + c] / rn) : 0.f;
    To[k] = (float)(x[(size_t)k * nc + c] * scale);
  }
  const double b = rn * (double)f[31];
  Wt[j] = (float)(b * b);
}

// one Newton step's weights divided by their mean (steps of very different
// residual size weigh alike); one CTA, fixed-order reduction
__global__ void __launch_bounds__(256) k_mlp_weight_norm(int count, float* __restrict__ Wt) {
  __shared__ double red[256];
  double s = 0.0;
  for (int j = threadIdx.x; j < count; j += 256) s += Wt[j];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double mean = red[0] / count;
  const float inv = (mean > 0.0) ? (float)(1.0 / mean) : 0.f;
  for (int j = threadIdx.x; j < count; j += 256) Wt[j] *= inv;
}

size_t train_smem() { return sizeof(MlpTrainSmem); }
// persistent inference grids: resident CTAs of the device
int inference_grid(int ntiles) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 1;
  }
  return std::max(1, std::min(ntiles, sms * 3));  // 3 CTAs of 8 warps per SM (80 registers)
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
#define MCK(expr)                                               \
  do {                                                          \
    fv3d_status st__ = ctx.cuda((expr), #expr);                 \
    if (st__ != FV3D_OK) return st__;                           \
  } while (0)

fv3d_status Mlp::init(Ctx& ctx, unsigned long long seed) {
  MCK(P.alloc(MLP_NPARAM));
  MCK(m.alloc(MLP_NPARAM));
  MCK(v.alloc(MLP_NPARAM));
  MCK(grad.alloc(MLP_NPARAM));
  std::vector<float> h(MLP_NPARAM, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off, int nout, int nin, double gain) {
    std::normal_distribution<double> nd(0.0, gain / sqrt((double)nin));
    for (int i = 0; i < nout * nin; ++i) h[off + i] = (float)nd(rng);
  };
  fill(MLP_W0, MLP_H, MLP_IN, sqrt(2.0));
  fill(MLP_W1, MLP_H, MLP_H, sqrt(2.0));
  fill(MLP_W2, MLP_H, MLP_H, sqrt(2.0));
  fill(MLP_W3, MLP_OUT, MLP_H, 0.1);
  MCK(cudaMemcpy(P.p, h.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice));
  MCK(cudaMemset(m.p, 0, sizeof(float) * MLP_NPARAM));
  MCK(cudaMemset(v.p, 0, sizeof(float) * MLP_NPARAM));
  adam_t = 0;
  ready = true;
  MCK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
  return tc_setup(ctx);  // outside any stream capture: the solve's graphs launch the tcgen05 kernels
}

fv3d_status Mlp::ensure_scratch(Ctx& ctx, int nbatch) {
  const int nparts = (nbatch + MLP_TILE - 1) / MLP_TILE;
  if (part.n < (size_t)nparts * MLP_NPARAM) MCK(part.alloc((size_t)nparts * MLP_NPARAM));
  if (loss_part.n < (size_t)nparts) MCK(loss_part.alloc(nparts));
  if (bidx.n < (size_t)nbatch) MCK(bidx.alloc(nbatch));
  return FV3D_OK;
}

fv3d_status Mlp::forward_host(Ctx& ctx, const float* X, int n, float* Y) {
  DevBuf<float> dX, dY;
  MCK(dX.alloc((size_t)n * MLP_IN));
  MCK(dY.alloc((size_t)n * MLP_OUT));
  MCK(cudaMemcpy(dX.p, X, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice));
  if (use_tc) {
    fv3d_status st = forward_tc(ctx, dX.p, n, dY.p);
    if (st != FV3D_OK) return st;
  } else {
    k_mlp_forward<<<inference_grid((n + 16 * kInfWarps - 1) / (16 * kInfWarps)), 32 * kInfWarps, 0, ctx.stream>>>(
        P.p, dX.p, n, dY.p);
  }
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(ctx.stream));
  if (use_tc) {
    int flag = 0;
    MCK(cudaMemcpy(&flag, tc_status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
      MCK(cudaMemset(tc_status.p, 0, sizeof(int)));
      return ctx.fail(FV3D_ERR_TIMEOUT, "tcgen05 forward: a bounded wait for the tensor cores ran out");
    }
  }
  MCK(cudaMemcpy(Y, dY.p, sizeof(float) * n * MLP_OUT, cudaMemcpyDeviceToHost));
  return FV3D_OK;
}

fv3d_status Mlp::grad_host(Ctx& ctx, const float* X, const float* T, int n, double* loss, float* g) {
  DevBuf<float> dX, dT;
  MCK(dX.alloc((size_t)n * MLP_IN));
  MCK(dT.alloc((size_t)n * MLP_OUT));
  MCK(cudaMemcpy(dX.p, X, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(dT.p, T, sizeof(float) * n * MLP_OUT, cudaMemcpyHostToDevice));
  fv3d_status st = ensure_scratch(ctx, n);
  if (st != FV3D_OK) return st;
  std::vector<int> id(n);
  std::iota(id.begin(), id.end(), 0);
  MCK(cudaMemcpy(bidx.p, id.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  const int nparts = (n + MLP_TILE - 1) / MLP_TILE;
  k_mlp_train<<<nparts, 128, train_smem(), ctx.stream>>>(P.p, dX.p, dT.p, nullptr, bidx.p, n, 1.f / n, part.p,
                                                         loss_part.p);
  k_mlp_reduce<<<(MLP_NPARAM + 255) / 256, 256, 0, ctx.stream>>>(nparts, part.p, grad.p);
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(ctx.stream));
  std::vector<float> lp(nparts);
  MCK(cudaMemcpy(lp.data(), loss_part.p, sizeof(float) * nparts, cudaMemcpyDeviceToHost));
  double L = 0.0;
  for (float x : lp) L += x;
  *loss = L / n;
  MCK(cudaMemcpy(g, grad.p, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost));
  return FV3D_OK;
}

// one Adam step of the master parameters with the gradient in grad
// (beta1 0.9, beta2 0.999, eps 1e-8; bias corrections from the step count)
fv3d_status Mlp::adam_step(Ctx& ctx, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  adam_t += 1;
  const float c1 = 1.f - powf(b1, (float)adam_t), c2 = 1.f - powf(b2, (float)adam_t);
  k_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, ctx.stream>>>(P.p, grad.p, m.p, v.p, lr, b1, b2, eps, c1, c2);
  MCK(cudaGetLastError());
  return FV3D_OK;
}

fv3d_status Mlp::train(Ctx& ctx, const fv3d_mlp_train_opts& o, fv3d_mlp_train_stats* stats) {
  if (n_samples <= 0) return ctx.fail(FV3D_ERR_STATE, "no training samples harvested");
  const int B = std::max(MLP_TILE, (o.batch / MLP_TILE) * MLP_TILE);
  fv3d_status st = ensure_scratch(ctx, B);
  if (st != FV3D_OK) return st;
  DevBuf<int> perm;
  MCK(perm.alloc((size_t)n_samples));
  std::vector<int> h(n_samples);
  std::mt19937_64 rng(o.seed);
  const auto t0 = std::chrono::steady_clock::now();
  const int nparts = B / MLP_TILE;
  double first = -1.0, last = 0.0;
  for (int ep = 0; ep < o.epochs; ++ep) {
    std::iota(h.begin(), h.end(), 0);
    std::shuffle(h.begin(), h.end(), rng);
    MCK(cudaMemcpyAsync(perm.p, h.data(), sizeof(int) * n_samples, cudaMemcpyHostToDevice, ctx.stream));
    double esum = 0.0;
    int ebat = 0;
    std::vector<float> lp(nparts);
    for (int b0 = 0; b0 + B <= n_samples; b0 += B) {
      k_mlp_train<<<nparts, 128, train_smem(), ctx.stream>>>(P.p, X.p, T.p, Wt.p, perm.p + b0, B, 1.f / B,
                                                             part.p, loss_part.p);
      k_mlp_reduce<<<(MLP_NPARAM + 255) / 256, 256, 0, ctx.stream>>>(nparts, part.p, grad.p);
      if ((st = adam_step(ctx, (float)o.lr)) != FV3D_OK) return st;
      if (b0 == 0 || b0 + 2 * B > n_samples) {  // loss of the first and last batch of the epoch
        MCK(cudaMemcpyAsync(lp.data(), loss_part.p, sizeof(float) * nparts, cudaMemcpyDeviceToHost, ctx.stream));
        MCK(cudaStreamSynchronize(ctx.stream));
        double L = 0.0;
        for (float x : lp) L += x;
        esum += L / B;
        ebat += 1;
        if (first < 0.0) first = L / B;
        last = L / B;
      }
    }
    (void)esum;
    (void)ebat;
  }
  MCK(cudaStreamSynchronize(ctx.stream));
  if (stats) {
    stats->loss_first = first;
    stats->loss_last = last;
    stats->samples = n_samples;
    stats->steps = adam_t;
    stats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return FV3D_OK;
}

fv3d_status Mlp::build_features(Ctx& ctx, const Implicit& im) {
  if (feat.n < (size_t)ctx.nc * MLP_FEAT) MCK(feat.alloc((size_t)ctx.nc * MLP_FEAT));
  k_mlp_features<<<(ctx.nc + 255) / 256, 256, 0, ctx.stream>>>(ctx.nc, ctx.mcf, ctx.d_cface.p,
                                                               (const double*)ctx.d_geo.p, ctx.d_vol.p, im.D.p,
                                                               feat.p);
  MCK(cudaGetLastError());
  return FV3D_OK;
}

fv3d_status Mlp::apply(Ctx& ctx, const double* vin, double* zout) {
  if (use_tc) return apply_tc<double>(ctx, vin, zout);
  k_mlp_apply<double><<<inference_grid((ctx.nc + 16 * kInfWarps - 1) / (16 * kInfWarps)), 32 * kInfWarps, 0,
                        ctx.stream>>>(P.p, ctx.nc, feat.p, vin,
                                                                                          zout);
  MCK(cudaGetLastError());
  return FV3D_OK;
}

fv3d_status Mlp::apply(Ctx& ctx, const float* vin, float* zout) {
  if (use_tc) return apply_tc<float>(ctx, vin, zout);
  k_mlp_apply<float><<<inference_grid((ctx.nc + 16 * kInfWarps - 1) / (16 * kInfWarps)), 32 * kInfWarps, 0,
                       ctx.stream>>>(P.p, ctx.nc, feat.p, vin,
                                                                                         zout);
  MCK(cudaGetLastError());
  return FV3D_OK;
}

fv3d_status Mlp::harvest(Ctx& ctx, const Implicit& im) {
  if (harvest_per_step <= 0 || n_samples >= max_samples) return FV3D_OK;
  const int count = std::min(harvest_per_step, max_samples - n_samples);
  if (X.n < (size_t)max_samples * MLP_IN) {
    MCK(X.alloc((size_t)max_samples * MLP_IN));
    MCK(T.alloc((size_t)max_samples * MLP_OUT));
    MCK(Wt.alloc((size_t)max_samples));
  }
  // a deterministic spread of cells: stride coprime-ish with nc, offset per step
  const long long stride = 2654435761LL % ctx.nc + 1;
  const long long j0 = (long long)harvest_calls * 7919LL;
  k_mlp_harvest<<<(count + 255) / 256, 256, 0, ctx.stream>>>(ctx.nc, count, j0, stride, feat.p, im.R.p, im.x.p,
                                                             X.p + (size_t)n_samples * MLP_IN,
                                                             T.p + (size_t)n_samples * MLP_OUT,
                                                             Wt.p + n_samples);
  k_mlp_weight_norm<<<1, 256, 0, ctx.stream>>>(count, Wt.p + n_samples);
  MCK(cudaGetLastError());
  n_samples += count;
  harvest_calls += 1;
  return FV3D_OK;
}

}  // namespace fv3d

using namespace fv3d;

static Mlp* mlp_of(Ctx* ctx) {
  if (!ctx->mlp) ctx->mlp = new Mlp();
  return ctx->mlp;
}

extern "C" fv3d_status fv3d_mlp_init(fv3d_ctx* handle, unsigned long long seed) {
  if (handle == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "cudaSetDevice");
  if (ctx->implicit) ctx->implicit->release_graphs();  // captured steps hold the old parameter buffer
  return mlp_of(ctx)->init(*ctx, seed);
}

extern "C" fv3d_status fv3d_mlp_get_params(fv3d_ctx* handle, float* params) {
  if (handle == nullptr || params == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mlp || !ctx->mlp->ready) return ctx->fail(FV3D_ERR_STATE, "MLP not initialised");
  if (cudaMemcpy(params, ctx->mlp->P.p, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost) != cudaSuccess)
    return ctx->fail(FV3D_ERR_DEVICE, "copy parameters");
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_mlp_set_params(fv3d_ctx* handle, const float* params) {
  if (handle == nullptr || params == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mlp || !ctx->mlp->ready) return ctx->fail(FV3D_ERR_STATE, "MLP not initialised");
  if (cudaMemcpy(ctx->mlp->P.p, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice) != cudaSuccess)
    return ctx->fail(FV3D_ERR_DEVICE, "copy parameters");
  return FV3D_OK;
}

extern "C" int fv3d_mlp_num_params(void) { return MLP_NPARAM; }

extern "C" fv3d_status fv3d_profile_mlp(fv3d_ctx* handle, int n_reps, double* ms) {
  if (handle == nullptr || ms == nullptr || n_reps < 1) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  Mlp* net = ctx->mlp;
  if (!net || !net->ready || net->feat.n < (size_t)ctx->nc * MLP_FEAT)
    return ctx->fail(FV3D_ERR_STATE, "no network or no cell features (run a learned or harvesting solve first)");
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "cudaSetDevice");
  DevBuf<float> v, z;
  if (v.alloc(5 * (size_t)ctx->nc) != cudaSuccess || z.alloc(5 * (size_t)ctx->nc) != cudaSuccess)
    return ctx->fail(FV3D_ERR_DEVICE, "allocation");
  std::vector<float> h(5 * (size_t)ctx->nc);
  for (size_t i = 0; i < h.size(); ++i) h[i] = 1.f + 0.25f * (float)((i * 2654435761u) % 97) / 97.f;
  if (cudaMemcpy(v.p, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return ctx->fail(FV3D_ERR_DEVICE, "copy");
  fv3d_status st = net->apply(*ctx, v.p, z.p);  // warm-up
  if (st != FV3D_OK) return st;
  if (cudaEventRecord(ctx->ev0, ctx->stream) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "event");
  for (int r = 0; r < n_reps; ++r)
    if ((st = net->apply(*ctx, v.p, z.p)) != FV3D_OK) return st;
  float t = 0.f;
  if (cudaEventRecord(ctx->ev1, ctx->stream) != cudaSuccess || cudaEventSynchronize(ctx->ev1) != cudaSuccess ||
      cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1) != cudaSuccess)
    return ctx->fail(FV3D_ERR_DEVICE, "timing");
  *ms = t / n_reps;
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_mlp_set_kernel(fv3d_ctx* handle, int tensor_core) {
  if (handle == nullptr || (tensor_core != 0 && tensor_core != 1)) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (ctx->implicit) ctx->implicit->release_graphs();  // captured steps hold the inference kernel
  mlp_of(ctx)->use_tc = tensor_core == 1;
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_mlp_adam_step(fv3d_ctx* handle, const float* grad, double lr) {
  if (handle == nullptr || grad == nullptr) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mlp || !ctx->mlp->ready) return ctx->fail(FV3D_ERR_STATE, "MLP not initialised");
  if (!(lr > 0.0)) return ctx->fail(FV3D_ERR_INVALID_ARG, "learning rate must be positive");
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "cudaSetDevice");
  Mlp& net = *ctx->mlp;
  if (cudaMemcpy(net.grad.p, grad, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice) != cudaSuccess)
    return ctx->fail(FV3D_ERR_DEVICE, "copy gradient");
  fv3d_status st = net.adam_step(*ctx, (float)lr);
  if (st != FV3D_OK) return st;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return ctx->fail(FV3D_ERR_DEVICE, "Adam step");
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_mlp_forward(fv3d_ctx* handle, const float* X, int n, float* Y) {
  if (handle == nullptr || X == nullptr || Y == nullptr || n <= 0) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mlp || !ctx->mlp->ready) return ctx->fail(FV3D_ERR_STATE, "MLP not initialised");
  return ctx->mlp->forward_host(*ctx, X, n, Y);
}

extern "C" fv3d_status fv3d_mlp_grad(fv3d_ctx* handle, const float* X, const float* T, int n, double* loss,
                                     float* grad) {
  if (handle == nullptr || X == nullptr || T == nullptr || loss == nullptr || grad == nullptr || n <= 0)
    return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mlp || !ctx->mlp->ready) return ctx->fail(FV3D_ERR_STATE, "MLP not initialised");
  return ctx->mlp->grad_host(*ctx, X, T, n, loss, grad);
}

extern "C" fv3d_status fv3d_mlp_harvest(fv3d_ctx* handle, int per_step, int max_samples) {
  if (handle == nullptr || per_step < 0 || max_samples < 0) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  Mlp* m = mlp_of(ctx);
  m->harvest_per_step = per_step;
  if (max_samples != m->max_samples) {
    m->max_samples = max_samples;
    m->n_samples = 0;
    m->X.release();
    m->T.release();
    m->Wt.release();
  }
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_mlp_dataset(const fv3d_ctx* handle, int* n_samples) {
  if (handle == nullptr || n_samples == nullptr) return FV3D_ERR_INVALID_ARG;
  const Ctx* ctx = reinterpret_cast<const Ctx*>(handle);
  *n_samples = ctx->mlp ? ctx->mlp->n_samples : 0;
  return FV3D_OK;
}

extern "C" fv3d_status fv3d_mlp_train(fv3d_ctx* handle, const fv3d_mlp_train_opts* opts,
                                      fv3d_mlp_train_stats* stats) {
  if (handle == nullptr || opts == nullptr || opts->epochs < 0 || !(opts->lr > 0.0)) return FV3D_ERR_INVALID_ARG;
  Ctx* ctx = reinterpret_cast<Ctx*>(handle);
  if (!ctx->mlp || !ctx->mlp->ready) return ctx->fail(FV3D_ERR_STATE, "MLP not initialised");
  return ctx->mlp->train(*ctx, *opts, stats);
}
