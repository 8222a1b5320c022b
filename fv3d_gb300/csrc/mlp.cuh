// Per-cell MLP used as a learned preconditioner inside FGMRES.
//
//   x (36) -> 64 -> 64 -> 64 -> 5,  GELU (tanh form) on the hidden layers
//   inputs:  25 entries of the cell's 5x5 block (scaled by 1/||D||_F),
//            6 face features A_k / V^(2/3) (face slots in reference face order),
//            5 components of the cell's vector (scaled to unit length)
//   output:  the preconditioned vector of the cell, in units of |v| / ||D||_F
// BF16 weights and activations as tensor-core operands, FP32 accumulation
// (tcgen05 with TMEM accumulators for inference, mlp_tc.cu; mma.sync
// m16n8k16 for training and as the alternative inference path), FP32 master
// weights and Adam state.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace fv3d {

constexpr int MLP_IN = 36, MLP_INP = 48, MLP_H = 64, MLP_OUT = 5, MLP_OUTP = 8;
// packed FP32 parameter offsets
constexpr int MLP_W0 = 0;
constexpr int MLP_B0 = MLP_W0 + MLP_H * MLP_IN;     // 2304
constexpr int MLP_W1 = MLP_B0 + MLP_H;               // 2368
constexpr int MLP_B1 = MLP_W1 + MLP_H * MLP_H;       // 6464
constexpr int MLP_W2 = MLP_B1 + MLP_H;               // 6528
constexpr int MLP_B2 = MLP_W2 + MLP_H * MLP_H;       // 10624
constexpr int MLP_W3 = MLP_B2 + MLP_H;               // 10688
constexpr int MLP_B3 = MLP_W3 + MLP_OUT * MLP_H;     // 11008
constexpr int MLP_NPARAM = MLP_B3 + MLP_OUT;         // 11013
constexpr int MLP_TILE = 64;                         // samples per CTA (4 warps x 16)
constexpr int MLP_FEAT = 32;                         // per-cell feature record (floats)

// GELU in its tanh form, 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))),
// with the hardware tanh approximation (one MUFU operation; relative error
// about 2^-11, below the BF16 rounding the activations then take)
__device__ __forceinline__ float mlp_tanh(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float mlp_gelu(float x) {
  const float t = mlp_tanh(0.7978845608028654f * fmaf(0.044715f * x, x * x, x));
  return 0.5f * x * (1.f + t);
}
// its derivative: 0.5 (1 + t) + 0.5 x (1 - t^2) sqrt(2/pi) (1 + 3 0.044715 x^2)
__device__ __forceinline__ float mlp_gelu_d(float x) {
  const float t = mlp_tanh(0.7978845608028654f * fmaf(0.044715f * x, x * x, x));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * 0.7978845608028654f * fmaf(0.134145f * x, x, 1.f);
}

}  // namespace fv3d
