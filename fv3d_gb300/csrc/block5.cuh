// Dense 5x5 block arithmetic shared by the implicit solve's block
// preconditioners.
#pragma once

namespace fv3d {

// 5x5 inverse (row-major, FP64 Gauss-Jordan with partial pivoting); false
// when singular.  Fully unrolled, the row exchange as selects over the
// candidate rows: the working matrix and the caller's block stay in
// registers (a conditional exchange put both in local memory)
__device__ __forceinline__ bool invert5(const double* B, double* X) {
  double M[5][10];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      M[i][j] = B[i * 5 + j];
      M[i][5 + j] = (i == j) ? 1.0 : 0.0;
    }
#pragma unroll
  for (int col = 0; col < 5; ++col) {
    int piv = col;
    double best = fabs(M[col][col]);
#pragma unroll
    for (int i = col + 1; i < 5; ++i)
      if (fabs(M[i][col]) > best) {
        best = fabs(M[i][col]);
        piv = i;
      }
    if (!(best > 1e-300)) return false;
#pragma unroll
    for (int i = col + 1; i < 5; ++i) {
      const bool sw = (piv == i);
#pragma unroll
      for (int j = 0; j < 10; ++j) {
        const double a = M[col][j], b = M[i][j];
        M[col][j] = sw ? b : a;
        M[i][j] = sw ? a : b;
      }
    }
    const double ip = 1.0 / M[col][col];
#pragma unroll
    for (int j = 0; j < 10; ++j) M[col][j] *= ip;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      if (i == col) continue;
      const double fct = M[i][col];
#pragma unroll
      for (int j = 0; j < 10; ++j) M[i][j] -= fct * M[col][j];
    }
  }
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) X[i * 5 + j] = M[i][5 + j];
  return true;
}

}  // namespace fv3d
