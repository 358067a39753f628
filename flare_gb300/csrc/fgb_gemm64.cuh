// FP64 tiled GEMM core shared by the kernel, variance and plain-form
// kernels: 64x64 output tiles, 16-deep k slices staged in shared memory,
// 256 threads with a 4x4 register block each.
#pragma once
#include "fgb_common.cuh"

namespace fgb {
namespace gemm64 {

constexpr int BM = 64, BN = 64, BK = 16, GT = 256;

// acc[i][j] += sum_k A[row(m0+ty+16i)][k] * Bop[n0+tx+16j][k] for k < kmax.
// B_NT: Bop[n][k] = B[n*ldb + k]; else Bop[n][k] = B[k*ldb + n].
template <typename T, bool B_NT>
__device__ __forceinline__ void gemm_mainloop_t(T (&acc)[4][4], int m0, int n0,
                                                int M, int N, int kmax,
                                                const T *__restrict__ A,
                                                long long lda,
                                                const int *__restrict__ arow,
                                                const T *__restrict__ B,
                                                long long ldb) {
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < kmax; k0 += BK) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      int idx = tid + r * GT;
      int mm = idx / BK, kk = idx % BK;
      int m = m0 + mm, k = k0 + kk;
      T v = T(0);
      if (m < M && k < kmax) {
        long long row = arow ? (long long)arow[m] : (long long)m;
        v = A[row * lda + k];
      }
      As[kk][mm] = v;
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      int idx = tid + r * GT;
      int nn, kk;
      if (B_NT) { nn = idx / BK; kk = idx % BK; }
      else { kk = idx / BN; nn = idx % BN; }
      int n = n0 + nn, k = k0 + kk;
      T v = T(0);
      if (n < N && k < kmax)
        v = B_NT ? B[(long long)n * ldb + k] : B[(long long)k * ldb + n];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
}

// FP64 instantiation used by the kernel, variance and plain-form GEMMs.
template <bool B_NT>
__device__ __forceinline__ void gemm_mainloop(double (&acc)[4][4], int m0,
                                              int n0, int M, int N, int kmax,
                                              const double *__restrict__ A,
                                              long long lda,
                                              const int *__restrict__ arow,
                                              const double *__restrict__ B,
                                              long long ldb) {
  gemm_mainloop_t<double, B_NT>(acc, m0, n0, M, N, kmax, A, lda, arow, B, ldb);
}

__device__ __forceinline__ double powx(double c, double xi) {
  if (xi == 2.0) return c * c;
  if (xi == 1.0) return c;
  return pow(c, xi);
}

}  // namespace gemm64
}  // namespace fgb
