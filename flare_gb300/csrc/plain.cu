// Plain FP64 form: the reference's algorithm on the GPU (stored
// forward-mode descriptor gradients, envs_struc GEMM + scatter), envs_envs,
// and the FP64 QR solve.
#include "fgb_internal.h"
#include "fgb_kernels.h"
#include "fgb_model.h"
#include "fgb_gemm64.cuh"

namespace fgb {
namespace {
using namespace gemm64;

// envs_envs block: K = sig2 (D1 D2^T / (n1 n2))^power
__global__ void __launch_bounds__(GT)
k_envs_envs(int M, int N, int K, const double *__restrict__ D1,
            const double *__restrict__ n1, const double *__restrict__ D2,
            const double *__restrict__ n2, double sig2, double power,
            double *__restrict__ out) {
  const int m0 = blockIdx.y * BM, nn0 = blockIdx.x * BN;
  double acc[4][4];
  gemm_mainloop<true>(acc, m0, nn0, M, N, K, D1, K, nullptr, D2, K);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int m = m0 + ty + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n = nn0 + tx + 16 * j;
      if (n >= N) continue;
      double a = n1[m], b = n2[n];
      double v = 0.0;
      if (a >= kEmptyThresh && b >= kEmptyThresh)
        v = sig2 * powx(acc[i][j] / (a * b), power);
      out[(long long)m * N + n] = v;
    }
  }
}

}  // namespace
}  // namespace fgb

using namespace fgb;

extern "C" int fgb_envs_envs(const double *d_desc1, const double *d_norm1,
                             int n1, const double *d_desc2,
                             const double *d_norm2, int n2, int n_desc,
                             double sig2, double power, double *d_kern,
                             void *stream) {
  if (n1 < 0 || n2 < 0 || n_desc <= 0 || (n1 && n2 && !d_kern)) {
    set_error("fgb_envs_envs: invalid arguments");
    return FGB_EINVAL;
  }
  if (n1 == 0 || n2 == 0) return FGB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  dim3 g(ceil_div(n2, BN), ceil_div(n1, BM));
  k_envs_envs<<<g, GT, 0, st>>>(n1, n2, n_desc, d_desc1, d_norm1, d_desc2,
                                d_norm2, sig2, power, d_kern);
  FGB_LAUNCH_CHECK("k_envs_envs");
  return FGB_OK;
}

extern "C" int fgb_b2_forward_dervs(fgb_b2_t, fgb_nlist_t, const int *,
                                    double *, double *, double *, double *,
                                    void *) {
  set_error("fgb_b2_forward_dervs: not built yet");
  return FGB_ENOTSUP;
}

extern "C" int fgb_envs_struc(fgb_model_t, fgb_nlist_t, const int *, double *,
                              void *) {
  set_error("fgb_envs_struc: not built yet");
  return FGB_ENOTSUP;
}

extern "C" int fgb_predict_plain(fgb_model_t, fgb_nlist_t, const int *,
                                 double *, double *, void *) {
  set_error("fgb_predict_plain: not built yet");
  return FGB_ENOTSUP;
}

extern "C" int fgb_solve_qr(int, int, const double *, const double *,
                            const double *, const double *, double, double *,
                            double *, double *, void *) {
  set_error("fgb_solve_qr: not built yet");
  return FGB_ENOTSUP;
}
