// FP64 dense linear algebra of the sparse-GP solve (SparseGP::
// update_matrices_QR, sparse_gp.cpp:607-641): the Cholesky factor of
// Kuu + jitter, lower-triangular inverses (L_inv, and R_inv through R^T),
// and the symmetric products Kuu^-1 = L_inv^T L_inv and Sigma = R_inv
// R_inv^T.
//
// Matrices are row-major.  The O(M^3) work runs as FP64-level products on
// the tensor cores (ozaki.cu: 9 exact BF16 slices, exact integer sums, one
// rounding; about 35x this GPU's FP64 DGEMM rate); the O(M nb^2) work on
// diagonal blocks of nb = 128 runs in shared memory, one CTA per block:
//   Cholesky, right-looking by block columns: factor the diagonal block
//     and invert it (k_potrf_block), L21 = A21 L11^-T as a product with
//     that inverse, then the trailing update A22 -= L21 L21^T;
//   lower-triangular inverse, recursive: X = [X11 0; X21 X22] with X11,
//     X22 the inverses of the diagonal halves (leaves of nb inverted by
//     k_trtri_block, all at once) and X21 = -X22 (L21 X11).
// Operation orders differ from Eigen's (the reference's LLT and triangular
// solves), so results agree with it to FP64 rounding, not bit for bit.
#include <cmath>
#include <vector>

#include "fgb_dense.h"
#include "fgb_internal.h"
#include "fgb_ozaki.h"

namespace fgb {
namespace dense {
namespace {

constexpr int kNB = 128;          // diagonal block
constexpr int kBlockThreads = 512;

// Cholesky of one kb x kb diagonal block (kb <= kNB) in shared memory,
// lower factor written back over A (upper part zeroed), and its inverse
// into X (ld kb; thread j owns column j, forward substitution).  A leading
// minor that is not positive sets *info = first bad row + 1 (global index
// base + j + 1) and the block stops.
__global__ void __launch_bounds__(kBlockThreads)
k_potrf_block(int kb, double *__restrict__ A, long long lda,
              double *__restrict__ X, int base, int *__restrict__ info) {
  extern __shared__ double sh[];   // kb x kb
  __shared__ int bad;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  for (int idx = tid; idx < kb * kb; idx += nt) {
    const int i = idx / kb, j = idx - i * kb;
    sh[idx] = j <= i ? A[(long long)i * lda + j] : 0.0;
  }
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < kb; j++) {
    const double d = sh[j * kb + j];
    if (tid == 0 && !(d > 0.0)) {
      bad = 1;
      atomicCAS(info, 0, base + j + 1);
    }
    __syncthreads();
    if (bad) break;
    const double ljj = sqrt(d);
    for (int i = j + 1 + tid; i < kb; i += nt) sh[i * kb + j] /= ljj;
    __syncthreads();
    if (tid == 0) sh[j * kb + j] = ljj;
    for (int i = j + 1 + warp; i < kb; i += nw) {
      const double lij = sh[i * kb + j];
      for (int k = j + 1 + lane; k <= i; k += 32)
        sh[i * kb + k] -= lij * sh[k * kb + j];
    }
    __syncthreads();
  }
  if (bad) return;
  for (int idx = tid; idx < kb * kb; idx += nt) {
    const int i = idx / kb, j = idx - i * kb;
    A[(long long)i * lda + j] = j <= i ? sh[idx] : 0.0;
  }
  // X = L^-1: column j by forward substitution
  for (int j = tid; j < kb; j += nt) {
    for (int i = 0; i < j; i++) X[(long long)i * kb + j] = 0.0;
    X[(long long)j * kb + j] = 1.0 / sh[j * kb + j];
    for (int i = j + 1; i < kb; i++) {
      double s = 0.0;
      for (int k = j; k < i; k++) s += sh[i * kb + k] * X[(long long)k * kb + j];
      X[(long long)i * kb + j] = -s / sh[i * kb + i];
    }
  }
}

// Inverses of the diagonal blocks of a lower-triangular M x M matrix L,
// one CTA per block of kNB (the last may be smaller), written into the same
// positions of X (the rest of X is left alone).
__global__ void __launch_bounds__(kBlockThreads)
k_trtri_block(int M, const double *__restrict__ L, long long ldl,
              double *__restrict__ X, long long ldx) {
  extern __shared__ double sh[];
  const int b0 = blockIdx.x * kNB;
  const int kb = min(kNB, M - b0);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int idx = tid; idx < kb * kb; idx += nt) {
    const int i = idx / kb, j = idx - i * kb;
    sh[idx] = j <= i ? L[(long long)(b0 + i) * ldl + b0 + j] : 0.0;
  }
  __syncthreads();
  double *Xb = X + (long long)b0 * ldx + b0;
  for (int j = tid; j < kb; j += nt) {
    for (int i = 0; i < j; i++) Xb[(long long)i * ldx + j] = 0.0;
    Xb[(long long)j * ldx + j] = 1.0 / sh[j * kb + j];
    for (int i = j + 1; i < kb; i++) {
      double s = 0.0;
      for (int k = j; k < i; k++) s += sh[i * kb + k] * Xb[(long long)k * ldx + j];
      Xb[(long long)i * ldx + j] = -s / sh[i * kb + i];
    }
  }
}

// out (cols x rows, ld ldo) = in^T (in: rows x cols, ld ldi), 32 x 32 tiles.
__global__ void k_transpose_tile(int rows, int cols, const double *__restrict__ in,
                                 long long ldi, double *__restrict__ out,
                                 long long ldo) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[k][threadIdx.x] = in[(long long)r * ldi + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(long long)c * ldo + r] = t[threadIdx.x][k];
  }
}

__global__ void k_zero_strict_upper(int M, double *__restrict__ A, long long lda) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)M * M) return;
  const int i = (int)(idx / M), j = (int)(idx - (long long)i * M);
  if (j > i) A[(long long)i * lda + j] = 0.0;
}

int transpose(int rows, int cols, const double *in, long long ldi, double *out,
              long long ldo, cudaStream_t st) {
  if (rows == 0 || cols == 0) return FGB_OK;
  dim3 g(ceil_div(cols, 32), ceil_div(rows, 32)), b(32, 8);
  k_transpose_tile<<<g, b, 0, st>>>(rows, cols, in, ldi, out, ldo);
  FGB_LAUNCH_CHECK("k_transpose_tile");
  return FGB_OK;
}

// Scratch of one factorisation: slices of the two operands and the
// tensor-core GEMM's time-out flag.
struct Work {
  oz::Sliced A, B;
  DevBuf err, t1, t2;
};

// C (m x n, ldc) = a A B^T + b C with A (m x k, lda) and B (n x k, ldb) at
// FP64 level on the tensor cores.
int gemm_nt(int m, int n, int k, const double *A, long long lda,
            const double *B, long long ldb, double *C, long long ldc,
            double a, double b, Work &w, cudaStream_t st) {
  if (m == 0 || n == 0) return FGB_OK;
  int rc;
  if ((rc = oz::slice({m, k, oz::kTM, A, lda, nullptr, nullptr}, w.A, st)) ||
      (rc = oz::slice({n, k, oz::kTN, B, ldb, nullptr, nullptr}, w.B, st)))
    return rc;
  return oz::gemm_axpby(w.A, w.B, C, ldc, a, b, w.err.as<int>(), st);
}

int finish(Work &w, cudaStream_t st, const char *what) {
  int h = 0;
  FGB_CUDA(cudaMemcpyAsync(&h, w.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error("%s: a bounded device wait ran out", what);
    return FGB_ETIMEOUT;
  }
  return FGB_OK;
}

int smem_for(int kb) {
  return (int)(sizeof(double) * (size_t)kb * kb);
}

// X (lower part, row-major, ld ldx) = L^-1 for rows/cols [lo, lo + n),
// given the diagonal blocks already inverted in place.
int trtri_rec(int lo, int n, const double *L, long long ldl, double *X,
              long long ldx, Work &w, cudaStream_t st) {
  if (n <= kNB) return FGB_OK;
  const int nblk = ceil_div(n, kNB);
  const int h = kNB * ((nblk + 1) / 2);
  const int n2 = n - h;
  int rc;
  if ((rc = trtri_rec(lo, h, L, ldl, X, ldx, w, st)) ||
      (rc = trtri_rec(lo + h, n2, L, ldl, X, ldx, w, st)))
    return rc;
  // T = L21 X11 (n2 x h): B operand X11^T
  if ((rc = w.t1.ensure(sizeof(double) * (size_t)h * h)) ||
      (rc = w.t2.ensure(sizeof(double) * (size_t)n2 * h)))
    return rc;
  const double *L21 = L + (long long)(lo + h) * ldl + lo;
  const double *X11 = X + (long long)lo * ldx + lo;
  const double *X22 = X + (long long)(lo + h) * ldx + lo + h;
  double *X21 = X + (long long)(lo + h) * ldx + lo;
  if ((rc = transpose(h, h, X11, ldx, w.t1.as<double>(), h, st))) return rc;
  // T into X21's place (n2 x h), then its transpose into t2 (h x n2)
  if ((rc = gemm_nt(n2, h, h, L21, ldl, w.t1.as<double>(), h, X21, ldx, 1.0,
                    0.0, w, st)))
    return rc;
  if ((rc = transpose(n2, h, X21, ldx, w.t2.as<double>(), n2, st))) return rc;
  // X21 = -X22 T
  return gemm_nt(n2, h, n2, X22, ldx, w.t2.as<double>(), n2, X21, ldx, -1.0,
                 0.0, w, st);
}

}  // namespace

// Lower Cholesky factor of the symmetric M x M matrix A (row-major; the
// lower triangle is read), in place (strict upper part zeroed).
int cholesky(int M, double *A, long long lda, cudaStream_t st) {
  if (M == 0) return FGB_OK;
  Work w;
  DevBuf info, Tinv;
  int rc;
  if ((rc = w.err.ensure(sizeof(int))) || (rc = info.ensure(sizeof(int))) ||
      (rc = Tinv.ensure(sizeof(double) * kNB * kNB)))
    return rc;
  FGB_CUDA(cudaMemsetAsync(w.err.p, 0, sizeof(int), st));
  FGB_CUDA(cudaMemsetAsync(info.p, 0, sizeof(int), st));
  FGB_CUDA(cudaFuncSetAttribute(k_potrf_block,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                smem_for(kNB)));
  for (int k0 = 0; k0 < M; k0 += kNB) {
    const int kb = std::min(kNB, M - k0);
    double *A11 = A + (long long)k0 * lda + k0;
    k_potrf_block<<<1, kBlockThreads, smem_for(kb), st>>>(
        kb, A11, lda, Tinv.as<double>(), k0, info.as<int>());
    FGB_LAUNCH_CHECK("k_potrf_block");
    const int r = M - k0 - kb;
    if (r == 0) break;
    double *A21 = A + (long long)(k0 + kb) * lda + k0;
    double *A22 = A + (long long)(k0 + kb) * lda + k0 + kb;
    // L21 = A21 L11^-T, in place (the product reads slices of A21)
    if ((rc = gemm_nt(r, kb, kb, A21, lda, Tinv.as<double>(), kb, A21, lda,
                      1.0, 0.0, w, st)))
      return rc;
    // A22 -= L21 L21^T (the whole square; the strict upper part is zeroed
    // at the end)
    if ((rc = gemm_nt(r, r, kb, A21, lda, A21, lda, A22, lda, -1.0, 1.0, w,
                      st)))
      return rc;
  }
  k_zero_strict_upper<<<ceil_div((long long)M * M, 256), 256, 0, st>>>(M, A,
                                                                       lda);
  FGB_LAUNCH_CHECK("k_zero_strict_upper");
  int hinfo = 0;
  FGB_CUDA(cudaMemcpyAsync(&hinfo, info.p, sizeof(int), cudaMemcpyDeviceToHost,
                           st));
  if ((rc = finish(w, st, "Cholesky"))) return rc;
  if (hinfo) {
    set_error("Cholesky of Kuu + jitter failed (leading minor %d not "
              "positive definite)", hinfo);
    return FGB_EINVAL;
  }
  return FGB_OK;
}

// X = L^-1 for a lower-triangular M x M matrix L (row-major; X's strict
// upper part zeroed).
int trtri_lower(int M, const double *L, long long ldl, double *X,
                long long ldx, cudaStream_t st) {
  if (M == 0) return FGB_OK;
  Work w;
  int rc;
  if ((rc = w.err.ensure(sizeof(int)))) return rc;
  FGB_CUDA(cudaMemsetAsync(w.err.p, 0, sizeof(int), st));
  k_zero_strict_upper<<<ceil_div((long long)M * M, 256), 256, 0, st>>>(M, X,
                                                                       ldx);
  FGB_LAUNCH_CHECK("k_zero_strict_upper");
  FGB_CUDA(cudaFuncSetAttribute(k_trtri_block,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                smem_for(kNB)));
  k_trtri_block<<<ceil_div(M, kNB), kBlockThreads, smem_for(std::min(M, kNB)),
                  st>>>(M, L, ldl, X, ldx);
  FGB_LAUNCH_CHECK("k_trtri_block");
  if ((rc = trtri_rec(0, M, L, ldl, X, ldx, w, st))) return rc;
  return finish(w, st, "triangular inverse");
}

// C = A^T A (transpose_first) or A A^T for a square M x M matrix A, FP64
// level on the tensor cores; C is symmetric (both triangles written).
int sym_product(int M, const double *A, bool transpose_first, double *C,
                cudaStream_t st) {
  if (M == 0) return FGB_OK;
  Work w;
  DevBuf At;
  int rc;
  if ((rc = w.err.ensure(sizeof(int)))) return rc;
  FGB_CUDA(cudaMemsetAsync(w.err.p, 0, sizeof(int), st));
  const double *op = A;
  if (transpose_first) {
    if ((rc = At.ensure(sizeof(double) * (size_t)M * M))) return rc;
    if ((rc = transpose(M, M, A, M, At.as<double>(), M, st))) return rc;
    op = At.as<double>();
  }
  if ((rc = gemm_nt(M, M, M, op, M, op, M, C, M, 1.0, 0.0, w, st))) return rc;
  return finish(w, st, "symmetric product");
}

}  // namespace dense
}  // namespace fgb

using namespace fgb;

extern "C" int fgb_cholesky(int M, double *d_A, void *stream) {
  if (M < 0 || (M > 0 && !d_A)) {
    set_error("fgb_cholesky: invalid arguments");
    return FGB_EINVAL;
  }
  return dense::cholesky(M, d_A, M, (cudaStream_t)stream);
}

extern "C" int fgb_trtri_lower(int M, const double *d_L, double *d_X,
                               void *stream) {
  if (M < 0 || (M > 0 && (!d_L || !d_X)) || d_L == d_X) {
    set_error("fgb_trtri_lower: invalid arguments (distinct L and X)");
    return FGB_EINVAL;
  }
  return dense::trtri_lower(M, d_L, M, d_X, M, (cudaStream_t)stream);
}

extern "C" int fgb_solve_products(int M, const double *d_L_inv,
                                  const double *d_R_inv, double *d_Kuu_inverse,
                                  double *d_Sigma, void *stream) {
  if (M < 0 || (d_Kuu_inverse && !d_L_inv) || (d_Sigma && !d_R_inv)) {
    set_error("fgb_solve_products: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc;
  if (d_Kuu_inverse &&
      (rc = dense::sym_product(M, d_L_inv, true, d_Kuu_inverse, st)))
    return rc;
  if (d_Sigma && (rc = dense::sym_product(M, d_R_inv, false, d_Sigma, st)))
    return rc;
  return FGB_OK;
}
