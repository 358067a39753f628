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
#include <cstdint>
#include <utility>
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

// At (M x (nl + M), row-major) = [Kuf diag(sqrt(noise)) | L]: the
// transpose of the reference's A = [sqrt(noise) Kuf^T ; L^T]
// (sparse_gp.cpp:621-630), built without a transpose (Kuf is M x nl
// row-major, L lower row-major); b = [sqrt(noise) y ; 0].
__global__ void k_build_At(int M, int nl, const double *__restrict__ Kuf,
                           const double *__restrict__ noise,
                           const double *__restrict__ y,
                           const double *__restrict__ L, double *__restrict__ At,
                           double *__restrict__ b) {
  const long long n = (long long)nl + M;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)M * n) return;
  const int c = (int)(idx / n);
  const long long r = idx - (long long)c * n;
  At[idx] = r < nl ? sqrt(noise[r]) * Kuf[(long long)c * nl + r]
                   : L[(long long)c * M + (r - nl)];
  if (c == 0) b[r] = r < nl ? sqrt(noise[r]) * y[r] : 0.0;
}

// Per-block partial sums of squares (fixed order), then one block adds them.
__global__ void k_sumsq_part(long long n, const double *__restrict__ x,
                             double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < n;
       i += (long long)gridDim.x * 256)
    s += x[i] * x[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// A += s I (M x M, row-major) with s = kShift * part sum (the shifted
// Cholesky QR's shift from the squared Frobenius norm).
__global__ void k_add_shift(int M, double *__restrict__ A, long long lda,
                            const double *__restrict__ part, int nparts,
                            double factor) {
  __shared__ double tot;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < nparts; k++) t += part[k];
    tot = t * factor;
  }
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M;
       i += gridDim.x * blockDim.x)
    A[(long long)i * lda + i] += tot;
}

// y[j] = sum_r Q[r][j] b[r] for Q (n x M, row-major): 32 columns per block
// (lane = column), 8 row groups, fixed-order sums.
__global__ void k_gemv_t(long long n, int M, const double *__restrict__ Q,
                         const double *__restrict__ b, double *__restrict__ y) {
  __shared__ double red[8][33];
  const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (j < M)
    for (long long r = g; r < n; r += 8) s += Q[r * M + j] * b[r];
  red[g][lane] = s;
  __syncthreads();
  if (g == 0 && j < M) {
    double t = 0.0;
    for (int k = 0; k < 8; k++) t += red[k][lane];
    y[j] = t;
  }
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

// The factor R (returned as R_inv = R^-1, row-major upper) and Q^T b of the
// Householder QR in update_matrices_QR (sparse_gp.cpp:621-640), by shifted
// Cholesky QR with two refinement passes: pass 0 factors A^T A + s I (s =
// 11 (n M + M (M + 1)) u |A|_F^2), Q0 = A R0^-1; passes 1 and 2 factor
// Q^T Q without shift, Q <- Q R_k^-1; R = R2 R1 R0 and Q^T b = Q2^T b.
// That is backward stable like Householder QR for condition numbers below
// 1/u; A here = [sqrt(noise) Kuf^T; L^T] has sigma_min >= sqrt(jitter).
// Every O(n M^2) product is an FP64-level tensor-core product.  R agrees
// with a Householder R up to the signs of its rows, so alpha = R^-1 Q^T b
// and Sigma = R^-1 R^-T are the same quantities.  At (M x n, row-major) is
// read; b has n entries.
int cholqr_solve(int M, long long n, double *At, const double *b,
                 double *R_inv, double *Qtb, cudaStream_t st) {
  Work w;
  DevBuf G, X[3], A0, Q, Qt, part, P;
  int rc;
  const size_t MM = (size_t)M * M, nM = (size_t)n * M;
  if ((rc = w.err.ensure(sizeof(int))) || (rc = G.ensure(sizeof(double) * MM)) ||
      (rc = X[0].ensure(sizeof(double) * MM)) ||
      (rc = X[1].ensure(sizeof(double) * MM)) ||
      (rc = X[2].ensure(sizeof(double) * MM)) ||
      (rc = P.ensure(sizeof(double) * MM)) ||
      (rc = A0.ensure(sizeof(double) * nM)) ||
      (rc = Q.ensure(sizeof(double) * nM)) ||
      (rc = part.ensure(sizeof(double) * 1024)))
    return rc;
  FGB_CUDA(cudaMemsetAsync(w.err.p, 0, sizeof(int), st));
  if (n > (long long)INT32_MAX) {
    set_error("update_matrices_QR: %lld rows exceed the product kernels' "
              "limit", n);
    return FGB_EINVAL;
  }
  const int ni = (int)n;
  const double u = std::ldexp(1.0, -53);
  const double shift = 11.0 * ((double)n * M + (double)M * (M + 1)) * u;
  // the rows of A (n x M) for the products Q = A R^-1
  if ((rc = transpose(M, ni, At, n, A0.as<double>(), M, st))) return rc;
  const double *Qprev = A0.as<double>();
  const double *Tprev = At;   // Q_prev^T (M x n)
  for (int pass = 0; pass < 3; pass++) {
    if ((rc = gemm_nt(M, M, ni, Tprev, n, Tprev, n, G.as<double>(), M, 1.0,
                      0.0, w, st)))
      return rc;
    if (pass == 0) {
      const int nparts = 1024;
      k_sumsq_part<<<nparts, 256, 0, st>>>((long long)M * n, At,
                                          part.as<double>());
      FGB_LAUNCH_CHECK("k_sumsq_part");
      k_add_shift<<<ceil_div(M, 256), 256, 0, st>>>(
          M, G.as<double>(), M, part.as<double>(), nparts, shift);
      FGB_LAUNCH_CHECK("k_add_shift");
    }
    if ((rc = cholesky(M, G.as<double>(), M, st)) ||
        (rc = trtri_lower(M, G.as<double>(), M, X[pass].as<double>(), M, st)))
      return rc;
    // Q_pass = Q_prev R_pass^-1 = Q_prev X_pass^T (X = L^-1, R = L^T)
    if ((rc = gemm_nt(ni, M, M, Qprev, M, X[pass].as<double>(), M,
                      Q.as<double>(), M, 1.0, 0.0, w, st)))
      return rc;
    if (pass < 2) {
      // Q becomes the next pass's input (A0's storage is free after pass 0)
      std::swap(Q.p, A0.p);
      std::swap(Q.bytes, A0.bytes);
      Qprev = A0.as<double>();
      if ((rc = Qt.ensure(sizeof(double) * nM))) return rc;
      if ((rc = transpose(ni, M, Qprev, M, Qt.as<double>(), n, st))) return rc;
      Tprev = Qt.as<double>();
    }
  }
  // Q^T b with the final Q
  k_gemv_t<<<ceil_div(M, 32), 256, 0, st>>>(n, M, Q.as<double>(), b, Qtb);
  FGB_LAUNCH_CHECK("k_gemv_t");
  // R^-1 = R0^-1 R1^-1 R2^-1 = (X2 X1 X0)^T
  double *T1 = G.as<double>();
  if ((rc = transpose(M, M, X[1].as<double>(), M, T1, M, st)) ||
      (rc = gemm_nt(M, M, M, X[2].as<double>(), M, T1, M, P.as<double>(), M,
                    1.0, 0.0, w, st)) ||
      (rc = transpose(M, M, X[0].as<double>(), M, T1, M, st)) ||
      (rc = gemm_nt(M, M, M, P.as<double>(), M, T1, M, X[1].as<double>(), M,
                    1.0, 0.0, w, st)) ||
      (rc = transpose(M, M, X[1].as<double>(), M, R_inv, M, st)))
    return rc;
  return finish(w, st, "Cholesky QR");
}

int build_At(int M, int nl, const double *Kuf, const double *noise,
             const double *y, const double *L, double *At, double *b,
             cudaStream_t st) {
  const long long n = (long long)nl + M;
  k_build_At<<<ceil_div((long long)M * n, 256), 256, 0, st>>>(M, nl, Kuf, noise,
                                                             y, L, At, b);
  FGB_LAUNCH_CHECK("k_build_At");
  return FGB_OK;
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
