// FP64 dense linear algebra of the sparse-GP solve (dense.cu).
#pragma once
#include <cuda_runtime.h>

namespace fgb {
namespace dense {
// Lower Cholesky factor of a symmetric M x M row-major matrix, in place
// (strict upper part zeroed); FGB_EINVAL if not positive definite.
int cholesky(int M, double *A, long long lda, cudaStream_t st);
// X = L^-1 for a lower-triangular M x M row-major L (strict upper of X
// zeroed); L and X distinct.
int trtri_lower(int M, const double *L, long long ldl, double *X,
                long long ldx, cudaStream_t st);
// C = A^T A (transpose_first) or A A^T for a square M x M matrix.
int sym_product(int M, const double *A, bool transpose_first, double *C,
                cudaStream_t st);
// R_inv (row-major upper) and Q^T b[:M] of the QR of A (n x M) given as
// At = A^T (M x n, row-major), by shifted Cholesky QR.
int cholqr_solve(int M, long long n, double *At, const double *b,
                 double *R_inv, double *Qtb, cudaStream_t st);
// At = [Kuf diag(sqrt(noise)) | L] (M x (nl + M)) and b = [sqrt(noise) y; 0].
int build_At(int M, int nl, const double *Kuf, const double *noise,
             const double *y, const double *L, double *At, double *b,
             cudaStream_t st);
}  // namespace dense
}  // namespace fgb
