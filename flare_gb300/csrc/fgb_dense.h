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
}  // namespace dense
}  // namespace fgb
