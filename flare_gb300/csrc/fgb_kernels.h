// Launchers shared between libflaregb translation units.
#pragma once
#include "fgb_internal.h"

namespace fgb {

size_t b2_forward_smem(const B2Params &p, bool regA = false);
// dfloat: compute in double-float (mixed-precision path) instead of FP64;
// d_rowmax (optional): each row's largest |B2| as written
// d_A32 (double-float forward only): A written in FP32 instead of d_A, for
// the FP32 adjoint
int launch_b2_forward(const B2Params &p, const fgb_nlist_s *nl,
                      const int *d_species, double *d_A, double *d_B2,
                      double *d_norms, cudaStream_t st, bool dfloat = false,
                      double *d_rowmax = nullptr, float *d_A32 = nullptr);
// d_gB2: dE/dB2 rows [N, n_d] and d_pair_grad: pair gradients [P], both in
// the compute type (float / float3 when fp32, else double / double3)
// d_A32 (fp32 only): A read in FP32 instead of from d_A
int launch_b2_adjoint(const B2Params &p, const fgb_nlist_s *nl,
                      const int *d_species, const double *d_A,
                      const void *d_gB2, void *d_pair_grad,
                      cudaStream_t st, bool fp32 = false,
                      const float *d_A32 = nullptr);
// d_pair_grad as the adjoint wrote it (fp32: float3)
int launch_forces(const fgb_nlist_s *nl, const void *d_pair_grad, bool fp32,
                  double *d_forces, double *d_virial, cudaStream_t st);
int launch_struct_reduce(int n_struc, const int *d_atom_off,
                         const double *d_volume, const double *d_e_atom,
                         const double *d_virial, double *d_energy,
                         double *d_stress, cudaStream_t st);

// Stored forward-mode gradients (the reference's algorithm).
int launch_b2_dervs(const B2Params &p, const fgb_nlist_s *nl,
                    const int *d_species, const double *d_A, const double *d_B2,
                    double *d_dB2, double *d_force_dots, cudaStream_t st);

// FP64 row energies E = K alpha and the local-variance finish
// var = k_self - sum(part) (predict.cu).
int launch_row_energy(int Mr, int Ms, const double *Kmat, const double *alpha,
                      const int *perm, double *e_rows, double *e_atom,
                      cudaStream_t st);
int launch_variance_final(int Mr, int ntiles, const double *part,
                          const int *perm, const double *norms, double sig2,
                          double xi, double *var, cudaStream_t st);

// FP64 triangular variance GEMM (Z = K L^T, row sums of Z^2 per 64-column
// tile), ntiles = ceil(R / 64).
int launch_variance_fp64(int Mr, int R, int Ms, const double *Kmat,
                         const double *Lp, double *part, int ntiles,
                         cudaStream_t st);

// Validate coded species in [0, n_species); returns FGB_EINVAL otherwise.
int check_species(const int *d_species, int n, int n_species, DevBuf &flag,
                  cudaStream_t st);

}  // namespace fgb
