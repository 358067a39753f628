// Mapped evaluation: energies, forces and stresses from the mapping
// coefficients beta of a power-1 or power-2 sparse GP, the model a LAMMPS
// run loads from an lmp.flare file (the reference's pair style flare,
// lammps_plugins/pair_flare.cpp:68-175 with lammps_descriptor.cpp:250-326),
// and the mapped local variance of compute flare/std/atom
// (compute_flare_std_atom.cpp:179-193).
//
// Per atom i of species s with descriptor B2_i and n2 = |B2_i|^2:
//   power 2, normalised: E_i = B2_i . (beta_s B2_i) / n2,
//                        dE/dB2 = 2 (beta_s B2_i - E_i B2_i) / n2
//   power 1, normalised: E_i = beta_s . B2_i / |B2_i|,
//                        dE/dB2 = beta_s / |B2_i| - E_i B2_i / n2
//   (DotProduct kernels: the same without the norms), zero for n2 < 1e-8;
//   variance (power-1 map): v_i = 1 - |Q_s^T B2_i / |B2_i||^2.
// Y = B2 beta_s (and B2 Q_s) run on the tensor cores by exact slicing (FP64
// level); forces and stresses come from dE/dB2 through the reverse-mode B2
// adjoint, as in the prediction pipeline.
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "fgb_df.cuh"
#include "fgb_internal.h"
#include "fgb_kernels.h"
#include "fgb_model.h"
#include "fgb_ozaki.h"

namespace fgb {
namespace {

constexpr double kEmptySq = 1e-8;   // pair_flare.cpp:92 (on |B2|^2)

// n2 and B2 . v for one row: lane-strided sums, fixed shuffle tree.
__device__ __forceinline__ void row_dots(int lane, int nd,
                                         const double *__restrict__ b,
                                         const double *__restrict__ v,
                                         double &n2, double &dot) {
  n2 = 0.0;
  dot = 0.0;
  for (int k = lane; k < nd; k += 32) {
    n2 += b[k] * b[k];
    if (v) dot += b[k] * v[k];
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    n2 += __shfl_xor_sync(0xffffffffu, n2, off);
    dot += __shfl_xor_sync(0xffffffffu, dot, off);
  }
}

// dE/dB2 in the adjoint's compute type (FP32: the mantissa cut the FP32
// adjoint applies to FP64 inputs)
__device__ __forceinline__ void put_g(double *g, double x) { *g = x; }
__device__ __forceinline__ void put_g(float *g, double x) { *g = trunc_float(x); }

// Power 2: warp per row m (atom perm[m]); Y row m = beta_s B2_atom.
template <typename G>
__global__ void k_mapped_pow2(int Mr, int nd, const int *__restrict__ perm,
                              const double *__restrict__ B2,
                              const double *__restrict__ Y, int normalized,
                              double *__restrict__ e_atom,
                              G *__restrict__ gB2) {
  const int m = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (m >= Mr) return;
  const int atom = perm[m];
  const double *b = B2 + (long long)atom * nd;
  const double *y = Y + (long long)m * nd;
  double n2, dot;
  row_dots(lane, nd, b, y, n2, dot);
  G *g = gB2 + (long long)atom * nd;
  if (n2 < kEmptySq) {
    for (int k = lane; k < nd; k += 32) put_g(g + k, 0.0);
    if (lane == 0) e_atom[atom] = 0.0;
    return;
  }
  const double e = normalized ? dot / n2 : dot;
  for (int k = lane; k < nd; k += 32)
    put_g(g + k, normalized ? 2.0 * (y[k] - e * b[k]) / n2 : 2.0 * y[k]);
  if (lane == 0) e_atom[atom] = e;
}

// Power 1: warp per row; beta_s a vector.
template <typename G>
__global__ void k_mapped_pow1(int Mr, int nd, const int *__restrict__ perm,
                              const double *__restrict__ B2,
                              const double *__restrict__ beta, int normalized,
                              double *__restrict__ e_atom,
                              G *__restrict__ gB2) {
  const int m = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (m >= Mr) return;
  const int atom = perm[m];
  const double *b = B2 + (long long)atom * nd;
  double n2, dot;
  row_dots(lane, nd, b, beta, n2, dot);
  G *g = gB2 + (long long)atom * nd;
  if (n2 < kEmptySq) {
    for (int k = lane; k < nd; k += 32) put_g(g + k, 0.0);
    if (lane == 0) e_atom[atom] = 0.0;
    return;
  }
  const double nrm = sqrt(n2);
  const double e = normalized ? dot / nrm : dot;
  for (int k = lane; k < nd; k += 32)
    put_g(g + k, normalized ? beta[k] / nrm - e * b[k] / n2 : beta[k]);
  if (lane == 0) e_atom[atom] = e;
}

// Mapped variance: row m of Q = B2 Q_s (Q_s^T B2 for the atom);
// v = K_self - |Q|^2 / n2 (normalised: K_self = 1) or K_self = n2, |Q|^2.
__global__ void k_mapped_var(int Mr, int nd, const int *__restrict__ perm,
                             const double *__restrict__ B2,
                             const double *__restrict__ Q, int normalized,
                             double *__restrict__ var) {
  const int m = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (m >= Mr) return;
  const int atom = perm[m];
  const double *b = B2 + (long long)atom * nd;
  const double *q = Q + (long long)m * nd;
  double n2, qq;
  row_dots(lane, nd, b, nullptr, n2, qq);
  qq = 0.0;
  for (int k = lane; k < nd; k += 32) qq += q[k] * q[k];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    qq += __shfl_xor_sync(0xffffffffu, qq, off);
  if (lane != 0) return;
  if (n2 < kEmptySq) { var[atom] = 0.0; return; }
  var[atom] = normalized ? 1.0 - qq / n2 : n2 - qq;
}

}  // namespace
}  // namespace fgb

using namespace fgb;

struct fgb_mapped_s {
  B2Params b2;
  int power = 2;
  bool normalized = true;
  bool has_var = false;
  // mixed precision: double-float descriptor and FP32 adjoint unless the
  // largest |beta| exceeds the fold guard's threshold (then both FP64)
  bool adjoint_f64 = false;
  DevBuf beta;                                        // FP64, per species
  std::vector<std::unique_ptr<oz::Sliced>> ozBeta;    // power 2: beta_s rows
  std::vector<std::unique_ptr<oz::Sliced>> ozQ;       // variance map: Q_s^T rows
  fgb_nlist_s nl;
  fgb_workspace ws;
};

namespace {

// Slices of the rows of n_species n_d x n_d matrices (FP64 level, B tiles).
int slice_blocks(const double *d_mats, int S, int nd,
                 std::vector<std::unique_ptr<oz::Sliced>> &out,
                 cudaStream_t st) {
  out.clear();
  int rc;
  for (int s = 0; s < S; s++) {
    out.emplace_back(new oz::Sliced());
    if ((rc = oz::slice({nd, nd, oz::kTN, d_mats + (size_t)s * nd * nd, nd,
                         nullptr, nullptr},
                        *out[s], st)))
      return rc;
  }
  return FGB_OK;
}

}  // namespace

extern "C" int fgb_mapped_create(fgb_mapped_t *out, fgb_b2_t b2, int power,
                                 int normalized, const double *h_beta,
                                 const double *h_varmap) {
  if (!out || !b2 || !h_beta || (power != 1 && power != 2)) {
    set_error("fgb_mapped_create: invalid arguments (power is 1 or 2)");
    return FGB_EINVAL;
  }
  const int S = b2->p.n_species, nd = b2->p.n_d;
  const size_t per = power == 2 ? (size_t)nd * nd : (size_t)nd;
  for (size_t i = 0; i < per * S; i++)
    if (!std::isfinite(h_beta[i])) {
      set_error("fgb_mapped_create: non-finite mapping coefficients");
      return FGB_EINVAL;
    }
  auto *m = new fgb_mapped_s();
  double bmax = 0.0;
  for (size_t i = 0; i < per * S; i++) bmax = std::max(bmax, std::fabs(h_beta[i]));
  m->adjoint_f64 = bmax > kFoldMaxF32;
  m->b2 = b2->p;
  m->power = power;
  m->normalized = normalized != 0;
  int rc;
  cudaError_t e;
  if ((rc = m->beta.ensure(sizeof(double) * per * S))) { delete m; return rc; }
  if ((e = cudaMemcpy(m->beta.p, h_beta, sizeof(double) * per * S,
                      cudaMemcpyHostToDevice)) != cudaSuccess) {
    delete m;
    return cuda_status(e, "fgb_mapped_create");
  }
  if (power == 2 && (rc = slice_blocks(m->beta.as<double>(), S, nd,
                                       m->ozBeta, nullptr))) {
    delete m;
    return rc;
  }
  if (h_varmap) {
    // Q_s is stored row-major n_d x n_d; the B operand rows are Q_s^T rows
    std::vector<double> qt((size_t)S * nd * nd);
    for (int s = 0; s < S; s++)
      for (int i = 0; i < nd; i++)
        for (int j = 0; j < nd; j++)
          qt[((size_t)s * nd + j) * nd + i] = h_varmap[((size_t)s * nd + i) * nd + j];
    DevBuf dq;
    if ((rc = dq.ensure(sizeof(double) * qt.size())) ||
        (e = cudaMemcpy(dq.p, qt.data(), sizeof(double) * qt.size(),
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
      delete m;
      return rc ? rc : cuda_status(e, "fgb_mapped_create");
    }
    if ((rc = slice_blocks(dq.as<double>(), S, nd, m->ozQ, nullptr))) {
      delete m;
      return rc;
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) {
      delete m;
      return cuda_status(e, "fgb_mapped_create");
    }
    m->has_var = true;
  }
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) {
    delete m;
    return cuda_status(e, "fgb_mapped_create");
  }
  *out = m;
  return FGB_OK;
}

extern "C" int fgb_mapped_destroy(fgb_mapped_t m) {
  delete m;
  return FGB_OK;
}

extern "C" int fgb_mapped_predict(fgb_mapped_t m, int n_struc,
                                  const int *h_atom_offsets,
                                  const double *h_cells,
                                  const double *d_positions,
                                  const int *d_species, double cutoff,
                                  int want, double *d_energy,
                                  double *d_forces, double *d_stress,
                                  double *d_atom_energy, double *d_local_var,
                                  int precision, void *stream) {
  if (!m) { set_error("fgb_mapped_predict: null handle"); return FGB_EINVAL; }
  if (precision != FGB_PREC_FP64 && precision != FGB_PREC_MIXED) {
    set_error("fgb_mapped_predict: unknown precision %d", precision);
    return FGB_EINVAL;
  }
  // mixed: the descriptor in double-float and the adjoint in FP32, as in
  // the prediction pipeline; Y = B2 beta stays FP64-level (exact slicing)
  const bool mixed = precision == FGB_PREC_MIXED;
  // FP32 adjoint (and dE/dB2 rows in FP32) unless the coefficients are large
  const bool adj32 = mixed && !m->adjoint_f64;
  if ((want & FGB_WANT_LOCAL_VAR) && !m->has_var) {
    set_error("fgb_mapped_predict: no variance map loaded");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc;
  if ((rc = nlist_build(&m->nl, n_struc, h_atom_offsets, h_cells, d_positions,
                        cutoff, st, false)))
    return rc;
  const B2Params &p = m->b2;
  const int N = m->nl.n_atoms, nd = p.n_d, S = p.n_species;
  const long long P = m->nl.n_pairs;
  const bool want_e = want & FGB_WANT_ENERGY, want_f = want & FGB_WANT_FORCES,
             want_s = want & FGB_WANT_STRESS, want_v = want & FGB_WANT_LOCAL_VAR;
  const bool want_grad = want_f || want_s;
  fgb_workspace &ws = m->ws;
  if ((rc = ws.A.ensure(sizeof(double) * ((size_t)N * p.n_A + 1))) ||
      (rc = ws.B2.ensure(sizeof(double) * ((size_t)N * nd + 1))) ||
      (rc = ws.norms.ensure(sizeof(double) * (N + 1))) ||
      (rc = ws.e_atom.ensure(sizeof(double) * (N + 1))) ||
      (rc = ws.var.ensure(sizeof(double) * (N + 1))) ||
      (rc = ws.gB2.ensure(sizeof(double) * ((size_t)N * nd + 1))) ||
      (rc = ws.pair_grad.ensure(sizeof(double3) * (P + 1))) ||
      (rc = ws.forces.ensure(sizeof(double) * (3 * (size_t)N + 1))) ||
      (rc = ws.virial.ensure(sizeof(double) * (6 * (size_t)N + 1))) ||
      (rc = ws.volume.ensure(sizeof(double) * (n_struc + 1))) ||
      (rc = ws.atom_off.ensure(sizeof(int) * (n_struc + 1))) ||
      (rc = ws.ozerr.ensure(sizeof(int))))
    return rc;
  FGB_CUDA(cudaMemcpyAsync(ws.volume.p, m->nl.h_volume.data(),
                           sizeof(double) * n_struc, cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(ws.atom_off.p, h_atom_offsets,
                           sizeof(int) * (n_struc + 1), cudaMemcpyHostToDevice,
                           st));
  FGB_CUDA(cudaMemsetAsync(ws.ozerr.p, 0, sizeof(int), st));
  if (N > 0) {
    FGB_CUDA(cudaMemsetAsync(ws.e_atom.p, 0, sizeof(double) * N, st));
    FGB_CUDA(cudaMemsetAsync(ws.var.p, 0, sizeof(double) * N, st));
  }
  // the FP32 adjoint's A is written in FP32 by the double-float forward
  if ((rc = launch_b2_forward(p, &m->nl, d_species,
                              adj32 ? nullptr : ws.A.as<double>(),
                              ws.B2.as<double>(), ws.norms.as<double>(), st,
                              mixed && !m->adjoint_f64, nullptr,
                              adj32 ? ws.A.as<float>() : nullptr)))
    return rc;
  std::vector<int> counts;
  if ((rc = species_permutation(S, ws, d_species, N, counts, st))) return rc;
  const int kRows = 32768;
  int base = 0;
  for (int s = 0; s < S; s++) {
    const int Ns = counts[s];
    const int *perm_s = ws.perm.as<int>() + base;
    base += Ns;
    for (int r0 = 0; r0 < Ns; r0 += kRows) {
      const int Mr = std::min(kRows, Ns - r0);
      const int *perm = perm_s + r0;
      const unsigned blocks = ceil_div((long long)Mr * 32, 256);
      const bool need_rows = m->power == 2 || want_v;
      if (need_rows &&
          ((rc = ws.kmat.ensure(sizeof(double) * (size_t)Mr * nd)) ||
           (rc = oz::slice({Mr, nd, oz::kTM, ws.B2.as<double>(), nd, perm,
                            nullptr},
                           ws.ozA, st))))
        return rc;
      if (m->power == 2) {
        if ((rc = oz::gemm_store(ws.ozA, *m->ozBeta[s], ws.kmat.as<double>(),
                                 nd, ws.ozerr.as<int>(), st)))
          return rc;
        if (adj32)
          k_mapped_pow2<<<blocks, 256, 0, st>>>(
              Mr, nd, perm, ws.B2.as<double>(), ws.kmat.as<double>(),
              m->normalized ? 1 : 0, ws.e_atom.as<double>(), ws.gB2.as<float>());
        else
          k_mapped_pow2<<<blocks, 256, 0, st>>>(
              Mr, nd, perm, ws.B2.as<double>(), ws.kmat.as<double>(),
              m->normalized ? 1 : 0, ws.e_atom.as<double>(),
              ws.gB2.as<double>());
        FGB_LAUNCH_CHECK("k_mapped_pow2");
      } else {
        if (adj32)
          k_mapped_pow1<<<blocks, 256, 0, st>>>(
              Mr, nd, perm, ws.B2.as<double>(),
              m->beta.as<double>() + (size_t)s * nd, m->normalized ? 1 : 0,
              ws.e_atom.as<double>(), ws.gB2.as<float>());
        else
          k_mapped_pow1<<<blocks, 256, 0, st>>>(
              Mr, nd, perm, ws.B2.as<double>(),
              m->beta.as<double>() + (size_t)s * nd, m->normalized ? 1 : 0,
              ws.e_atom.as<double>(), ws.gB2.as<double>());
        FGB_LAUNCH_CHECK("k_mapped_pow1");
      }
      if (want_v) {
        if ((rc = oz::gemm_store(ws.ozA, *m->ozQ[s], ws.kmat.as<double>(), nd,
                                 ws.ozerr.as<int>(), st)))
          return rc;
        k_mapped_var<<<blocks, 256, 0, st>>>(
            Mr, nd, perm, ws.B2.as<double>(), ws.kmat.as<double>(),
            m->normalized ? 1 : 0, ws.var.as<double>());
        FGB_LAUNCH_CHECK("k_mapped_var");
      }
    }
  }
  if (want_grad) {
    if ((rc = launch_b2_adjoint(p, &m->nl, d_species,
                                adj32 ? nullptr : ws.A.as<double>(), ws.gB2.p,
                                ws.pair_grad.p, st, adj32,
                                adj32 ? ws.A.as<float>() : nullptr)) ||
        (rc = launch_forces(&m->nl, ws.pair_grad.p, adj32,
                            ws.forces.as<double>(), ws.virial.as<double>(),
                            st)))
      return rc;
    if (d_forces && want_f && N > 0)
      FGB_CUDA(cudaMemcpyAsync(d_forces, ws.forces.p, sizeof(double) * 3 * N,
                               cudaMemcpyDeviceToDevice, st));
  }
  if ((want_e && d_energy) || (want_s && d_stress))
    if ((rc = launch_struct_reduce(
             n_struc, ws.atom_off.as<int>(), ws.volume.as<double>(),
             ws.e_atom.as<double>(),
             want_grad ? ws.virial.as<double>() : nullptr,
             want_e ? d_energy : nullptr, want_s ? d_stress : nullptr, st)))
      return rc;
  if (d_atom_energy && N > 0)
    FGB_CUDA(cudaMemcpyAsync(d_atom_energy, ws.e_atom.p, sizeof(double) * N,
                             cudaMemcpyDeviceToDevice, st));
  if (want_v && d_local_var && N > 0)
    FGB_CUDA(cudaMemcpyAsync(d_local_var, ws.var.p, sizeof(double) * N,
                             cudaMemcpyDeviceToDevice, st));
  int h[5] = {0, 0, 0, 0, 0};
  FGB_CUDA(cudaMemcpyAsync(h, m->nl.flag.p, sizeof(int) * 4,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaMemcpyAsync(h + 4, ws.ozerr.p, sizeof(int),
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  rc = nlist_finish(&m->nl, h);
  if (rc == kNlistRetry) {
    // an atom had more pairs than its single-pass slots: again, with a
    // count pass
    m->nl.count_pass = true;
    rc = fgb_mapped_predict(m, n_struc, h_atom_offsets, h_cells, d_positions,
                            d_species, cutoff, want, d_energy, d_forces,
                            d_stress, d_atom_energy, d_local_var, precision,
                            stream);
    m->nl.count_pass = false;
    return rc;
  }
  if (rc) return rc;
  if (h[4]) {
    set_error("mapped evaluation: a bounded tensor-core wait ran out");
    return FGB_ETIMEOUT;
  }
  return FGB_OK;
}
