// Plain FP64 form: the reference's algorithm on the GPU (stored
// forward-mode descriptor gradients, envs_struc GEMM + scatter), envs_envs,
// and the FP64 QR solve.
#include <cusolverDn.h>

#include "fgb_dense.h"
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


// Stored forward-mode gradients (b2.cpp:181-242 with single-bond gradients
// from :367-395): one CTA per atom, pairs in order.  For pair p (i -> j,
// species s_j) the single-bond gradient is nonzero only in block s_j:
// dA_p[c][n][lm] = dg_n (x_c/r) Y_lm + g_n dY_lm/dx_c, and
// dB2_p[c][(n1,n2,l)] = sum_m A[n1][lm] dA_p[c][n2][lm] + dA_p[c][n1][lm] A[n2][lm].
// Shared: A[nA] | B2[nd] | g,dg[nm] | Y[nh] | Yd[3nh] | dA[3 nm nh] | red[3*64]
constexpr int kDT = 64;

__global__ void __launch_bounds__(kDT)
k_b2_dervs(B2Params p, int n_atoms, const long long *__restrict__ offsets,
           const int *__restrict__ nbr_j, const double4_16a *__restrict__ rel,
           const int *__restrict__ species, const double *__restrict__ A_in,
           const double *__restrict__ B2_in, double *__restrict__ dB2,
           double *__restrict__ fdots) {
  extern __shared__ double smem[];
  const int i = blockIdx.x;
  if (i >= n_atoms) return;
  const int nA = p.n_A, nh = p.n_harm, nm = p.n_max, nr = p.n_rad,
            L1 = p.l_max + 1, nd = p.n_d;
  double *A = smem;
  double *Bv = A + nA;
  double *g = Bv + nd;
  double *dg = g + nm;
  double *Y = dg + nm;
  double *Yd = Y + nh;
  double *dA = Yd + 3 * nh;
  double *red = dA + 3 * nm * nh;
  const int t = threadIdx.x;
  for (int e = t; e < nA; e += blockDim.x) A[e] = A_in[(long long)i * nA + e];
  for (int q = t; q < nd; q += blockDim.x) Bv[q] = B2_in[(long long)i * nd + q];
  const int si = species[i];
  __syncthreads();
  for (long long pp = offsets[i]; pp < offsets[i + 1]; pp++) {
    const int j = nbr_j[pp];
    const double4_16a r = rel[pp];
    const int sj = species[j];
    const double rc = p.cutoffs[si * kMaxSpecies + sj];
    const bool keep = r.x <= rc;
    if (t == 0 && keep) {
      radial_eval<double>(p, r.x, rc, g, dg);
      ylm_eval<double>(p.l_max, r.y, r.z, r.w, Y, Yd);
    }
    __syncthreads();
    if (keep) {
      const double ir = 1.0 / r.x;
      const double e3[3] = {r.y * ir, r.z * ir, r.w * ir};
      for (int e = t; e < 3 * nm * nh; e += blockDim.x) {
        int c = e / (nm * nh), n = (e / nh) % nm, lm = e % nh;
        dA[e] = dg[n] * e3[c] * Y[lm] + g[n] * Yd[3 * lm + c];
      }
    }
    __syncthreads();
    double fd[3] = {0.0, 0.0, 0.0};
    for (int q = t; q < nd; q += blockDim.x) {
      double v[3] = {0.0, 0.0, 0.0};
      if (keep) {
        int l = q % L1, pidx = q / L1, n1 = 0;
        while (pidx >= nr - n1) { pidx -= nr - n1; n1++; }
        int n2 = n1 + pidx;
        int b1 = n1 / nm, b2 = n2 / nm;
        const double *a1 = A + n1 * nh + l * l, *a2 = A + n2 * nh + l * l;
        for (int c = 0; c < 3; c++) {
          double acc = 0.0;
          const double *d1 = dA + c * nm * nh + (n1 - b1 * nm) * nh + l * l;
          const double *d2 = dA + c * nm * nh + (n2 - b2 * nm) * nh + l * l;
          for (int m = 0; m < 2 * l + 1; m++) {
            if (b2 == sj) acc += a1[m] * d2[m];
            if (b1 == sj) acc += d1[m] * a2[m];
          }
          v[c] = acc;
        }
      }
      for (int c = 0; c < 3; c++) {
        dB2[(3 * pp + c) * nd + q] = v[c];
        fd[c] += v[c] * Bv[q];
      }
    }
    for (int c = 0; c < 3; c++) red[c * kDT + t] = fd[c];
    __syncthreads();
    for (int h = kDT / 2; h > 0; h >>= 1) {
      if (t < h)
        for (int c = 0; c < 3; c++) red[c * kDT + t] += red[c * kDT + t + h];
      __syncthreads();
    }
    if (t == 0)
      for (int c = 0; c < 3; c++) fdots[3 * pp + c] = red[c * kDT];
    __syncthreads();
  }
}

// Dots_s = B2[perm] S_s^T (raw descriptors), Ns x Ms.
__global__ void __launch_bounds__(GT)
k_dots(int M, int N, int K, const double *__restrict__ B2,
       const int *__restrict__ perm, const double *__restrict__ S,
       double *__restrict__ out) {
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  double acc[4][4];
  gemm_mainloop<true>(acc, m0, n0, M, N, K, B2, K, perm, S, K);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int m = m0 + ty + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n = n0 + tx + 16 * j;
      if (n < N) out[(long long)m * N + n] = acc[i][j];
    }
  }
}

// Force-kernel values for the pairs of species-s centres
// (normalized_dot_product.cpp:185-198): rows are dB2 rows 3p+c (gathered),
// columns the species' sparse environments.  Written into FK[3P x M].
__global__ void __launch_bounds__(GT)
k_force_kernel(int R, int Ms, int K, const double *__restrict__ dB2,
               const int *__restrict__ rows, const double *__restrict__ S,
               const int *__restrict__ pair_center,
               const int *__restrict__ inv_perm,
               const double *__restrict__ dots, const double *__restrict__ dnorm,
               const double *__restrict__ snorm,
               const double *__restrict__ fdots, double sig2, double power,
               int c_s, int M, double *__restrict__ FK) {
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  double acc[4][4];
  gemm_mainloop<true>(acc, m0, n0, R, Ms, K, dB2, K, rows, S, K);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int m = m0 + ty + 16 * i;
    if (m >= R) continue;
    long long gr = rows[m];
    int pair = (int)(gr / 3);
    int atom = pair_center[pair];
    int jl = inv_perm[atom];
    double nj = dnorm[atom];
#pragma unroll
    for (int jj = 0; jj < 4; jj++) {
      int n = n0 + tx + 16 * jj;
      if (n >= Ms) continue;
      double ni = snorm[n];
      double v = 0.0;
      if (ni >= kEmptyThresh && nj >= kEmptyThresh) {
        double nij = ni * nj, nij3 = nij * nj * nj;
        double dv = dots[(long long)jl * Ms + n];
        double nd_ = dv / nij;
        double dval = power * pow(nd_, power - 1.0);
        double f1 = acc[i][jj] / nij;
        double f2 = dv * fdots[gr] / nij3;
        v = sig2 * dval * (f1 - f2);
      }
      FK[gr * M + c_s + n] = v;
    }
  }
}

// Energy column: K[c_s + i][0] = sum_j sig2 (dot_ij / |s_i||d_j|)^power.
__global__ void k_energy_col(int Ns, int Ms, const double *__restrict__ dots,
                             const int *__restrict__ perm,
                             const double *__restrict__ dnorm,
                             const double *__restrict__ snorm, double sig2,
                             double power, int c_s, long long ncol,
                             double *__restrict__ kern) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Ms) return;
  double ni = snorm[i];
  double acc = 0.0;
  if (ni >= kEmptyThresh)
    for (int j = 0; j < Ns; j++) {
      double nj = dnorm[perm[j]];
      if (nj < kEmptyThresh) continue;
      acc += sig2 * pow(dots[(long long)j * Ms + i] / (ni * nj), power);
    }
  kern[(long long)(c_s + i) * ncol] = acc;
}

// Force columns by owner-computes: K[i][1+3a+c] = sum_{p in out(a)}
// FK[3p+c][i] - FK[3 twin(p)+c][i].  Thread per (sparse i, atom a).
__global__ void k_force_cols(int M, int N, const long long *__restrict__ off,
                             const long long *__restrict__ twin,
                             const double *__restrict__ FK, long long ncol,
                             double *__restrict__ kern) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)M * N) return;
  int i = (int)(idx % M), a = (int)(idx / M);
  double f[3] = {0.0, 0.0, 0.0};
  for (long long q = off[a]; q < off[a + 1]; q++) {
    long long tw = twin[q];
    for (int c = 0; c < 3; c++) {
      double v = FK[(3 * q + c) * M + i];
      if (tw >= 0) v -= FK[(3 * tw + c) * M + i];
      f[c] += v;
    }
  }
  for (int c = 0; c < 3; c++) kern[(long long)i * ncol + 1 + 3 * a + c] = f[c];
}

// Stress columns: -(1/V) sum_p fk_a r_b for b >= a (flare order).
__global__ void k_stress_cols(int M, long long P, const double4_16a *__restrict__ rel,
                              const double *__restrict__ FK, double vol_inv,
                              int n_atoms, long long ncol,
                              double *__restrict__ kern) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (long long p = 0; p < P; p++) {
    double4_16a r = rel[p];
    double c3[3] = {r.y, r.z, r.w};
    int k = 0;
    for (int a = 0; a < 3; a++) {
      double fk = FK[(3 * p + a) * M + i];
      for (int b = a; b < 3; b++) s[k++] -= fk * c3[b] * vol_inv;
    }
  }
  for (int k = 0; k < 6; k++)
    kern[(long long)i * ncol + 1 + 3LL * n_atoms + k] = s[k];
}

// mean_efs[o] = sum_i kern[i][o] alpha[i]
__global__ void k_kern_t_alpha(int M, long long ncol, const double *__restrict__ kern,
                               const double *__restrict__ alpha,
                               double *__restrict__ out) {
  long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= ncol) return;
  double acc = 0.0;
  for (int i = 0; i < M; i++) acc += kern[(long long)i * ncol + o] * alpha[i];
  out[o] = acc;
}

__global__ void k_pair_center(int N, const long long *__restrict__ off,
                              int *__restrict__ center) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  for (long long p = off[a]; p < off[a + 1]; p++) center[p] = a;
}

__global__ void k_rownorms(int M, int nd, const double *__restrict__ S,
                           double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  double acc = 0.0;
  for (int q = 0; q < nd; q++) acc += S[(long long)i * nd + q] * S[(long long)i * nd + q];
  out[i] = sqrt(acc);
}

}  // namespace

int launch_b2_dervs(const B2Params &p, const fgb_nlist_s *nl,
                    const int *d_species, const double *d_A, const double *d_B2,
                    double *d_dB2, double *d_force_dots, cudaStream_t st) {
  const int N = nl->n_atoms;
  if (N == 0 || nl->n_pairs == 0) return FGB_OK;
  size_t sm = sizeof(double) * ((size_t)p.n_A + p.n_d + 2 * p.n_max +
                                4 * p.n_harm + 3 * (size_t)p.n_max * p.n_harm +
                                3 * kDT);
  if (sm > 200 * 1024) {
    set_error("stored-gradient form needs %zu bytes of shared memory", sm);
    return FGB_EINVAL;
  }
  FGB_CUDA(cudaFuncSetAttribute(k_b2_dervs,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sm));
  k_b2_dervs<<<N, kDT, sm, st>>>(p, N, nl->offsets.as<long long>(),
                                 nl->nbr_j.as<int>(), nl->nbr_rel.as<double4_16a>(),
                                 d_species, d_A, d_B2, d_dB2, d_force_dots);
  FGB_LAUNCH_CHECK("k_b2_dervs");
  return FGB_OK;
}

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


extern "C" int fgb_b2_forward_dervs(fgb_b2_t b2, fgb_nlist_t nl,
                                    const int *d_species, double *d_B2,
                                    double *d_norms, double *d_dB2,
                                    double *d_force_dots, void *stream) {
  if (!b2 || !nl || !d_B2 || !d_norms || !d_dB2 || !d_force_dots) {
    set_error("fgb_b2_forward_dervs: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf A, flag;
  int rc;
  if ((rc = check_species(d_species, nl->n_atoms, b2->p.n_species, flag, st)))
    return rc;
  if ((rc = A.ensure(sizeof(double) * ((size_t)nl->n_atoms * b2->p.n_A + 1))))
    return rc;
  if ((rc = launch_b2_forward(b2->p, nl, d_species, A.as<double>(), d_B2,
                              d_norms, st)))
    return rc;
  rc = launch_b2_dervs(b2->p, nl, d_species, A.as<double>(), d_B2, d_dB2,
                       d_force_dots, st);
  if (!rc) FGB_CUDA(cudaStreamSynchronize(st));
  return rc;
}

namespace fgb {
// envs_struc for one structure into d_kern; B2/norms of the structure are
// left in ws (for the plain prediction's variance stage).
int envs_struc_impl(const B2Params &p, double sigma, double power,
                           const int *h_counts, const double *d_sparse,
                           fgb_nlist_s *nl, const int *d_species,
                           double *d_kern, fgb_workspace &ws,
                           cudaStream_t st) {
  if (nl->n_struc != 1) {
    set_error("envs_struc needs a single-structure neighbour list");
    return FGB_EINVAL;
  }
  const int N = nl->n_atoms, S = p.n_species, nd = p.n_d;
  const long long P = nl->n_pairs;
  int rc;
  if ((rc = check_species(d_species, N, S, ws.flag, st))) return rc;
  std::vector<int> off(S + 1, 0);
  for (int s = 0; s < S; s++) off[s + 1] = off[s] + h_counts[s];
  const int M = off[S];
  const long long ncol = 1 + 3LL * N + 6;
  if (M == 0) return FGB_OK;
  FGB_CUDA(cudaMemsetAsync(d_kern, 0, sizeof(double) * M * ncol, st));
  if (N == 0) return FGB_OK;
  if ((rc = ws.A.ensure(sizeof(double) * ((size_t)N * p.n_A + 1))) ||
      (rc = ws.B2.ensure(sizeof(double) * ((size_t)N * nd + 1))) ||
      (rc = ws.norms.ensure(sizeof(double) * (N + 1))) ||
      (rc = ws.dB2.ensure(sizeof(double) * ((size_t)3 * P * nd + 1))) ||
      (rc = ws.fdots.ensure(sizeof(double) * (3 * P + 1))) ||
      (rc = ws.kern.ensure(sizeof(double) * ((size_t)3 * P * M + 1))) ||
      (rc = ws.var.ensure(sizeof(double) * (M + 1))) ||
      (rc = ws.pos.ensure(sizeof(int) * (P + 1))) ||
      (rc = ws.perm.ensure(sizeof(int) * (N + 1))) ||
      (rc = ws.flags.ensure(sizeof(int) * (N + 1))) ||
      (rc = ws.scal.ensure(sizeof(int) * (3 * P + 1))))
    return rc;
  if ((rc = launch_b2_forward(p, nl, d_species, ws.A.as<double>(),
                              ws.B2.as<double>(), ws.norms.as<double>(), st)))
    return rc;
  if ((rc = launch_b2_dervs(p, nl, d_species, ws.A.as<double>(),
                            ws.B2.as<double>(), ws.dB2.as<double>(),
                            ws.fdots.as<double>(), st)))
    return rc;
  // host-side species permutation and pair rows (plain path: sync is fine)
  std::vector<int> hs(N);
  std::vector<long long> hoff(N + 1);
  FGB_CUDA(cudaMemcpyAsync(hs.data(), d_species, sizeof(int) * N,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaMemcpyAsync(hoff.data(), nl->offsets.p,
                           sizeof(long long) * (N + 1), cudaMemcpyDeviceToHost,
                           st));
  FGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int> perm, inv(N), rows;
  std::vector<int> sbase(S + 1, 0);
  for (int s = 0; s < S; s++) {
    sbase[s] = (int)perm.size();
    for (int a = 0; a < N; a++)
      if (hs[a] == s) { inv[a] = (int)perm.size() - sbase[s]; perm.push_back(a); }
  }
  sbase[S] = N;
  FGB_CUDA(cudaMemcpyAsync(ws.perm.p, perm.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(ws.flags.p, inv.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  k_pair_center<<<ceil_div(N, 128), 128, 0, st>>>(
      N, nl->offsets.as<long long>(), ws.pos.as<int>());
  FGB_LAUNCH_CHECK("k_pair_center");
  DevBuf snorm, dots, rowsd;
  if ((rc = snorm.ensure(sizeof(double) * (M + 1)))) return rc;
  k_rownorms<<<ceil_div(M, 128), 128, 0, st>>>(M, nd, d_sparse,
                                               snorm.as<double>());
  FGB_LAUNCH_CHECK("k_rownorms");
  FGB_CUDA(cudaMemsetAsync(ws.kern.p, 0, sizeof(double) * 3 * P * M, st));
  const double sig2 = sigma * sigma;
  for (int s = 0; s < S; s++) {
    const int Ns = sbase[s + 1] - sbase[s], Ms = h_counts[s];
    if (Ns == 0 || Ms == 0) continue;
    const double *Ss = d_sparse + (size_t)off[s] * nd;
    const int *perm_s = ws.perm.as<int>() + sbase[s];
    if ((rc = dots.ensure(sizeof(double) * (size_t)Ns * Ms))) return rc;
    dim3 g1(ceil_div(Ms, BN), ceil_div(Ns, BM));
    k_dots<<<g1, GT, 0, st>>>(Ns, Ms, nd, ws.B2.as<double>(), perm_s, Ss,
                              dots.as<double>());
    FGB_LAUNCH_CHECK("k_dots");
    k_energy_col<<<ceil_div(Ms, 128), 128, 0, st>>>(
        Ns, Ms, dots.as<double>(), perm_s, ws.norms.as<double>(),
        snorm.as<double>() + off[s], sig2, power, off[s], ncol, d_kern);
    FGB_LAUNCH_CHECK("k_energy_col");
    rows.clear();
    for (int k = sbase[s]; k < sbase[s + 1]; k++) {
      int a = perm[k];
      for (long long q = hoff[a]; q < hoff[a + 1]; q++)
        for (int c = 0; c < 3; c++) rows.push_back((int)(3 * q + c));
    }
    const int R = (int)rows.size();
    if (R == 0) continue;
    if ((rc = rowsd.ensure(sizeof(int) * R))) return rc;
    FGB_CUDA(cudaMemcpyAsync(rowsd.p, rows.data(), sizeof(int) * R,
                             cudaMemcpyHostToDevice, st));
    dim3 g2(ceil_div(Ms, BN), ceil_div(R, BM));
    k_force_kernel<<<g2, GT, 0, st>>>(
        R, Ms, nd, ws.dB2.as<double>(), rowsd.as<int>(), Ss, ws.pos.as<int>(),
        ws.flags.as<int>(), dots.as<double>(), ws.norms.as<double>(),
        snorm.as<double>() + off[s], ws.fdots.as<double>(), sig2, power,
        off[s], M, ws.kern.as<double>());
    FGB_LAUNCH_CHECK("k_force_kernel");
    FGB_CUDA(cudaStreamSynchronize(st));   // rows buffer reused next species
  }
  k_force_cols<<<ceil_div((long long)M * N, 128), 128, 0, st>>>(
      M, N, nl->offsets.as<long long>(), nl->nbr_twin.as<long long>(),
      ws.kern.as<double>(), ncol, d_kern);
  FGB_LAUNCH_CHECK("k_force_cols");
  k_stress_cols<<<ceil_div(M, 64), 64, 0, st>>>(
      M, P, nl->nbr_rel.as<double4_16a>(), ws.kern.as<double>(),
      1.0 / nl->h_volume[0], N, ncol, d_kern);
  FGB_LAUNCH_CHECK("k_stress_cols");
  return FGB_OK;
}
}  // namespace fgb

extern "C" int fgb_envs_struc(fgb_b2_t b2, double sigma, double power,
                              const int *h_counts, const double *d_sparse,
                              fgb_nlist_t nl, const int *d_species,
                              double *d_kern, void *stream) {
  if (!b2 || !nl || !h_counts || !d_kern) {
    set_error("fgb_envs_struc: invalid arguments");
    return FGB_EINVAL;
  }
  fgb_workspace ws;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = envs_struc_impl(b2->p, sigma, power, h_counts, d_sparse, nl,
                           d_species, d_kern, ws, st);
  if (!rc) FGB_CUDA(cudaStreamSynchronize(st));
  return rc;
}

extern "C" int fgb_predict_plain(fgb_model_t m, fgb_nlist_t nl,
                                 const int *d_species, double *d_mean_efs,
                                 double *d_local_var, void *stream) {
  if (!m || !nl || !d_mean_efs) {
    set_error("fgb_predict_plain: invalid arguments");
    return FGB_EINVAL;
  }
  if (!m->solved) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N = nl->n_atoms, M = m->M;
  const long long ncol = 1 + 3LL * N + 6;
  int rc;
  DevBuf kern;
  if ((rc = kern.ensure(sizeof(double) * ((size_t)M * ncol + 1)))) return rc;
  if ((rc = envs_struc_impl(m->b2, m->sigma, m->power, m->h_counts.data(),
                            m->Sraw.as<double>(), nl, d_species,
                            kern.as<double>(), m->ws, st)))
    return rc;
  k_kern_t_alpha<<<ceil_div(ncol, 128), 128, 0, st>>>(
      M, ncol, kern.as<double>(), m->alpha.as<double>(), d_mean_efs);
  FGB_LAUNCH_CHECK("k_kern_t_alpha");
  if (d_local_var && N > 0) {
    // local variances: envs_envs(structure, sparse) then |L_inv k|^2
    // (sparse_gp.cpp:116-133), on the B2 values left in the workspace.
    std::vector<int> counts;
    if ((rc = species_permutation(m, d_species, N, counts, st))) return rc;
    if ((rc = m->ws.var.ensure(sizeof(double) * (N + 1)))) return rc;
    if ((rc = kernel_stage_fp64(m, N, counts, false, true, nullptr, nullptr,
                                m->ws.var.as<double>(), st)))
      return rc;
    FGB_CUDA(cudaMemcpyAsync(d_local_var, m->ws.var.p, sizeof(double) * N,
                             cudaMemcpyDeviceToDevice, st));
  }
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}

// ------------------------------------------------------------ QR solve
// SparseGP::update_matrices_QR (sparse_gp.cpp:607-641) in FP64:
//   L = chol(Kuu + jitter I);  L_inv = L^-1
//   A = [diag(sqrt(noise)) Kuf^T ; L^T],  b = [sqrt(noise) y ; 0]
//   A = QR;  alpha = R^-1 (Q^T b)[:M];  R_inv = R^-1
// (dense.cu holds the factorisations)
namespace fgb {
namespace {
__global__ void k_add_diag(int M, double *A, double v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < M) A[(long long)i * M + i] += v;
}
// alpha = R_inv Qb (R_inv row-major upper): a warp per row, lanes over
// columns, fixed-order shuffle tree.
__global__ void k_upper_gemv(int M, const double *R, const double *x,
                             double *y) {
  const int row = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= M) return;
  double s = 0.0;
  for (int j = row + lane; j < M; j += 32) s += R[(long long)row * M + j] * x[j];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) y[row] = s;
}
}  // namespace
}  // namespace fgb

#define FGB_SOLVER(call, what)                                          \
  do {                                                                  \
    int s_ = (int)(call);                                               \
    if (s_ != 0) {                                                      \
      set_error("%s failed with status %d", what, s_);                  \
      rc = FGB_ECUDA;                                                   \
      goto done;                                                        \
    }                                                                   \
  } while (0)

// SparseGP::update_matrices_QR (sparse_gp.cpp:607-641) on the GPU in FP64,
// by the kernels of dense.cu: L = chol(Kuu + jitter I), L_inv = L^-1, the
// QR of A = [sqrt(noise) Kuf^T; L^T] by shifted Cholesky QR (R_inv and
// Q^T b; every O(n M^2) and O(M^3) product an FP64-level tensor-core
// product), alpha = R_inv (Q^T b)[:M] (the reference's R_inv * Q_b).
extern "C" int fgb_solve_qr(int M, int n_labels, const double *d_Kuu,
                            const double *d_Kuf, const double *d_y,
                            const double *d_noise, double jitter,
                            double *d_alpha, double *d_L_inv, double *d_R_inv,
                            void *stream) {
  if (M <= 0 || n_labels < 0 || !d_Kuu || !d_alpha || !d_L_inv ||
      (n_labels > 0 && (!d_Kuf || !d_y || !d_noise))) {
    set_error("fgb_solve_qr: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const long long rows = (long long)n_labels + M;
  int rc = FGB_OK;
  DevBuf L, At, b, Qtb, Rinv;
  double *R_inv = d_R_inv;
  if ((rc = L.ensure(sizeof(double) * (size_t)M * M)) ||
      (rc = At.ensure(sizeof(double) * (size_t)rows * M)) ||
      (rc = b.ensure(sizeof(double) * (size_t)rows)) ||
      (rc = Qtb.ensure(sizeof(double) * (size_t)M)))
    return rc;
  if (!R_inv) {
    if ((rc = Rinv.ensure(sizeof(double) * (size_t)M * M))) return rc;
    R_inv = Rinv.as<double>();
  }
  FGB_CUDA(cudaMemcpyAsync(L.p, d_Kuu, sizeof(double) * (size_t)M * M,
                           cudaMemcpyDeviceToDevice, st));
  k_add_diag<<<ceil_div(M, 256), 256, 0, st>>>(M, L.as<double>(), jitter);
  FGB_LAUNCH_CHECK("k_add_diag");
  if ((rc = dense::cholesky(M, L.as<double>(), M, st)) ||
      (rc = dense::trtri_lower(M, L.as<double>(), M, d_L_inv, M, st)) ||
      (rc = dense::build_At(M, n_labels, d_Kuf, d_noise, d_y, L.as<double>(),
                            At.as<double>(), b.as<double>(), st)) ||
      (rc = dense::cholqr_solve(M, rows, At.as<double>(), b.as<double>(),
                                R_inv, Qtb.as<double>(), st)))
    return rc;
  k_upper_gemv<<<ceil_div((long long)M * 32, 256), 256, 0, st>>>(
      M, R_inv, Qtb.as<double>(), d_alpha);
  FGB_LAUNCH_CHECK("k_upper_gemv");
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}

// Thin Q of a Householder QR (cuSOLVER geqrf + orgqr): A and Q column-major
// rows x cols (rows >= cols).  The varmap coefficients of a power-1 model
// (normalized_dot_product.cpp:769-830) are the leading rows of such a Q.
extern "C" int fgb_qr_thin_q(int rows, int cols, const double *d_A,
                             double *d_Q, void *stream) {
  if (rows <= 0 || cols <= 0 || rows < cols || !d_A || !d_Q) {
    set_error("fgb_qr_thin_q: invalid arguments (rows >= cols > 0)");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc = FGB_OK;
  cusolverDnHandle_t sol = nullptr;
  DevBuf tau, work, info;
  int lwork = 0, lw2 = 0, hinfo = 0;
  if ((rc = tau.ensure(sizeof(double) * (size_t)cols)) ||
      (rc = info.ensure(sizeof(int))))
    return rc;
  FGB_SOLVER(cusolverDnCreate(&sol), "cusolverDnCreate");
  FGB_SOLVER(cusolverDnSetStream(sol, st), "cusolverDnSetStream");
  FGB_SOLVER(cudaMemcpyAsync(d_Q, d_A, sizeof(double) * (size_t)rows * cols,
                             cudaMemcpyDeviceToDevice, st), "copy A");
  FGB_SOLVER(cusolverDnDgeqrf_bufferSize(sol, rows, cols, d_Q, rows, &lwork),
             "geqrf_bufferSize");
  FGB_SOLVER(cusolverDnDorgqr_bufferSize(sol, rows, cols, cols, d_Q, rows,
                                         tau.as<double>(), &lw2),
             "orgqr_bufferSize");
  lwork = std::max(lwork, lw2);
  if ((rc = work.ensure(sizeof(double) * ((size_t)lwork + 1)))) goto done;
  FGB_SOLVER(cusolverDnDgeqrf(sol, rows, cols, d_Q, rows, tau.as<double>(),
                              work.as<double>(), lwork, info.as<int>()),
             "geqrf");
  FGB_SOLVER(cusolverDnDorgqr(sol, rows, cols, cols, d_Q, rows,
                              tau.as<double>(), work.as<double>(), lwork,
                              info.as<int>()),
             "orgqr");
  FGB_SOLVER(cudaMemcpyAsync(&hinfo, info.p, sizeof(int),
                             cudaMemcpyDeviceToHost, st), "info");
  FGB_SOLVER(cudaStreamSynchronize(st), "sync");
  if (hinfo != 0) {
    set_error("fgb_qr_thin_q: QR failed (info %d)", hinfo);
    rc = FGB_ECUDA;
  }
done:
  if (sol) cusolverDnDestroy(sol);
  return rc;
}
