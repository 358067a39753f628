// K3/K4: kernel against the sparse set, adjoint GEMM and local variance in
// FP64, plus the device-resident model and the fgb_predict pipeline.
//
// For the atoms of species s (rows gathered through a species permutation):
//   GEMM1 (NT)  C = B2_s S^_s^T;  epilogue c = C/|d|, k = sigma^2 c^xi,
//               w = sigma^2 xi alpha c^(xi-1)   (normalized_dot_product.cpp:171-181)
//   E_i = sum_t alpha_t k_it                     (sparse_gp.cpp:751 mean = K^T alpha)
//   GEMM2 (NN)  G = W S^_s;  epilogue dE/dB2 = (G - xi E d^)/|d|
//   GEMM3 (NT, lower-triangular)  Z = K L_s^T;  epilogue row sums of Z^2
//   var_i = k_self - sum_r Z_ir^2                (sparse_gp.cpp:116-133)
// L_inv of a single-kernel model is block-diagonal by species (cross-species
// Kuu blocks are exactly zero), so species s only needs its panel of L_inv.
#include <cstring>
#include <vector>

#include "fgb_internal.h"
#include "fgb_kernels.h"
#include "fgb_model.h"
#include "fgb_gemm64.cuh"
#include "fgb_profile.h"

namespace fgb {

namespace {

constexpr int kRowChunk = 32768;
using namespace gemm64;

// GEMM1: rows = atoms of one species (through perm), cols = sparse envs.
__global__ void __launch_bounds__(GT)
k_kernel_gemm(int M, int N, int K, const double *__restrict__ B2,
              const int *__restrict__ perm, const double *__restrict__ norms,
              const double *__restrict__ S, const double *__restrict__ alpha,
              const unsigned char *__restrict__ svalid, double sig2, double xi,
              double *__restrict__ Kmat, double *__restrict__ Wmat) {
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  double acc[4][4];
  gemm_mainloop<true>(acc, m0, n0, M, N, K, B2, K, perm, S, K);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int m = m0 + ty + 16 * i;
    if (m >= M) continue;
    double nd = norms[perm[m]];
    bool dok = nd >= kEmptyThresh;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n = n0 + tx + 16 * j;
      if (n >= N) continue;
      double kv = 0.0, wv = 0.0;
      if (dok && svalid[n]) {
        double c = acc[i][j] / nd;
        kv = sig2 * powx(c, xi);
        wv = sig2 * xi * powx(c, xi - 1.0) * alpha[n];
      }
      Kmat[(long long)m * N + n] = kv;
      Wmat[(long long)m * N + n] = wv;
    }
  }
}

// E_m = sum_n alpha_n K[m][n]: warp per row, fixed-order shuffle tree.
__global__ void k_row_energy(int M, int N, const double *__restrict__ Kmat,
                             const double *__restrict__ alpha,
                             const int *__restrict__ perm,
                             double *__restrict__ e_rows,
                             double *__restrict__ e_atom) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= M) return;
  const double *row = Kmat + (long long)warp * N;
  double acc = 0.0;
  for (int n = lane; n < N; n += 32) acc += alpha[n] * row[n];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    acc += __shfl_down_sync(0xffffffffu, acc, off);
  if (lane == 0) {
    e_rows[warp] = acc;
    if (e_atom) e_atom[perm[warp]] = acc;
  }
}

// GEMM2: G = W S (NN); epilogue dE/dB2 rows in atom order.
__global__ void __launch_bounds__(GT)
k_adjoint_gemm(int M, int N, int K, const double *__restrict__ Wmat,
               const double *__restrict__ S, const int *__restrict__ perm,
               const double *__restrict__ norms, const double *__restrict__ B2,
               const double *__restrict__ e_rows, double xi,
               double *__restrict__ gB2) {
  // M rows (atoms), N = n_d columns, K = M_s
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  double acc[4][4];
  gemm_mainloop<false>(acc, m0, n0, M, N, K, Wmat, K, nullptr, S, N);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int m = m0 + ty + 16 * i;
    if (m >= M) continue;
    int atom = perm[m];
    double nd = norms[atom];
    bool dok = nd >= kEmptyThresh;
    double inv = dok ? 1.0 / nd : 0.0;
    double xe = xi * e_rows[m];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n = n0 + tx + 16 * j;
      if (n >= N) continue;
      double v = 0.0;
      if (dok) {
        double dh = B2[(long long)atom * N + n] * inv;
        v = (acc[i][j] - xe * dh) * inv;
      }
      gB2[(long long)atom * N + n] = v;
    }
  }
}

// GEMM3: Z = K L^T over the lower-triangular panel; row sums of Z^2 per
// column tile.
__global__ void __launch_bounds__(GT)
k_variance_gemm(int M, int R, int Ms, const double *__restrict__ Kmat,
                const double *__restrict__ Lp, double *__restrict__ part,
                int ntiles) {
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int kmax = min(Ms, n0 + BN);
  double acc[4][4];
  gemm_mainloop<true>(acc, m0, n0, M, R, kmax, Kmat, Ms, nullptr, Lp, Ms);
  __shared__ double red[16][BM + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n = n0 + tx + 16 * j;
      if (n < R) s += acc[i][j] * acc[i][j];
    }
    red[tx][ty + 16 * i] = s;
  }
  __syncthreads();
  if (threadIdx.x < BM) {
    int mm = threadIdx.x;
    double s = 0.0;
    for (int q = 0; q < 16; q++) s += red[q][mm];
    int m = m0 + mm;
    if (m < M) part[(long long)m * ntiles + blockIdx.x] = s;
  }
}

__global__ void k_variance_final(int M, int ntiles, const double *__restrict__ part,
                                 const int *__restrict__ perm,
                                 const double *__restrict__ norms, double sig2,
                                 double xi, double *__restrict__ var) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int m = (int)(gt / kRowLanes), q = (int)(gt % kRowLanes);
  if (m >= M) return;   // whole lane groups
  const double s = row_slots_sum(part, m, ntiles, q);
  if (q) return;
  int atom = perm[m];
  double nd = norms[atom];
  // K_self = sig^2 (d.d/(|d||d|))^xi, zero for an empty environment.
  double kself = nd >= kEmptyThresh ? sig2 * powx((nd * nd) / (nd * nd), xi)
                                    : 0.0;
  var[atom] = kself - s;
}

__global__ void k_transpose_rm(int R, int C, const double *__restrict__ in,
                               double *__restrict__ out) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)R * C) return;
  int r = (int)(idx / C), c = (int)(idx % C);
  out[(long long)c * R + r] = in[idx];
}

__global__ void k_sum_parts(int M, int ntiles, const double *__restrict__ part,
                            double *__restrict__ out) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  double s = 0.0;
  for (int t = 0; t < ntiles; t++) s += part[(long long)m * ntiles + t];
  out[m] = s;
}

// variance_efs = K_self - Q_self + V_SOR (sparse_gp.cpp:726)
__global__ void k_dtc_combine(long long n, const double *__restrict__ kself,
                              const double *__restrict__ q,
                              double *__restrict__ v) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = kself[i] - q[i] + v[i];
}

__global__ void k_kt_alpha(int M, long long ncol, const double *__restrict__ KT,
                           const double *__restrict__ alpha,
                           double *__restrict__ out) {
  long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= ncol) return;
  double acc = 0.0;
  for (int i = 0; i < M; i++) acc += KT[o * M + i] * alpha[i];
  out[o] = acc;
}

__global__ void k_check_species(int n, const int *__restrict__ species, int ns,
                                int *__restrict__ flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && (species[i] < 0 || species[i] >= ns)) atomicExch(flag, 1);
}

// Species permutation as a counting sort over blocks of kPermBlock atoms
// (n_species <= kMaxSpecies): per-block histograms, one block of offsets,
// then a stable scatter (atoms of a species keep their index order).
constexpr int kPermBlock = 1024;

// hist[s * nb + b] = atoms of species s in block b; flag: a species out of
// [0, ns)
__global__ void __launch_bounds__(kPermBlock)
k_species_hist(int n, const int *__restrict__ species, int ns,
               int *__restrict__ hist, int *__restrict__ flag) {
  __shared__ int cnt[kMaxSpecies];
  const int t = threadIdx.x, b = blockIdx.x, nb = gridDim.x;
  if (t < kMaxSpecies) cnt[t] = 0;
  __syncthreads();
  const int i = b * kPermBlock + t;
  if (i < n) {
    const int sp = species[i];
    if (sp < 0 || sp >= ns) atomicExch(flag, 1);
    else atomicAdd(&cnt[sp], 1);
  }
  __syncthreads();
  if (t < ns) hist[t * nb + b] = cnt[t];
}

// In place: hist becomes the exclusive prefix over (species, block) in
// species-major order, i.e. the first perm slot of each (species, block);
// totals[s] = atoms of species s.  One block; each thread scans a
// contiguous run, then the runs' sums are scanned.
__global__ void __launch_bounds__(kPermBlock)
k_species_offsets(int nb, int ns, int *__restrict__ hist,
                  int *__restrict__ totals) {
  __shared__ int run[kPermBlock];
  __shared__ int grand;
  const int t = threadIdx.x, L = ns * nb;
  const int per = (L + kPermBlock - 1) / kPermBlock;
  const int lo = min(L, t * per), hi = min(L, lo + per);
  int sum = 0;
  for (int k = lo; k < hi; k++) sum += hist[k];
  run[t] = sum;
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    for (int k = 0; k < kPermBlock; k++) {
      const int v = run[k];
      run[k] = acc;
      acc += v;
    }
    grand = acc;
  }
  __syncthreads();
  int acc = run[t];
  for (int k = lo; k < hi; k++) {
    const int v = hist[k];
    hist[k] = acc;
    acc += v;
  }
  __syncthreads();
  if (t < ns) totals[t] = (t + 1 < ns ? hist[(t + 1) * nb] : grand) - hist[t * nb];
}

// perm[first(s, b) + rank of atom i among block b's species-s atoms] = i
__global__ void __launch_bounds__(kPermBlock)
k_species_scatter(int n, const int *__restrict__ species, int ns,
                  const int *__restrict__ first, int *__restrict__ perm) {
  __shared__ int wc[kPermBlock / 32][kMaxSpecies];   // per-warp counts
  const int t = threadIdx.x, b = blockIdx.x, nb = gridDim.x;
  const int w = t >> 5, lane = t & 31;
  const int i = b * kPermBlock + t;
  int sp = i < n ? species[i] : -1;
  if (sp >= ns) sp = -1;
  const unsigned same = __match_any_sync(0xffffffffu, sp);
  const int rank = __popc(same & ((1u << lane) - 1u));
  if (lane < kMaxSpecies) wc[w][lane] = 0;
  __syncwarp();
  if (sp >= 0 && rank == 0) wc[w][sp] = __popc(same);
  __syncthreads();
  if (sp >= 0) {
    int before = 0;
    for (int q = 0; q < w; q++) before += wc[q][sp];
    perm[first[sp * nb + b] + before + rank] = i;
  }
}

}  // namespace

int launch_row_energy(int Mr, int Ms, const double *Kmat, const double *alpha,
                      const int *perm, double *e_rows, double *e_atom,
                      cudaStream_t st) {
  StageTimer _pt(kStRowEnergy, st);
  k_row_energy<<<ceil_div((long long)Mr * 32, 256), 256, 0, st>>>(
      Mr, Ms, Kmat, alpha, perm, e_rows, e_atom);
  FGB_LAUNCH_CHECK("k_row_energy");
  return FGB_OK;
}

int launch_variance_final(int Mr, int ntiles, const double *part,
                          const int *perm, const double *norms, double sig2,
                          double xi, double *var, cudaStream_t st) {
  StageTimer _pt(kStVarianceFinal, st);
  k_variance_final<<<
      ceil_div((long long)Mr * kRowLanes, 128), 128, 0, st>>>(
      Mr, ntiles, part, perm, norms, sig2, xi, var);
  FGB_LAUNCH_CHECK("k_variance_final");
  return FGB_OK;
}

int launch_variance_fp64(int Mr, int R, int Ms, const double *Kmat,
                         const double *Lp, double *part, int ntiles,
                         cudaStream_t st) {
  StageTimer _pt(kStVarianceGemm, st);
  dim3 g3(ntiles, ceil_div(Mr, BM));
  k_variance_gemm<<<g3, GT, 0, st>>>(Mr, R, Ms, Kmat, Lp, part, ntiles);
  FGB_LAUNCH_CHECK("k_variance_gemm");
  return FGB_OK;
}

int check_species(const int *d_species, int n, int n_species, DevBuf &flag,
                  cudaStream_t st) {
  if (n == 0) return FGB_OK;
  int rc = flag.ensure(sizeof(int));
  if (rc) return rc;
  FGB_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
  k_check_species<<<ceil_div(n, 256), 256, 0, st>>>(n, d_species, n_species,
                                                    flag.as<int>());
  FGB_LAUNCH_CHECK("k_check_species");
  int h = 0;
  FGB_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error("species must lie in [0, %d)", n_species);
    return FGB_EINVAL;
  }
  return FGB_OK;
}

// Species permutation: perm = atoms of species 0 (ascending), then 1, ...
// The species range check and every species count come back to the host in
// one read (a single wait).
int species_permutation(fgb_model_s *m, const int *d_species, int N,
                        std::vector<int> &counts, cudaStream_t st,
                        const int *h_species) {
  return species_permutation(m->b2.n_species, m->ws, d_species, N, counts, st,
                             h_species);
}

int species_permutation(int S, fgb_workspace &ws, const int *d_species, int N,
                        std::vector<int> &counts, cudaStream_t st,
                        const int *h_species) {
  bool pending = false;
  int rc = species_permutation_start(S, ws, d_species, N, counts, st,
                                     h_species, pending);
  if (rc || !pending) return rc;
  return species_permutation_finish(S, ws, counts);
}

int species_permutation_start(int S, fgb_workspace &ws, const int *d_species,
                              int N, std::vector<int> &counts, cudaStream_t st,
                              const int *h_species, bool &pending) {
  pending = false;
  counts.assign(S, 0);
  if (S < 1 || S > kMaxSpecies) {
    set_error("species permutation: %d species (at most %d)", S, kMaxSpecies);
    return FGB_EINVAL;
  }
  if (h_species) {
    for (int i = 0; i < N; i++) {
      const int q = h_species[i];
      if (q < 0 || q >= S) {
        set_error("species must lie in [0, %d)", S);
        return FGB_EINVAL;
      }
      counts[q]++;
    }
  }
  const int nb = ceil_div(std::max(N, 1), kPermBlock);
  int rc;
  if ((rc = ws.perm.ensure(sizeof(int) * (N + 1))) ||
      (rc = ws.flags.ensure(sizeof(int) * ((size_t)S * nb + 1))) ||
      (rc = ws.scal.ensure(sizeof(int) * (S + 2))))
    return rc;
  if (N == 0) return FGB_OK;
  int *tot = ws.scal.as<int>();   // [0, S): counts; [S]: range flag
  int *hist = ws.flags.as<int>();
  FGB_CUDA(cudaMemsetAsync(tot + S, 0, sizeof(int), st));
  k_species_hist<<<nb, kPermBlock, 0, st>>>(N, d_species, S, hist, tot + S);
  FGB_LAUNCH_CHECK("k_species_hist");
  k_species_offsets<<<1, kPermBlock, 0, st>>>(nb, S, hist, tot);
  FGB_LAUNCH_CHECK("k_species_offsets");
  k_species_scatter<<<nb, kPermBlock, 0, st>>>(N, d_species, S, hist,
                                               ws.perm.as<int>());
  FGB_LAUNCH_CHECK("k_species_scatter");
  if (h_species) return FGB_OK;   // counted and checked above
  fgb_pinned_counts &pc = ws.counts;
  if (!pc.h)
    FGB_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&pc.h),
                           sizeof(int) * (kMaxSpecies + 1),
                           cudaHostAllocDefault));
  if (!pc.ev) FGB_CUDA(cudaEventCreateWithFlags(&pc.ev, cudaEventDisableTiming));
  FGB_CUDA(cudaMemcpyAsync(pc.h, tot, sizeof(int) * (S + 1),
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaEventRecord(pc.ev, st));
  pending = true;
  return FGB_OK;
}

int species_permutation_finish(int S, fgb_workspace &ws,
                               std::vector<int> &counts) {
  const fgb_pinned_counts &pc = ws.counts;
  FGB_CUDA(cudaEventSynchronize(pc.ev));
  if (pc.h[S]) {
    set_error("species must lie in [0, %d)", S);
    return FGB_EINVAL;
  }
  counts.assign(pc.h, pc.h + S);
  return FGB_OK;
}

// Kernel, energy, adjoint GEMM and variance for all species (FP64).
int kernel_stage_fp64(fgb_model_s *m, int N, const std::vector<int> &counts,
                      bool want_grad, bool want_var, double *d_e_atom,
                      double *d_gB2, double *d_var, cudaStream_t st) {
  const B2Params &p = m->b2;
  const int nd = p.n_d;
  const double sig2 = m->sigma * m->sigma;
  int base = 0;
  for (int s = 0; s < p.n_species; s++) {
    const int Ns = counts[s];
    const int Ms = m->h_counts[s];
    const int *perm_s = m->ws.perm.as<int>() + base;
    if (Ns > 0 && Ms == 0 && want_var) {
      // No sparse environments of this species: k = 0 and E = 0 (zero
      // filled), var = k_self.
      k_variance_final<<<
          ceil_div((long long)Ns * kRowLanes, 128), 128, 0, st>>>(
          Ns, 0, nullptr, perm_s, m->ws.norms.as<double>(), sig2, m->power,
          d_var);
      FGB_LAUNCH_CHECK("k_variance_final");
    }
    for (int r0 = 0; r0 < Ns && Ms > 0; r0 += kRowChunk) {
      const int Mr = std::min(kRowChunk, Ns - r0);
      const int *perm = perm_s + r0;
      int rc;
      if ((rc = m->ws.kmat.ensure(sizeof(double) * (size_t)Mr * Ms)) ||
          (rc = m->ws.wmat.ensure(sizeof(double) * (size_t)Mr * Ms)) ||
          (rc = m->ws.erows.ensure(sizeof(double) * (size_t)Mr)))
        return rc;
      dim3 g1(ceil_div(Ms, BN), ceil_div(Mr, BM));
      {
        StageTimer _pt(kStKernelGemm, st, 1);
        k_kernel_gemm<<<g1, GT, 0, st>>>(
            Mr, Ms, nd, m->ws.B2.as<double>(), perm, m->ws.norms.as<double>(),
            m->S.as<double>() + (size_t)m->h_offsets[s] * nd,
            m->alpha.as<double>() + m->h_offsets[s],
            m->svalid.as<unsigned char>() + m->h_offsets[s], sig2, m->power,
            m->ws.kmat.as<double>(), m->ws.wmat.as<double>());
        FGB_LAUNCH_CHECK("k_kernel_gemm");
      }
      {
        StageTimer _pt(kStRowEnergy, st, 1);
        k_row_energy<<<ceil_div((long long)Mr * 32, 256), 256, 0, st>>>(
            Mr, Ms, m->ws.kmat.as<double>(),
            m->alpha.as<double>() + m->h_offsets[s], perm,
            m->ws.erows.as<double>(), d_e_atom);
        FGB_LAUNCH_CHECK("k_row_energy");
      }
      if (want_grad) {
        dim3 g2(ceil_div(nd, BN), ceil_div(Mr, BM));
        {
          StageTimer _pt(kStAdjointGemm, st, 1);
          k_adjoint_gemm<<<g2, GT, 0, st>>>(
              Mr, nd, Ms, m->ws.wmat.as<double>(),
              m->S.as<double>() + (size_t)m->h_offsets[s] * nd, perm,
              m->ws.norms.as<double>(), m->ws.B2.as<double>(),
              m->ws.erows.as<double>(), m->power, d_gB2);
          FGB_LAUNCH_CHECK("k_adjoint_gemm");
        }
      }
      if (want_var) {
        const int R = m->h_panel_rows[s];
        const int ntiles = ceil_div(R, BN);
        if ((rc = m->ws.part.ensure(sizeof(double) * (size_t)Mr * ntiles)))
          return rc;
        dim3 g3(ntiles, ceil_div(Mr, BM));
        {
          StageTimer _pt(kStVarianceGemm, st, 1);
          k_variance_gemm<<<g3, GT, 0, st>>>(
              Mr, R, Ms, m->ws.kmat.as<double>(),
              m->Lp.as<double>() + m->h_panel_off[s], m->ws.part.as<double>(),
              ntiles);
          FGB_LAUNCH_CHECK("k_variance_gemm");
        }
        {
          StageTimer _pt(kStVarianceFinal, st, 1);
          k_variance_final<<<
              ceil_div((long long)Mr * kRowLanes, 128), 128, 0, st>>>(
              Mr, ntiles, m->ws.part.as<double>(), perm,
              m->ws.norms.as<double>(), sig2, m->power, d_var);
          FGB_LAUNCH_CHECK("k_variance_final");
        }
      }
    }
    base += Ns;
  }
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

// ----------------------------------------------------------------- model
extern "C" int fgb_model_create(fgb_model_t *out, fgb_b2_t b2, double sigma,
                                double power) {
  if (!out || !b2) { set_error("fgb_model_create: invalid arguments"); return FGB_EINVAL; }
  if (!std::isfinite(sigma) || !std::isfinite(power)) {
    set_error("fgb_model_create: non-finite hyperparameters");
    return FGB_EINVAL;
  }
  fgb_model_s *m = new fgb_model_s();
  m->b2 = b2->p;
  m->sigma = sigma;
  m->power = power;
  *out = m;
  return FGB_OK;
}

extern "C" int fgb_model_destroy(fgb_model_t m) {
  delete m;
  return FGB_OK;
}

extern "C" int fgb_model_set(fgb_model_t m, const int *h_counts,
                             const double *h_desc, const double *h_alpha,
                             const double *h_L_inv) {
  if (!m || !h_counts) { set_error("fgb_model_set: invalid arguments"); return FGB_EINVAL; }
  const int S = m->b2.n_species, nd = m->b2.n_d;
  m->h_counts.assign(h_counts, h_counts + S);
  m->h_offsets.assign(S + 1, 0);
  for (int s = 0; s < S; s++) {
    if (h_counts[s] < 0) { set_error("fgb_model_set: negative count"); return FGB_EINVAL; }
    m->h_offsets[s + 1] = m->h_offsets[s] + h_counts[s];
  }
  const int M = m->h_offsets[S];
  m->M = M;
  if (M > 0 && !h_desc) { set_error("fgb_model_set: descriptors required"); return FGB_EINVAL; }
  // normalised sparse descriptors, validity flags (norm >= 1e-8)
  std::vector<double> Sh((size_t)M * nd);
  std::vector<unsigned char> valid(M);
  std::vector<double> snorm(M);
  for (int t = 0; t < M; t++) {
    const double *row = h_desc + (size_t)t * nd;
    double nn = 0;
    for (int q = 0; q < nd; q++) nn += row[q] * row[q];
    double n = std::sqrt(nn);
    snorm[t] = n;
    valid[t] = n >= kEmptyThresh;
    for (int q = 0; q < nd; q++) Sh[(size_t)t * nd + q] = valid[t] ? row[q] / n : 0.0;
  }
  m->h_snorm = snorm;
  m->h_desc.assign(h_desc, h_desc + (size_t)M * nd);
  int rc;
  if ((rc = m->S.ensure(sizeof(double) * (size_t)M * nd)) ||
      (rc = m->svalid.ensure(M + 1)) ||
      (rc = m->Sraw.ensure(sizeof(double) * (size_t)M * nd)) ||
      (rc = m->snorm.ensure(sizeof(double) * (M + 1))))
    return rc;
  if (M > 0) {
    FGB_CUDA(cudaMemcpy(m->S.p, Sh.data(), sizeof(double) * (size_t)M * nd,
                        cudaMemcpyHostToDevice));
    FGB_CUDA(cudaMemcpy(m->Sraw.p, h_desc, sizeof(double) * (size_t)M * nd,
                        cudaMemcpyHostToDevice));
    FGB_CUDA(cudaMemcpy(m->svalid.p, valid.data(), M, cudaMemcpyHostToDevice));
    FGB_CUDA(cudaMemcpy(m->snorm.p, snorm.data(), sizeof(double) * M,
                        cudaMemcpyHostToDevice));
  }
  m->solved = false;
  m->bmap_ready = false;
  m->lfull_ready = false;
  m->slices_chosen = false;
  m->oz_S = oz::kS;
  m->oz_Sv = oz::kS;
  m->oz_err_est = 0.0;
  m->oz_var_err_est = 0.0;
  m->force_f64 = false;
  m->fold_max = 0.0;
  for (bool &r : m->ozS_ready) r = false;
  for (bool &r : m->ozL_ready) r = false;
  for (bool &r : m->ozB_ready) r = false;
  if (!h_alpha || !h_L_inv) return FGB_OK;
  if ((rc = m->alpha.ensure(sizeof(double) * (M + 1)))) return rc;
  if (M > 0)
    FGB_CUDA(cudaMemcpy(m->alpha.p, h_alpha, sizeof(double) * M,
                        cudaMemcpyHostToDevice));
  m->h_alpha.assign(h_alpha, h_alpha + M);
  m->h_L_inv.assign(h_L_inv, h_L_inv + (size_t)M * M);
  // L_inv panels: species s uses rows [c_s, c_s + R_s) and columns
  // [c_s, c_s + M_s); R_s = M_s when everything below the diagonal block is
  // exactly zero (the single-kernel case), else M - c_s.
  std::vector<double> panels;
  m->h_panel_rows.assign(S, 0);
  m->h_panel_off.assign(S, 0);
  for (int s = 0; s < S; s++) {
    const int cs = m->h_offsets[s], Ms = h_counts[s];
    bool below_zero = true;
    for (int r = cs + Ms; r < M && below_zero; r++)
      for (int c = cs; c < cs + Ms; c++)
        if (h_L_inv[(size_t)r * M + c] != 0.0) { below_zero = false; break; }
    const int R = below_zero ? Ms : M - cs;
    m->h_panel_rows[s] = R;
    m->h_panel_off[s] = (long long)panels.size();
    for (int r = 0; r < R; r++)
      for (int c = 0; c < Ms; c++)
        panels.push_back(h_L_inv[(size_t)(cs + r) * M + cs + c]);
  }
  if ((rc = m->Lp.ensure(sizeof(double) * (panels.size() + 1)))) return rc;
  if (!panels.empty())
    FGB_CUDA(cudaMemcpy(m->Lp.p, panels.data(), sizeof(double) * panels.size(),
                        cudaMemcpyHostToDevice));
  m->solved = true;
  return FGB_OK;
}

// A model with the same weights and its own device workspace.
fgb_model_s *model_replicate(const fgb_model_s *src, int &rc) {
  fgb_model_s *m = new fgb_model_s();
  m->b2 = src->b2;
  m->sigma = src->sigma;
  m->power = src->power;
  rc = fgb_model_set(m, src->h_counts.data(), src->h_desc.data(),
                     src->solved ? src->h_alpha.data() : nullptr,
                     src->solved ? src->h_L_inv.data() : nullptr);
  if (rc) { delete m; return nullptr; }
  if (src->has_rinv) {
    if ((rc = m->RinvT.ensure(src->RinvT.bytes))) { delete m; return nullptr; }
    cudaError_t e = cudaMemcpy(m->RinvT.p, src->RinvT.p, src->RinvT.bytes,
                               cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
      rc = cuda_status(e, "model_replicate");
      delete m;
      return nullptr;
    }
    m->has_rinv = true;
  }
  return m;
}

// ------------------------------------------------------------- predict
int predict_impl(fgb_model_s *m, int n_struc, const int *h_atom_offsets,
                 const double *h_cells, const double *d_positions,
                 const int *d_species, double cutoff, int want, int precision,
                 double *d_energy, double *d_forces, double *d_stress,
                 double *d_local_var, cudaStream_t st, const FixedPlan *fixed,
                 const PredictHostIO *hio) {
  if (!m->solved) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  if (precision != FGB_PREC_FP64 && precision != FGB_PREC_MIXED) {
    set_error("fgb_predict: unknown precision %d", precision);
    return FGB_EINVAL;
  }
  int rc;
  if (fixed && (m->nl.n_struc != n_struc || m->nl.n_atoms !=
                    h_atom_offsets[n_struc] ||
                (int)fixed->counts.size() != m->b2.n_species)) {
    set_error("fgb_predict: fixed call on a different batch than the last");
    return FGB_EINVAL;
  }
  {
    StageTimer _pt(kStNeighbors, st);
    rc = fixed ? nlist_rebuild_fixed(&m->nl, d_positions, cutoff,
                                     fixed->pair_cap, st)
               : nlist_build(&m->nl, n_struc, h_atom_offsets, h_cells,
                             d_positions, cutoff, st, false);
    _pt.set_launches(m->nl.last_launches);
    if (rc) return rc;
  }
  const B2Params &p = m->b2;
  const int N = m->nl.n_atoms;
  const long long P = m->nl.n_pairs;
  const bool mixed = precision == FGB_PREC_MIXED;
  // the bounded tensor-core waits report into ws.ozerr, read at the end (a
  // fixed call's caller clears and reads it)
  if ((rc = m->ws.ozerr.ensure(sizeof(int)))) return rc;
  if (!fixed && mixed)
    FGB_CUDA(cudaMemsetAsync(m->ws.ozerr.p, 0, sizeof(int), st));
  const bool want_e = want & FGB_WANT_ENERGY, want_f = want & FGB_WANT_FORCES,
             want_s = want & FGB_WANT_STRESS, want_v = want & FGB_WANT_LOCAL_VAR;
  const bool want_grad = want_f || want_s;
  // forces and local variances go straight to the caller's buffers when
  // given (no device-to-device copy at the end)
  const bool f_direct = want_f && d_forces, v_direct = want_v && d_local_var;
  if ((rc = m->ws.A.ensure(sizeof(float) * ((size_t)N * p.n_A + 2))) ||
      (rc = m->ws.B2.ensure(sizeof(double) * ((size_t)N * p.n_d + 1))) ||
      (rc = m->ws.norms.ensure(sizeof(double) * (N + 1))) ||
      (rc = m->ws.e_atom.ensure(sizeof(double) * (N + 1))) ||
      (rc = m->ws.var.ensure(sizeof(double) * (N + 1))) ||
      (rc = m->ws.rowmax.ensure(sizeof(double) * (N + 1))) ||
      (rc = m->ws.volume.ensure(sizeof(double) * (n_struc + 1))) ||
      (rc = m->ws.atom_off.ensure(sizeof(int) * (n_struc + 1))))
    return rc;
  if (want_grad &&
      ((rc = m->ws.gB2.ensure(sizeof(double) * ((size_t)N * p.n_d + 1))) ||
       (rc = m->ws.pair_grad.ensure(sizeof(double3) * (P + 1))) ||
       (rc = m->ws.forces.ensure(sizeof(double) * (3 * (size_t)N + 1))) ||
       (rc = m->ws.virial.ensure(sizeof(double) * (6 * (size_t)N + 1)))))
    return rc;
  if (!fixed) {   // a fixed call keeps the last call's (same cells, atoms)
    FGB_CUDA(cudaMemcpyAsync(m->ws.volume.p, m->nl.h_volume.data(),
                             sizeof(double) * n_struc, cudaMemcpyHostToDevice,
                             st));
    FGB_CUDA(cudaMemcpyAsync(m->ws.atom_off.p, h_atom_offsets,
                             sizeof(int) * (n_struc + 1),
                             cudaMemcpyHostToDevice, st));
  }
  if (N > 0) {
    FGB_CUDA(cudaMemsetAsync(m->ws.e_atom.p, 0, sizeof(double) * N, st));
    FGB_CUDA(cudaMemsetAsync(v_direct ? d_local_var : m->ws.var.as<double>(),
                             0, sizeof(double) * N, st));
  }
  // the fold guard is known before the descriptor: models with large folded
  // coefficients take the descriptor, force product and adjoint at FP64
  // level (a fixed call reuses the full call's fold)
  if (mixed && !fixed && (rc = prepare_mixed(m, st))) return rc;
  // FP32 adjoint (and FP32 pair gradients and force sums) in the mixed
  // path (dE/dB2 written in FP32 by the mapped gradient), unless the fold
  // guard asked for FP64-level forces or the power has no folded form
  // (FP64 kernel stage); its A is written in FP32 by the forward
  const bool adj32 = mixed && !m->force_f64 &&
                     (m->power == 2.0 || m->power == 1.0);
  if (!adj32 &&
      (rc = m->ws.A.ensure(sizeof(double) * ((size_t)N * p.n_A + 1))))
    return rc;
  // species counts: queued before the descriptor and waited for after it,
  // so the GPU runs the descriptor while the host waits (on device species)
  std::vector<int> counts;
  bool counts_pending = false;
  if (fixed) {
    counts = fixed->counts;
  } else {
    StageTimer _pt(kStSpeciesPerm, st, 3);
    if ((rc = species_permutation_start(p.n_species, m->ws, d_species, N,
                                        counts, st,
                                        hio ? hio->species : nullptr,
                                        counts_pending)))
      return rc;
  }
  {
    StageTimer _pt(kStB2Forward, st);
    // mixed precision: the descriptor in double-float (about 46 bits)
    if ((rc = launch_b2_forward(p, &m->nl, d_species,
                                adj32 ? nullptr : m->ws.A.as<double>(),
                                m->ws.B2.as<double>(), m->ws.norms.as<double>(),
                                st, mixed && !m->force_f64,
                                mixed ? m->ws.rowmax.as<double>() : nullptr,
                                adj32 ? m->ws.A.as<float>() : nullptr)))
      return rc;
  }
  if (counts_pending &&
      (rc = species_permutation_finish(p.n_species, m->ws, counts)))
    return rc;
  if (!fixed) m->last_species_counts = counts;
  // dE/dB2 rows: the kernel stages write every row of a species with sparse
  // environments; rows of species without any stay zero
  if (want_grad && N > 0) {
    bool zero = false;
    for (int s = 0; s < p.n_species; s++)
      zero |= counts[s] > 0 && m->h_counts[s] == 0;
    if (zero)
      FGB_CUDA(cudaMemsetAsync(m->ws.gB2.p, 0,
                               sizeof(double) * (size_t)N * p.n_d, st));
  }
  if (precision == FGB_PREC_MIXED) {
    if ((rc = kernel_stage_mixed(m, N, counts, want_grad, want_v,
                                 m->ws.e_atom.as<double>(),
                                 m->ws.gB2.as<double>(),
                                 v_direct ? d_local_var : m->ws.var.as<double>(),
                                 st, fixed != nullptr)))
      return rc;
  } else {
    if ((rc = kernel_stage_fp64(m, N, counts, want_grad, want_v,
                                m->ws.e_atom.as<double>(),
                                m->ws.gB2.as<double>(),
                                v_direct ? d_local_var : m->ws.var.as<double>(),
                                st)))
      return rc;
  }
  if (want_grad) {
    {
      StageTimer _pt(kStB2Adjoint, st);
      if ((rc = launch_b2_adjoint(p, &m->nl, d_species,
                                  adj32 ? nullptr : m->ws.A.as<double>(),
                                  m->ws.gB2.p, m->ws.pair_grad.p, st, adj32,
                                  adj32 ? m->ws.A.as<float>() : nullptr)))
        return rc;
    }
    {
      StageTimer _pt(kStForces, st);
      if ((rc = launch_forces(&m->nl, m->ws.pair_grad.p, adj32,
                              f_direct ? d_forces : m->ws.forces.as<double>(),
                              m->ws.virial.as<double>(), st)))
        return rc;
    }
  }
  if ((want_e && d_energy) || (want_s && d_stress)) {
    StageTimer _ptr(kStStructReduce, st);
    if ((rc = launch_struct_reduce(
             n_struc, m->ws.atom_off.as<int>(), m->ws.volume.as<double>(),
             m->ws.e_atom.as<double>(),
             want_grad ? m->ws.virial.as<double>() : nullptr,
             want_e ? d_energy : nullptr, want_s ? d_stress : nullptr, st)))
      return rc;
  }
  if (fixed) return FGB_OK;
  if (hio) {   // results to the host ahead of the one synchronisation below
    if (hio->energy && want_e)
      FGB_CUDA(cudaMemcpyAsync(hio->energy, d_energy, sizeof(double) * n_struc,
                               cudaMemcpyDeviceToHost, st));
    if (hio->forces && want_f && N > 0)
      FGB_CUDA(cudaMemcpyAsync(hio->forces, d_forces, sizeof(double) * 3 * N,
                               cudaMemcpyDeviceToHost, st));
    if (hio->stress && want_s)
      FGB_CUDA(cudaMemcpyAsync(hio->stress, d_stress, sizeof(double) * 6 * n_struc,
                               cudaMemcpyDeviceToHost, st));
    if (hio->local_var && want_v && N > 0)
      FGB_CUDA(cudaMemcpyAsync(hio->local_var, d_local_var,
                               sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  }
  // deferred checks: neighbour-list consistency, tensor-core waits
  int h[5] = {0, 0, 0, 0, 0};
  FGB_CUDA(cudaMemcpyAsync(h, m->nl.flag.p, sizeof(int) * 4,
                           cudaMemcpyDeviceToHost, st));
  if (mixed)
    FGB_CUDA(cudaMemcpyAsync(h + 4, m->ws.ozerr.p, sizeof(int),
                             cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  rc = nlist_finish(&m->nl, h);
  if (rc == kNlistRetry) {
    // an atom had more pairs than its single-pass slots: the whole call
    // again, its list built with a count pass
    m->nl.count_pass = true;
    rc = predict_impl(m, n_struc, h_atom_offsets, h_cells, d_positions,
                      d_species, cutoff, want, precision, d_energy, d_forces,
                      d_stress, d_local_var, st, nullptr, hio);
    m->nl.count_pass = false;
    return rc;
  }
  if (rc) return rc;
  if (h[4]) {
    set_error("tensor-core stage: a bounded device wait ran out");
    return FGB_ETIMEOUT;
  }
  return FGB_OK;
}

extern "C" int fgb_predict(fgb_model_t m, int n_struc, const int *h_atom_offsets,
                           const double *h_cells, const double *d_positions,
                           const int *d_species, double cutoff, int want,
                           int precision, double *d_energy, double *d_forces,
                           double *d_stress, double *d_local_var, void *stream) {
  if (!m) { set_error("fgb_predict: null model"); return FGB_EINVAL; }
  return predict_impl(m, n_struc, h_atom_offsets, h_cells, d_positions,
                      d_species, cutoff, want, precision, d_energy, d_forces,
                      d_stress, d_local_var, (cudaStream_t)stream);
}

extern "C" int fgb_predict_host(fgb_model_t m, int n_struc,
                                const int *h_atom_offsets, const double *h_cells,
                                const double *h_positions, const int *h_species,
                                double cutoff, int want, int precision,
                                double *h_energy, double *h_forces,
                                double *h_stress, double *h_local_var,
                                void *stream) {
  if (!m || n_struc <= 0 || !h_atom_offsets) {
    set_error("fgb_predict_host: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N = h_atom_offsets[n_struc];
  int rc;
  if ((rc = m->io.pos.ensure(sizeof(double) * (3 * (size_t)N + 1))) ||
      (rc = m->io.species.ensure(sizeof(int) * (N + 1))) ||
      (rc = m->io.energy.ensure(sizeof(double) * (n_struc + 1))) ||
      (rc = m->io.forces.ensure(sizeof(double) * (3 * (size_t)N + 1))) ||
      (rc = m->io.stress.ensure(sizeof(double) * (6 * (size_t)n_struc + 1))) ||
      (rc = m->io.var.ensure(sizeof(double) * (N + 1))))
    return rc;
  if (N > 0) {
    FGB_CUDA(cudaMemcpyAsync(m->io.pos.p, h_positions, sizeof(double) * 3 * N,
                             cudaMemcpyHostToDevice, st));
    FGB_CUDA(cudaMemcpyAsync(m->io.species.p, h_species, sizeof(int) * N,
                             cudaMemcpyHostToDevice, st));
  }
  // species counted on the host (no read-back) and results copied back
  // before the prediction's final synchronisation
  PredictHostIO hio;
  hio.species = h_species;
  hio.energy = h_energy;
  hio.forces = h_forces;
  hio.stress = h_stress;
  hio.local_var = h_local_var;
  return predict_impl(m, n_struc, h_atom_offsets, h_cells,
                      m->io.pos.as<double>(), m->io.species.as<int>(), cutoff,
                      want, precision, m->io.energy.as<double>(),
                      m->io.forces.as<double>(), m->io.stress.as<double>(),
                      m->io.var.as<double>(), st, nullptr, &hio);
}

extern "C" int fgb_model_set_R_inv(fgb_model_t m, const double *h_R_inv) {
  if (!m || !h_R_inv) { set_error("fgb_model_set_R_inv: invalid arguments"); return FGB_EINVAL; }
  const int M = m->M;
  std::vector<double> t((size_t)M * M);
  for (int r = 0; r < M; r++)
    for (int c = 0; c < M; c++) t[(size_t)c * M + r] = h_R_inv[(size_t)r * M + c];
  int rc;
  if ((rc = m->RinvT.ensure(sizeof(double) * ((size_t)M * M + 1)))) return rc;
  if (M > 0)
    FGB_CUDA(cudaMemcpy(m->RinvT.p, t.data(), sizeof(double) * (size_t)M * M,
                        cudaMemcpyHostToDevice));
  m->has_rinv = true;
  return FGB_OK;
}

extern "C" int fgb_predict_sor(fgb_model_t m, fgb_nlist_t nl,
                               const int *d_species, double *d_mean_efs,
                               double *d_variance_efs, void *stream) {
  if (!m || !nl || !d_mean_efs || !d_variance_efs) {
    set_error("fgb_predict_sor: invalid arguments");
    return FGB_EINVAL;
  }
  if (!m->solved || !m->has_rinv) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N = nl->n_atoms, M = m->M;
  const long long ncol = 1 + 3LL * N + 6;
  if (ncol > (1LL << 30)) { set_error("fgb_predict_sor: structure too large"); return FGB_EINVAL; }
  int rc;
  DevBuf kern, kt, part;
  const int ntiles = ceil_div(M, BN);
  if ((rc = kern.ensure(sizeof(double) * ((size_t)M * ncol + 1))) ||
      (rc = kt.ensure(sizeof(double) * ((size_t)M * ncol + 1))) ||
      (rc = part.ensure(sizeof(double) * ((size_t)ncol * ntiles + 1))))
    return rc;
  if ((rc = envs_struc_impl(m->b2, m->sigma, m->power, m->h_counts.data(),
                            m->Sraw.as<double>(), nl, d_species,
                            kern.as<double>(), m->ws, st)))
    return rc;
  if (M == 0) {
    FGB_CUDA(cudaMemsetAsync(d_mean_efs, 0, sizeof(double) * ncol, st));
    FGB_CUDA(cudaMemsetAsync(d_variance_efs, 0, sizeof(double) * ncol, st));
    return FGB_OK;
  }
  k_transpose_rm<<<ceil_div((long long)M * ncol, 256), 256, 0, st>>>(
      M, (int)ncol, kern.as<double>(), kt.as<double>());
  FGB_LAUNCH_CHECK("k_transpose_rm");
  k_kt_alpha<<<ceil_div(ncol, 128), 128, 0, st>>>(M, ncol, kt.as<double>(),
                                                  m->alpha.as<double>(),
                                                  d_mean_efs);
  FGB_LAUNCH_CHECK("k_kt_alpha");
  // V = K^T R_inv = K^T (R_inv^T)^T: the triangular NT GEMM with the lower
  // factor R_inv^T; variance_efs = row sums of V^2 (sparse_gp.cpp:689-691).
  dim3 g(ntiles, ceil_div(ncol, BM));
  k_variance_gemm<<<g, GT, 0, st>>>((int)ncol, M, M, kt.as<double>(),
                                    m->RinvT.as<double>(), part.as<double>(),
                                    ntiles);
  FGB_LAUNCH_CHECK("k_variance_gemm");
  k_sum_parts<<<ceil_div(ncol, 128), 128, 0, st>>>((int)ncol, ntiles,
                                                   part.as<double>(),
                                                   d_variance_efs);
  FGB_LAUNCH_CHECK("k_sum_parts");
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}

extern "C" int fgb_predict_dtc(fgb_model_t m, fgb_nlist_t nl,
                               const int *d_species, double *d_mean_efs,
                               double *d_variance_efs, void *stream) {
  if (!m || !nl || !d_mean_efs || !d_variance_efs) {
    set_error("fgb_predict_dtc: invalid arguments");
    return FGB_EINVAL;
  }
  if (!m->solved || !m->has_rinv) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N = nl->n_atoms, M = m->M;
  const long long ncol = 1 + 3LL * N + 6;
  if (ncol > (1LL << 30)) { set_error("fgb_predict_dtc: structure too large"); return FGB_EINVAL; }
  int rc;
  if (!m->lfull_ready && M > 0) {
    if ((rc = m->Lfull.ensure(sizeof(double) * (size_t)M * M))) return rc;
    FGB_CUDA(cudaMemcpy(m->Lfull.p, m->h_L_inv.data(),
                        sizeof(double) * (size_t)M * M, cudaMemcpyHostToDevice));
    m->lfull_ready = true;
  }
  DevBuf kern, kt, part, kself, q;
  const int ntiles = ceil_div(M, BN);
  if ((rc = kern.ensure(sizeof(double) * ((size_t)M * ncol + 1))) ||
      (rc = kt.ensure(sizeof(double) * ((size_t)M * ncol + 1))) ||
      (rc = part.ensure(sizeof(double) * ((size_t)ncol * ntiles + 1))) ||
      (rc = kself.ensure(sizeof(double) * ncol)) ||
      (rc = q.ensure(sizeof(double) * ncol)))
    return rc;
  if ((rc = envs_struc_impl(m->b2, m->sigma, m->power, m->h_counts.data(),
                            m->Sraw.as<double>(), nl, d_species,
                            kern.as<double>(), m->ws, st)))
    return rc;
  // K_self from the descriptors and stored gradients envs_struc left in the
  // workspace (envs_struc_impl computes them only when M > 0 and N > 0)
  if ((rc = self_kernel_impl(m->b2, m->sigma, m->power, nl, d_species,
                             kself.as<double>(), m->ws, st, M > 0)))
    return rc;
  if (M == 0) {
    FGB_CUDA(cudaMemsetAsync(d_mean_efs, 0, sizeof(double) * ncol, st));
    FGB_CUDA(cudaMemcpyAsync(d_variance_efs, kself.p, sizeof(double) * ncol,
                             cudaMemcpyDeviceToDevice, st));
    FGB_CUDA(cudaStreamSynchronize(st));
    return FGB_OK;
  }
  k_transpose_rm<<<ceil_div((long long)M * ncol, 256), 256, 0, st>>>(
      M, (int)ncol, kern.as<double>(), kt.as<double>());
  FGB_LAUNCH_CHECK("k_transpose_rm");
  k_kt_alpha<<<ceil_div(ncol, 128), 128, 0, st>>>(M, ncol, kt.as<double>(),
                                                  m->alpha.as<double>(),
                                                  d_mean_efs);
  FGB_LAUNCH_CHECK("k_kt_alpha");
  dim3 g(ntiles, ceil_div(ncol, BM));
  // diag(K^T Kuu^-1 K) = column sums of (L_inv K)^2 (sparse_gp.cpp:723)
  k_variance_gemm<<<g, GT, 0, st>>>((int)ncol, M, M, kt.as<double>(),
                                    m->Lfull.as<double>(), part.as<double>(),
                                    ntiles);
  FGB_LAUNCH_CHECK("k_variance_gemm");
  k_sum_parts<<<ceil_div(ncol, 128), 128, 0, st>>>((int)ncol, ntiles,
                                                   part.as<double>(),
                                                   q.as<double>());
  FGB_LAUNCH_CHECK("k_sum_parts");
  // diag(K^T Sigma K) = column sums of (R_inv^T K)^2 (sparse_gp.cpp:724)
  k_variance_gemm<<<g, GT, 0, st>>>((int)ncol, M, M, kt.as<double>(),
                                    m->RinvT.as<double>(), part.as<double>(),
                                    ntiles);
  FGB_LAUNCH_CHECK("k_variance_gemm");
  k_sum_parts<<<ceil_div(ncol, 128), 128, 0, st>>>((int)ncol, ntiles,
                                                   part.as<double>(),
                                                   d_variance_efs);
  FGB_LAUNCH_CHECK("k_sum_parts");
  k_dtc_combine<<<ceil_div(ncol, 256), 256, 0, st>>>(
      ncol, kself.as<double>(), q.as<double>(), d_variance_efs);
  FGB_LAUNCH_CHECK("k_dtc_combine");
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}
