// C-ABI plumbing for libflaregb: error state, device buffers, host cell
// algebra, deterministic scans, B2 settings.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "fgb_internal.h"

namespace fgb {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char *where) {
  set_error("CUDA error %d (%s) at %s", (int)e, cudaGetErrorString(e), where);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return FGB_ENOMEM;
  }
  return FGB_ECUDA;
}

static std::atomic<unsigned long long> g_allocations{0};

unsigned long long devbuf_allocations() { return g_allocations.load(); }

int DevBuf::ensure(size_t n) {
  if (n == 0) n = 16;
  if (n <= bytes) return FGB_OK;
  g_allocations.fetch_add(1);
  release();
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    set_error("device allocation of %zu bytes failed (%s)", n,
              cudaGetErrorString(e));
    return FGB_ENOMEM;
  }
  bytes = n;
  return FGB_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

// Canonical 3x3 algebra (same formulas and order as the oracle's):
// inverse by cofactors over the first-row determinant; products summed
// k = 0, 1, 2 left to right.  Compiled with -ffp-contract=off.
static void inv3(const double *a, double *out) {
  double c00 = a[4] * a[8] - a[5] * a[7];
  double c01 = a[5] * a[6] - a[3] * a[8];
  double c02 = a[3] * a[7] - a[4] * a[6];
  double c10 = a[2] * a[7] - a[1] * a[8];
  double c11 = a[0] * a[8] - a[2] * a[6];
  double c12 = a[1] * a[6] - a[0] * a[7];
  double c20 = a[1] * a[5] - a[2] * a[4];
  double c21 = a[2] * a[3] - a[0] * a[5];
  double c22 = a[0] * a[4] - a[1] * a[3];
  double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  out[0] = c00 / det; out[1] = c10 / det; out[2] = c20 / det;
  out[3] = c01 / det; out[4] = c11 / det; out[5] = c21 / det;
  out[6] = c02 / det; out[7] = c12 / det; out[8] = c22 / det;
}

static void mul3(const double *a, const double *b, double *c) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      c[3 * i + j] = (a[3 * i + 0] * b[0 + j] + a[3 * i + 1] * b[3 + j]) +
                     a[3 * i + 2] * b[6 + j];
}

// structure.cpp:14-21 (cell matrices, volume) and :135-165 (single sweep).
void cell_setup(const double *cell, double *ct, double *cti, double *cd,
                double *cdi, double *volume, double *single_sweep_cutoff) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) ct[3 * i + j] = cell[3 * j + i];
  inv3(ct, cti);
  mul3(cell, ct, cd);
  inv3(cd, cdi);
  double det = cell[0] * (cell[4] * cell[8] - cell[5] * cell[7]) +
               cell[1] * (cell[5] * cell[6] - cell[3] * cell[8]) +
               cell[2] * (cell[3] * cell[7] - cell[4] * cell[6]);
  *volume = std::fabs(det);
  const double *v1 = cell, *v2 = cell + 3, *v3 = cell + 6;
  double ab = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
  double ac = v1[0] * v3[0] + v1[1] * v3[1] + v1[2] * v3[2];
  double bc = v2[0] * v3[0] + v2[1] * v3[1] + v2[2] * v3[2];
  double a = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  double b = std::sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  double c = std::sqrt(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]);
  double m[6];
  m[0] = a * std::sqrt(1 - std::pow(ab / (a * b), 2));
  m[1] = b * std::sqrt(1 - std::pow(ab / (a * b), 2));
  m[2] = a * std::sqrt(1 - std::pow(ac / (a * c), 2));
  m[3] = c * std::sqrt(1 - std::pow(ac / (a * c), 2));
  m[4] = b * std::sqrt(1 - std::pow(bc / (b * c), 2));
  m[5] = c * std::sqrt(1 - std::pow(bc / (b * c), 2));
  double s = m[0];
  for (int i = 0; i < 6; i++)
    if (m[i] < s) s = m[i];
  *single_sweep_cutoff = s;
}

// ------------------------------------------------------------------ scans
// Two-level exclusive scan: blocks of 1024 elements scanned in shared
// memory, block totals scanned by one block (<= 4096 blocks), then added.
namespace {

constexpr int kScanBlock = 1024;

template <typename TI, typename TO>
__global__ void k_scan_block(const TI *__restrict__ in, TO *__restrict__ out,
                             int n, TO *__restrict__ block_sums) {
  __shared__ TO s[kScanBlock];
  int base = blockIdx.x * kScanBlock;
  int t = threadIdx.x;
  TO v = (base + t < n) ? (TO)in[base + t] : (TO)0;
  s[t] = v;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    TO add = (t >= off) ? s[t - off] : (TO)0;
    __syncthreads();
    s[t] += add;
    __syncthreads();
  }
  if (base + t < n) out[base + t] = s[t] - v;
  if (t == kScanBlock - 1 && block_sums) block_sums[blockIdx.x] = s[t];
}

template <typename TO>
__global__ void k_scan_sums(TO *__restrict__ sums, int nb, TO *__restrict__ total) {
  // single block of 1024 threads, up to 4 elements each
  __shared__ TO s[kScanBlock];
  int t = threadIdx.x;
  TO loc[4];
  TO acc = 0;
  for (int k = 0; k < 4; k++) {
    int idx = t * 4 + k;
    loc[k] = idx < nb ? sums[idx] : (TO)0;
    acc += loc[k];
  }
  s[t] = acc;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    TO add = (t >= off) ? s[t - off] : (TO)0;
    __syncthreads();
    s[t] += add;
    __syncthreads();
  }
  TO run = s[t] - acc;
  for (int k = 0; k < 4; k++) {
    int idx = t * 4 + k;
    if (idx < nb) sums[idx] = run;
    run += loc[k];
  }
  if (t == kScanBlock - 1 && total) *total = s[t];
}

template <typename TO>
__global__ void k_scan_add(TO *__restrict__ out, int n,
                           const TO *__restrict__ sums) {
  int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

template <typename TI, typename TO>
int scan_impl(const TI *d_in, TO *d_out, int n, TO *d_total, DevBuf &tmp,
              cudaStream_t st) {
  if (n <= 0) {
    if (d_total) FGB_CUDA(cudaMemsetAsync(d_total, 0, sizeof(TO), st));
    return FGB_OK;
  }
  int nb = (n + kScanBlock - 1) / kScanBlock;
  if (nb > 4 * kScanBlock) {
    set_error("scan: %d elements exceed the two-level scan limit", n);
    return FGB_EINVAL;
  }
  int rc = tmp.ensure(sizeof(TO) * (nb + 1));
  if (rc) return rc;
  TO *sums = tmp.as<TO>();
  k_scan_block<TI, TO><<<nb, kScanBlock, 0, st>>>(d_in, d_out, n, sums);
  FGB_LAUNCH_CHECK("k_scan_block");
  k_scan_sums<TO><<<1, kScanBlock, 0, st>>>(sums, nb, d_total);
  FGB_LAUNCH_CHECK("k_scan_sums");
  k_scan_add<TO><<<nb, kScanBlock, 0, st>>>(d_out, n, sums);
  FGB_LAUNCH_CHECK("k_scan_add");
  return FGB_OK;
}

// Same scan with caller-provided block-sum storage (no allocation):
// `sums` holds at least ceil(n / 1024) + 1 elements.
template <typename TI, typename TO>
int scan_impl_raw(const TI *d_in, TO *d_out, int n, TO *d_total, TO *sums,
                  cudaStream_t st) {
  if (n <= 0) {
    if (d_total) FGB_CUDA(cudaMemsetAsync(d_total, 0, sizeof(TO), st));
    return FGB_OK;
  }
  int nb = (n + kScanBlock - 1) / kScanBlock;
  if (nb > 4 * kScanBlock) {
    set_error("scan: %d elements exceed the two-level scan limit", n);
    return FGB_EINVAL;
  }
  k_scan_block<TI, TO><<<nb, kScanBlock, 0, st>>>(d_in, d_out, n, sums);
  FGB_LAUNCH_CHECK("k_scan_block");
  k_scan_sums<TO><<<1, kScanBlock, 0, st>>>(sums, nb, d_total);
  FGB_LAUNCH_CHECK("k_scan_sums");
  k_scan_add<TO><<<nb, kScanBlock, 0, st>>>(d_out, n, sums);
  FGB_LAUNCH_CHECK("k_scan_add");
  return FGB_OK;
}

}  // namespace

int scan_int_to_int_raw(const int *d_in, int *d_out, int n, int *d_total,
                        int *d_sums, cudaStream_t st) {
  return scan_impl_raw<int, int>(d_in, d_out, n, d_total, d_sums, st);
}

int scan_int_to_ll_raw(const int *d_in, long long *d_out, int n,
                       long long *d_total, long long *d_sums,
                       cudaStream_t st) {
  return scan_impl_raw<int, long long>(d_in, d_out, n, d_total, d_sums, st);
}

int scan_int_to_int(const int *d_in, int *d_out, int n, int *d_total,
                    DevBuf &tmp, cudaStream_t st) {
  return scan_impl<int, int>(d_in, d_out, n, d_total, tmp, st);
}

int scan_int_to_ll(const int *d_in, long long *d_out, int n,
                   long long *d_total, DevBuf &tmp, cudaStream_t st) {
  return scan_impl<int, long long>(d_in, d_out, n, d_total, tmp, st);
}

}  // namespace fgb

using namespace fgb;

extern "C" const char *fgb_last_error(void) { return g_err; }

extern "C" int fgb_version(void) { return 1; }

extern "C" int fgb_b2_create(fgb_b2_t *out, int radial_basis,
                             int cutoff_function, const double *radial_hyps,
                             int n_radial_hyps, const double *cutoff_hyps,
                             int n_cutoff_hyps, int n_species, int n_max,
                             int l_max, const double *h_cutoffs) {
  if (!out) { set_error("fgb_b2_create: null output"); return FGB_EINVAL; }
  if (radial_basis < FGB_RADIAL_CHEBYSHEV || radial_basis > FGB_RADIAL_FOURIER) {
    set_error("fgb_b2_create: unknown radial basis %d", radial_basis);
    return FGB_EINVAL;
  }
  const bool three = radial_basis == FGB_RADIAL_WEIGHTED_CHEBYSHEV ||
                     radial_basis == FGB_RADIAL_EQUISPACED_GAUSSIANS ||
                     radial_basis == FGB_RADIAL_WEIGHTED_POSITIVE_CHEBYSHEV ||
                     radial_basis == FGB_RADIAL_FOURIER;
  if (three && (n_radial_hyps < 3 || !radial_hyps)) {
    set_error("fgb_b2_create: radial basis %d needs three radial_hyps",
              radial_basis);
    return FGB_EINVAL;
  }
  if (cutoff_function < FGB_CUTOFF_QUADRATIC ||
      cutoff_function > FGB_CUTOFF_POWER) {
    set_error("fgb_b2_create: unknown cutoff function %d", cutoff_function);
    return FGB_EINVAL;
  }
  if ((cutoff_function == FGB_CUTOFF_POLYNOMIAL ||
       cutoff_function == FGB_CUTOFF_POWER) && n_cutoff_hyps < 1) {
    set_error("fgb_b2_create: cutoff function needs one hyperparameter");
    return FGB_EINVAL;
  }
  if (n_radial_hyps < 2 || !radial_hyps) {
    set_error("fgb_b2_create: radial_hyps needs [r1, r2]");
    return FGB_EINVAL;
  }
  if (n_species < 1 || n_species > kMaxSpecies || n_max < 1 ||
      n_max > kMaxNmax || l_max < 0 || l_max > kMaxL) {
    set_error("fgb_b2_create: settings out of range (species <= %d, "
              "n_max <= %d, l_max <= %d)", kMaxSpecies, kMaxNmax, kMaxL);
    return FGB_EINVAL;
  }
  fgb_b2_s *b = new fgb_b2_s();
  B2Params &p = b->p;
  std::memset(&p, 0, sizeof(p));
  p.radial_basis = radial_basis;
  p.cutoff_function = cutoff_function;
  p.n_species = n_species;
  p.n_max = n_max;
  p.l_max = l_max;
  p.n_harm = (l_max + 1) * (l_max + 1);
  p.n_rad = n_species * n_max;
  p.n_A = p.n_rad * p.n_harm;
  p.n_d = p.n_rad * (p.n_rad + 1) / 2 * (l_max + 1);
  p.r1 = radial_hyps[0];
  p.radial_hyp2 = n_radial_hyps > 2 ? radial_hyps[2] : 0.0;
  p.n_cutoff_hyps = n_cutoff_hyps < 4 ? n_cutoff_hyps : 4;
  for (int k = 0; k < p.n_cutoff_hyps; k++) p.cutoff_hyps[k] = cutoff_hyps[k];
  p.max_cutoff = 0;
  for (int a = 0; a < n_species; a++)
    for (int c = 0; c < n_species; c++) {
      double v = h_cutoffs ? h_cutoffs[a * n_species + c] : radial_hyps[1];
      p.cutoffs[a * kMaxSpecies + c] = v;
      if (v > p.max_cutoff) p.max_cutoff = v;
    }
  *out = b;
  return FGB_OK;
}

extern "C" int fgb_b2_destroy(fgb_b2_t b2) {
  delete b2;
  return FGB_OK;
}

extern "C" int fgb_b2_size(fgb_b2_t b2, int *n_descriptors,
                           int *n_single_bond) {
  if (!b2) { set_error("fgb_b2_size: null handle"); return FGB_EINVAL; }
  if (n_descriptors) *n_descriptors = b2->p.n_d;
  if (n_single_bond) *n_single_bond = b2->p.n_A;
  return FGB_OK;
}
