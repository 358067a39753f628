// Shared device-side definitions for libflaregb (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "flaregb.h"

namespace fgb {

constexpr int kMaxL = 10;                      // y_grad.cpp supports l <= 10
constexpr int kMaxHarm = (kMaxL + 1) * (kMaxL + 1);
constexpr int kMaxNmax = 16;
constexpr int kMaxSpecies = 8;
constexpr double kPi = 3.14159265358979323846;
constexpr double kEmptyThresh = 1e-8;          // normalized_dot_product.cpp:50

// Row sums of GEMM partial slots (part[m * nslots + t]) by kRowLanes
// consecutive lanes per row: lane q adds slots q, q + kRowLanes, ... and a
// fixed butterfly joins the lanes (coalesced slot reads; launch
// rows x kRowLanes threads in blocks of whole groups).  Every lane of the
// group returns the sum.
constexpr int kRowLanes = 4;
__device__ __forceinline__ double row_slots_sum(const double *__restrict__ part,
                                                long long m, int nslots,
                                                int q) {
  double s = 0.0;
  for (int t = q; t < nslots; t += kRowLanes) s += part[m * nslots + t];
  const unsigned gmask = ((1u << kRowLanes) - 1u)
                         << ((threadIdx.x & 31) & ~(kRowLanes - 1));
#pragma unroll
  for (int off = kRowLanes / 2; off > 0; off >>= 1)
    s += __shfl_xor_sync(gmask, s, off);
  return s;
}

// Error state shared by the C-ABI (defined in capi.cu).
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *where);

#define FGB_CUDA(call)                                        \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::fgb::cuda_status(e_, #call); \
  } while (0)

#define FGB_LAUNCH_CHECK(name)                                      \
  do {                                                              \
    cudaError_t e_ = cudaGetLastError();                            \
    if (e_ != cudaSuccess) return ::fgb::cuda_status(e_, name);     \
  } while (0)

// Descriptor settings in constant-friendly POD form.
struct B2Params {
  int radial_basis;      // FGB_RADIAL_*
  int cutoff_function;   // FGB_CUTOFF_*
  int n_species, n_max, l_max;
  int n_harm, n_rad, n_A, n_d;
  double r1;             // radial_hyps[0]
  double radial_hyp2;    // radial_hyps[2] (0 when absent)
  double cutoff_hyps[4];
  int n_cutoff_hyps;
  double cutoffs[kMaxSpecies * kMaxSpecies];   // per species pair
  double max_cutoff;
};

// Spherical-harmonic normalisation K_lm = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!),
// times sqrt2 for m > 0, indexed [l * (kMaxL + 1) + m] (double-precision
// values of the formula, evaluated once and written out), as FP64, as FP32
// (nearest) and as the FP32 remainder K - (double)(float)K, so that FP32 and
// double-float evaluations read their constants without conversions.
#define FGB_YLM_NORM(X) \
  X(0.28209479177387814) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0)  /* l = 0 */ \
  X(0.4886025119029199) X(0.48860251190292) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0)  /* l = 1 */ \
  X(0.6307831305050401) X(0.3641828101973597) X(0.18209140509867985) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0)  /* l = 2 */ \
  X(0.7463526651802308) X(0.3046971996429772) X(0.09635371475468515) X(0.03933623932844291) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0)  /* l = 3 */ \
  X(0.8462843753216345) X(0.2676186174229157) X(0.063078313050504) X(0.016858388283618388) X(0.005960340337611203) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0)  /* l = 4 */ \
  X(0.9356025796273888) X(0.2415715473043717) X(0.045652731285460234) X(0.009318824751147628) X(0.002196468058075176) X(0.0006945841871324552) X(0.0) X(0.0) X(0.0) X(0.0) X(0.0)  /* l = 5 */ \
  X(1.0171072362820548) X(0.22195099524523101) X(0.03509353369580661) X(0.005848922282634434) X(0.0010678622237644956) X(0.00022766899107568565) X(6.57223766418388e-05) X(0.0) X(0.0) X(0.0) X(0.0)  /* l = 6 */ \
  X(1.0925484305920792) X(0.20647224590289676) X(0.028097313806030647) X(0.003973560225074135) X(0.0005990367431114117) X(9.983945718523528e-05) X(1.958012847746254e-05) X(5.233009453691467e-06) X(0.0) X(0.0) X(0.0)  /* l = 7 */ \
  X(1.1631066229203195) X(0.19385110382005324) X(0.023169638523677944) X(0.0028519853513317033) X(0.00036818972564450655) X(5.1058728265780266e-05) X(7.878532816214048e-06) X(1.4384167144950456e-06) X(3.596041786237614e-07) X(0.0) X(0.0)  /* l = 8 */ \
  X(1.2296226898414837) X(0.1833013280774465) X(0.019539987227523183) X(0.0021319873940141734) X(0.00024140003633280337) X(2.8852822971932874e-05) X(3.7248834287122265e-06) X(5.376406125667451e-07) X(9.220460437034855e-08) X(2.1732833668965406e-08) X(0.0)  /* l = 9 */ \
  X(1.2927207364566027) X(0.17431042854448453) X(0.016773028807119526) X(0.001644730792106853) X(0.0001661428994750111) X(1.7512999313514277e-05) X(1.958012847746254e-06) X(2.37443934928654e-07) X(3.231202683854524e-08) X(5.24170291336415e-09) X(1.1720804032140929e-09)  /* l = 10 */
#define FGB_AS_F64(v) v,
#define FGB_AS_F32(v) (float)(v),
#define FGB_AS_F32_LO(v) (float)((v) - (double)(float)(v)),
static __constant__ double c_ylm_norm[(kMaxL + 1) * (kMaxL + 1)] = {
    FGB_YLM_NORM(FGB_AS_F64)};
static __constant__ float c_ylm_norm_f[(kMaxL + 1) * (kMaxL + 1)] = {
    FGB_YLM_NORM(FGB_AS_F32)};
static __constant__ float c_ylm_norm_lo[(kMaxL + 1) * (kMaxL + 1)] = {
    FGB_YLM_NORM(FGB_AS_F32_LO)};

// K_lm in the compute type T (FP64 and FP32 here; the double-float type
// adds its overload in fgb_df.cuh).
__device__ __forceinline__ void ylm_norm(int i, double &k) { k = c_ylm_norm[i]; }
__device__ __forceinline__ void ylm_norm(int i, float &k) { k = c_ylm_norm_f[i]; }

// The double factorials (2m - 1)!! (m = 0 .. kMaxL, exact in FP64 and as
// FP32 head + FP32 tail) and the reciprocals 1/k (k = 1 .. 2 kMaxL + 1,
// FP32 nearest and its FP32 remainder): the associated-Legendre recurrence
// multiplies by these instead of dividing (a double-float or FP32 division
// costs tens of instructions; the FP64 evaluation keeps its divisions).
constexpr int kNumInv = 2 * kMaxL + 2;
__host__ __device__ constexpr double dfact_value(int m) {
  double v = 1.0;
  for (int k = 1; k <= m; k++) v *= (double)(2 * k - 1);
  return v;
}
#define FGB_DFACT(X) X(dfact_value(0)) X(dfact_value(1)) X(dfact_value(2)) \
  X(dfact_value(3)) X(dfact_value(4)) X(dfact_value(5)) X(dfact_value(6)) \
  X(dfact_value(7)) X(dfact_value(8)) X(dfact_value(9)) X(dfact_value(10))
#define FGB_INV(X) X(0.0) X(1.0) X(1.0 / 2) X(1.0 / 3) X(1.0 / 4) X(1.0 / 5) \
  X(1.0 / 6) X(1.0 / 7) X(1.0 / 8) X(1.0 / 9) X(1.0 / 10) X(1.0 / 11) \
  X(1.0 / 12) X(1.0 / 13) X(1.0 / 14) X(1.0 / 15) X(1.0 / 16) X(1.0 / 17) \
  X(1.0 / 18) X(1.0 / 19) X(1.0 / 20) X(1.0 / 21)
static_assert(kMaxL == 10, "the double-factorial and reciprocal tables");
static __constant__ double c_dfact[kMaxL + 1] = {FGB_DFACT(FGB_AS_F64)};
static __constant__ float c_dfact_f[kMaxL + 1] = {FGB_DFACT(FGB_AS_F32)};
static __constant__ float c_dfact_lo[kMaxL + 1] = {FGB_DFACT(FGB_AS_F32_LO)};
static __constant__ float c_inv_f[kNumInv] = {FGB_INV(FGB_AS_F32)};
static __constant__ float c_inv_lo[kNumInv] = {FGB_INV(FGB_AS_F32_LO)};

__device__ __forceinline__ void dfact_const(int m, double &v) { v = c_dfact[m]; }
__device__ __forceinline__ void dfact_const(int m, float &v) { v = c_dfact_f[m]; }
// x / k for a small positive integer k
__device__ __forceinline__ double div_int(double x, int k) {
  return x / (double)k;
}
__device__ __forceinline__ float div_int(float x, int k) {
  return x * c_inv_f[k];
}

// ------------------------------------------------------------ cutoff
// cutoffs.cpp:7-85.  Returns value and derivative w.r.t. r.
template <typename T>
__device__ __forceinline__ void cutoff_eval(const B2Params &p, T r, T rc,
                                            T &fc, T &dfc) {
  if (r > rc) { fc = T(0); dfc = T(0); return; }
  switch (p.cutoff_function) {
    case FGB_CUTOFF_QUADRATIC: {
      T d = r - rc; fc = d * d; dfc = T(2) * d; return;
    }
    case FGB_CUTOFF_HARD: fc = T(1); dfc = T(0); return;
    case FGB_CUTOFF_COSINE: {
      T a = T(kPi) * r / rc;
      fc = T(0.5) * (cos(a) + T(1));
      dfc = -T(kPi) * sin(a) / (T(2) * rc);
      return;
    }
    case FGB_CUTOFF_POLYNOMIAL: {
      int pp = (int)p.cutoff_hyps[0];
      T d = r / rc;
      T c1 = T((pp + 1) * (pp + 2) / 2), c2 = T(pp * (pp + 2)),
        c3 = T(pp * (pp + 1) / 2);
      fc = T(1) - c1 * pow(d, T(pp)) + c2 * pow(d, T(pp + 1)) -
           c3 * pow(d, T(pp + 2));
      T c4 = c1 * pp / rc, c5 = c2 * (pp + 1) / rc, c6 = c3 * (pp + 2) / rc;
      dfc = -c4 * pow(d, T(pp - 1)) + c5 * pow(d, T(pp)) -
            c6 * pow(d, T(pp + 1));
      return;
    }
    case FGB_CUTOFF_POWER: {
      T pw = T(p.cutoff_hyps[0]), rd = rc - r;
      fc = pow(rd, pw); dfc = -pw * pow(rd, pw - T(1));
      return;
    }
  }
  fc = T(0); dfc = T(0);
}

// Conversions between the compute types and FP64 (the double-float type
// adds its own in fgb_df.cuh).
__device__ __forceinline__ double rad_to_double(double x) { return x; }
__device__ __forceinline__ double rad_to_double(float x) { return (double)x; }
template <typename T> __device__ __forceinline__ T rad_from_double(double x);
template <> __device__ __forceinline__ double rad_from_double<double>(double x) {
  return x;
}
template <> __device__ __forceinline__ float rad_from_double<float>(double x) {
  return (float)x;
}

// The radial bases other than Chebyshev (radial.cpp:6-336), in FP64 for
// every compute type: b[n] and db/dr[n] before the cutoff.  r2 is the pair
// cutoff (the descriptor overwrites radial_hyps[1] with it, b2.cpp:352);
// every basis but the Gaussians is zero outside [radial_hyps[0], r2].
static __device__ __noinline__ void radial_basis_f64(const B2Params &p, double r,
                                              double r2, int N, double *b,
                                              double *db) {
  const double r1 = p.r1, h2 = p.radial_hyp2;
  for (int n = 0; n < N; n++) { b[n] = 0.0; db[n] = 0.0; }
  switch (p.radial_basis) {
    case FGB_RADIAL_EQUISPACED_GAUSSIANS: {
      // width radial_hyps[0], centres from radial_hyps[1] to radial_hyps[2]
      const double sigma = r1, first = r2, sep = h2 - r2;
      const double norm = 1.0 / (sigma * sqrt(2.0 * kPi));
      const double s2 = 1.0 / (sigma * sigma), hs2 = s2 / 2.0;
      for (int n = 0; n < N; n++) {
        const double mean = first + (n * sep / (N - 1));
        const double d = r - mean;
        b[n] = norm * exp(-hs2 * d * d);
        db[n] = -s2 * b[n] * d;
      }
      return;
    }
    default: break;
  }
  if (r < r1 || r > r2) return;
  switch (p.radial_basis) {
    case FGB_RADIAL_POSITIVE_CHEBYSHEV: {
      // (1 - T_n)/2; the reference's recurrence runs on the transformed
      // values themselves (radial.cpp:195-206)
      const double c = 1.0 / (r2 - r1), x = (r - r1) * c;
      for (int n = 0; n < N; n++) {
        if (n == 0) { b[n] = 1.0; db[n] = 0.0; continue; }
        double t, dt;
        if (n == 1) { t = x; dt = c; }
        else {
          t = 2.0 * x * b[n - 1] - b[n - 2];
          dt = 2.0 * b[n - 1] * c + 2.0 * x * db[n - 1] - db[n - 2];
        }
        b[n] = 0.5 * (1.0 - t);
        db[n] = -0.5 * dt;
      }
      return;
    }
    case FGB_RADIAL_WEIGHTED_CHEBYSHEV:
    case FGB_RADIAL_WEIGHTED_POSITIVE_CHEBYSHEV: {
      // T_n of the exponentially weighted coordinate (lambda = h2)
      const bool pos = p.radial_basis == FGB_RADIAL_WEIGHTED_POSITIVE_CHEBYSHEV;
      const double c = 1.0 / (r2 - r1), x = (r - r1) * c;
      const double e = exp(-h2 * (x - 1.0)), lc = exp(h2) - 1.0;
      const double xw = 1.0 - 2.0 * (e - 1.0) / lc, dxdr = 2.0 * c * h2 * e / lc;
      double t0 = 1.0, d0 = 0.0, t1 = xw, d1 = 1.0;
      for (int n = 0; n < N; n++) {
        if (n == 0) { b[n] = 1.0; db[n] = 0.0; continue; }
        double t, dt;
        if (n == 1) { t = t1; dt = d1; }
        else {
          t = 2.0 * xw * t1 - t0;
          dt = 2.0 * t1 + 2.0 * xw * d1 - d0;
          t0 = t1; d0 = d1; t1 = t; d1 = dt;
        }
        if (pos) { b[n] = 0.5 * (1.0 - t); db[n] = -0.5 * dt * dxdr; }
        else { b[n] = t; db[n] = dt * dxdr; }
      }
      return;
    }
    case FGB_RADIAL_BESSEL: {
      const double c = r2 - r1, c1 = sqrt(2.0 / c), d = r - r1;
      for (int n = 0; n < N; n++) {
        const double a = kPi * (n + 1) * d, q = a / c, e = c * d * d;
        b[n] = c1 * sin(q) / d;
        db[n] = c1 * (a * cos(q) - c * sin(q)) / e;
      }
      return;
    }
    case FGB_RADIAL_FOURIER_QUARTER:
    case FGB_RADIAL_FOURIER_HALF:
    case FGB_RADIAL_FOURIER: {
      // 1, cos(k w x), sin(k w x), ... with w = pi/2, pi or pi h2
      const double c = 1.0 / (r2 - r1), x = (r - r1) * c;
      const double w = p.radial_basis == FGB_RADIAL_FOURIER_QUARTER
                           ? kPi / 2.0
                           : (p.radial_basis == FGB_RADIAL_FOURIER_HALF
                                  ? kPi : kPi * h2);
      int kc = 1, ks = 1;
      for (int n = 0; n < N; n++) {
        if (n == 0) { b[n] = 1.0; db[n] = 0.0; }
        else if (n % 2 == 1) {
          const double a = w * kc++;
          b[n] = cos(a * x); db[n] = -sin(a * x) * a * c;
        } else {
          const double a = w * ks++;
          b[n] = sin(a * x); db[n] = cos(a * x) * a * c;
        }
      }
      return;
    }
    default: return;
  }
}

// Radial basis on x = (r - r1)/(rc - r1) times the cutoff (radial.cpp:
// 344-379): Chebyshev (radial.cpp:138-169) in the compute type T, the
// other bases through radial_basis_f64.  Writes g[n] and dg/dr[n] (radial
// derivative; Cartesian derivatives are dg/dr * x_k / r); dg may be null.
// NC > 0 fixes n_max at compile time (loops unrolled, arrays of the caller
// kept in registers) and is used for the Chebyshev basis only; NC = 0 reads
// n_max from p.
template <typename T, int NC = 0>
__device__ __forceinline__ void radial_eval(const B2Params &p, T r, T rc,
                                            T *g, T *dg) {
  T fc, dfc;
  cutoff_eval<T>(p, r, rc, fc, dfc);
  const int N = NC > 0 ? NC : p.n_max;
  if (NC == 0 && p.radial_basis != FGB_RADIAL_CHEBYSHEV) {
    double b[kMaxNmax], db[kMaxNmax];
    radial_basis_f64(p, rad_to_double(r), rad_to_double(rc), N, b, db);
    for (int n = 0; n < N; n++) {
      const T bn = rad_from_double<T>(b[n]);
      g[n] = bn * fc;
      if (dg) dg[n] = rad_from_double<T>(db[n]) * fc + bn * dfc;
    }
    return;
  }
  T r1 = T(p.r1);
  if (r < r1 || r > rc) {
#pragma unroll
    for (int n = 0; n < N; n++) {
      g[n] = T(0);
      if (dg) dg[n] = T(0);
    }
    return;
  }
  T c = T(1) / (rc - r1);
  T x = (r - r1) * c;
  T b0 = T(1), db0 = T(0), b1 = x, db1 = c;
#pragma unroll
  for (int n = 0; n < N; n++) {
    T b, db;
    if (n == 0) { b = b0; db = db0; }
    else if (n == 1) { b = b1; db = db1; }
    else {
      b = T(2) * x * b1 - b0;
      db = T(2) * b1 * c + T(2) * x * db1 - db0;
      b0 = b1; db0 = db1; b1 = b; db1 = db;
    }
    g[n] = b * fc;
    if (dg) dg[n] = db * fc + b * dfc;   // dg may be null (values only)
  }
}

// Real spherical harmonics, l-major and m = -l..l (the y_grad.cpp:667
// convention), by the associated-Legendre recurrence on the unit vector.
// Calls fn(idx, Y, Gx, Gy, Gz) once per harmonic (idx = l*l + l + m, visited
// m = L..0, l = m..L) with the Cartesian gradient when Grad (zeros
// otherwise).  LC > 0 fixes l_max at compile time (loops unrolled, the
// recurrence state kept in registers); LC = 0 takes Lrt.
template <typename T, int LC, bool Grad, typename Fn>
__device__ __forceinline__ void ylm_visit(int Lrt, T x, T y, T z, Fn &&fn) {
  constexpr int LA = LC > 0 ? LC : kMaxL;
  const int L = LC > 0 ? LC : Lrt;
  T r = sqrt(x * x + y * y + z * z);
  T ir = T(1) / r;
  T ux = x * ir, uy = y * ir, uz = z * ir;
  T C[LA + 1], S[LA + 1];
  C[0] = T(1); S[0] = T(0);
#pragma unroll
  for (int m = 1; m <= L; m++) {
    C[m] = ux * C[m - 1] - uy * S[m - 1];
    S[m] = ux * S[m - 1] + uy * C[m - 1];
  }
  T qnext[LA + 2];   // Q_l^{m+1}, indexed by l
  T qcur[LA + 2];
#pragma unroll
  for (int l = 0; l <= L + 1; l++) qnext[l] = T(0);
  // (2m-1)!! for m = L
#pragma unroll
  for (int m = L; m >= 0; m--) {
    T dfact;
    dfact_const(m, dfact);                  // (2m-1)!!
#pragma unroll
    for (int l = 0; l <= L; l++) qcur[l] = T(0);
    qcur[m] = dfact;
    if (m + 1 <= L) qcur[m + 1] = T(2 * m + 1) * uz * dfact;
#pragma unroll
    for (int l = m + 2; l <= L; l++)
      qcur[l] = div_int(T(2 * l - 1) * uz * qcur[l - 1] -
                            T(l + m - 1) * qcur[l - 2],
                        l - m);
#pragma unroll
    for (int l = m; l <= L; l++) {
      T K;
      ylm_norm(l * (kMaxL + 1) + m, K);
      T qv = qcur[l], qd = qnext[l];
      if (m == 0) {
        const int idx = l * l + l;
        if (Grad) {
          T G2 = K * qd;
          T ug = uz * G2;
          fn(idx, K * qv, (-ux * ug) * ir, (-uy * ug) * ir, (G2 - uz * ug) * ir);
        } else {
          fn(idx, K * qv, T(0), T(0), T(0));
        }
      } else {
        const int ip = l * l + l + m, in = l * l + l - m;
        if (Grad) {
          T a = K * qv * T(m);
          // +m: G = K (Q m C_{m-1}, -Q m S_{m-1}, Q' C_m)
          T G0 = a * C[m - 1], G1 = -a * S[m - 1], G2 = K * qd * C[m];
          T ug = ux * G0 + uy * G1 + uz * G2;
          fn(ip, K * qv * C[m], (G0 - ux * ug) * ir, (G1 - uy * ug) * ir,
             (G2 - uz * ug) * ir);
          // -m: G = K (Q m S_{m-1}, Q m C_{m-1}, Q' S_m)
          G0 = a * S[m - 1]; G1 = a * C[m - 1]; G2 = K * qd * S[m];
          ug = ux * G0 + uy * G1 + uz * G2;
          fn(in, K * qv * S[m], (G0 - ux * ug) * ir, (G1 - uy * ug) * ir,
             (G2 - uz * ug) * ir);
        } else {
          fn(ip, K * qv * C[m], T(0), T(0), T(0));
          fn(in, K * qv * S[m], T(0), T(0), T(0));
        }
      }
    }
#pragma unroll
    for (int l = 0; l <= L; l++) qnext[l] = qcur[l];
  }
}

// The harmonics into Y[] (and, if Yd != nullptr, the Cartesian gradient
// into Yd[3*idx + k]).
template <typename T, int LC = 0>
__device__ __forceinline__ void ylm_eval(int L, T x, T y, T z, T *Y, T *Yd) {
  if (Yd) {
    ylm_visit<T, LC, true>(L, x, y, z, [&](int idx, T v, T gx, T gy, T gz) {
      Y[idx] = v;
      Yd[3 * idx] = gx;
      Yd[3 * idx + 1] = gy;
      Yd[3 * idx + 2] = gz;
    });
  } else {
    ylm_visit<T, LC, false>(L, x, y, z,
                            [&](int idx, T v, T, T, T) { Y[idx] = v; });
  }
}

// Largest power of two >= x (x >= 1).
__host__ __device__ inline int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace fgb
