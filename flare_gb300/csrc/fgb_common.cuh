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
  double cutoff_hyps[4];
  int n_cutoff_hyps;
  double cutoffs[kMaxSpecies * kMaxSpecies];   // per species pair
  double max_cutoff;
};

// Spherical-harmonic normalisation K_lm = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!),
// times sqrt2 for m > 0, indexed [l * (kMaxL + 1) + m] (double-precision
// values of the formula, evaluated once and written out).
static __constant__ double c_ylm_norm[(kMaxL + 1) * (kMaxL + 1)] = {
    0.28209479177387814, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,  // l = 0
    0.4886025119029199, 0.48860251190292, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,  // l = 1
    0.6307831305050401, 0.3641828101973597, 0.18209140509867985, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,  // l = 2
    0.7463526651802308, 0.3046971996429772, 0.09635371475468515, 0.03933623932844291, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,  // l = 3
    0.8462843753216345, 0.2676186174229157, 0.063078313050504, 0.016858388283618388, 0.005960340337611203, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,  // l = 4
    0.9356025796273888, 0.2415715473043717, 0.045652731285460234, 0.009318824751147628, 0.002196468058075176, 0.0006945841871324552, 0.0, 0.0, 0.0, 0.0, 0.0,  // l = 5
    1.0171072362820548, 0.22195099524523101, 0.03509353369580661, 0.005848922282634434, 0.0010678622237644956, 0.00022766899107568565, 6.57223766418388e-05, 0.0, 0.0, 0.0, 0.0,  // l = 6
    1.0925484305920792, 0.20647224590289676, 0.028097313806030647, 0.003973560225074135, 0.0005990367431114117, 9.983945718523528e-05, 1.958012847746254e-05, 5.233009453691467e-06, 0.0, 0.0, 0.0,  // l = 7
    1.1631066229203195, 0.19385110382005324, 0.023169638523677944, 0.0028519853513317033, 0.00036818972564450655, 5.1058728265780266e-05, 7.878532816214048e-06, 1.4384167144950456e-06, 3.596041786237614e-07, 0.0, 0.0,  // l = 8
    1.2296226898414837, 0.1833013280774465, 0.019539987227523183, 0.0021319873940141734, 0.00024140003633280337, 2.8852822971932874e-05, 3.7248834287122265e-06, 5.376406125667451e-07, 9.220460437034855e-08, 2.1732833668965406e-08, 0.0,  // l = 9
    1.2927207364566027, 0.17431042854448453, 0.016773028807119526, 0.001644730792106853, 0.0001661428994750111, 1.7512999313514277e-05, 1.958012847746254e-06, 2.37443934928654e-07, 3.231202683854524e-08, 5.24170291336415e-09, 1.1720804032140929e-09,  // l = 10
};

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

// Chebyshev radial basis on x = (r - r1)/(rc - r1) (radial.cpp:138-169)
// times the cutoff (radial.cpp:344-379).  Writes g[n] and dg/dr[n]
// (radial derivative; Cartesian derivatives are dg/dr * x_k / r).
template <typename T>
__device__ __forceinline__ void radial_eval(const B2Params &p, T r, T rc,
                                            T *g, T *dg) {
  T fc, dfc;
  cutoff_eval<T>(p, r, rc, fc, dfc);
  const int N = p.n_max;
  T r1 = T(p.r1);
  if (r < r1 || r > rc) {
    for (int n = 0; n < N; n++) {
      g[n] = T(0);
      if (dg) dg[n] = T(0);
    }
    return;
  }
  T c = T(1) / (rc - r1);
  T x = (r - r1) * c;
  T b0 = T(1), db0 = T(0), b1 = x, db1 = c;
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
// If Yd != nullptr, also writes the Cartesian gradient: Yd[3*idx + k].
template <typename T>
__device__ __forceinline__ void ylm_eval(int L, T x, T y, T z, T *Y, T *Yd) {
  T r = sqrt(x * x + y * y + z * z);
  T ir = T(1) / r;
  T ux = x * ir, uy = y * ir, uz = z * ir;
  T C[kMaxL + 1], S[kMaxL + 1];
  C[0] = T(1); S[0] = T(0);
  for (int m = 1; m <= L; m++) {
    C[m] = ux * C[m - 1] - uy * S[m - 1];
    S[m] = ux * S[m - 1] + uy * C[m - 1];
  }
  T qnext[kMaxL + 2];   // Q_l^{m+1}, indexed by l
  T qcur[kMaxL + 2];
  for (int l = 0; l <= L + 1; l++) qnext[l] = T(0);
  // (2m-1)!! for m = L
  T dfact = T(1);
  for (int k = 1; k <= L; k++) dfact *= T(2 * k - 1);
  for (int m = L; m >= 0; m--) {
    if (m < L) dfact /= T(2 * m + 1);       // (2m-1)!!
    for (int l = 0; l <= L; l++) qcur[l] = T(0);
    qcur[m] = dfact;
    if (m + 1 <= L) qcur[m + 1] = T(2 * m + 1) * uz * dfact;
    for (int l = m + 2; l <= L; l++)
      qcur[l] = (T(2 * l - 1) * uz * qcur[l - 1] - T(l + m - 1) * qcur[l - 2]) /
                T(l - m);
    for (int l = m; l <= L; l++) {
      T K = T(c_ylm_norm[l * (kMaxL + 1) + m]);
      T qv = qcur[l], qd = qnext[l];
      if (m == 0) {
        int idx = l * l + l;
        Y[idx] = K * qv;
        if (Yd) {
          T G2 = K * qd;
          T ug = uz * G2;
          Yd[3 * idx + 0] = (-ux * ug) * ir;
          Yd[3 * idx + 1] = (-uy * ug) * ir;
          Yd[3 * idx + 2] = (G2 - uz * ug) * ir;
        }
      } else {
        int ip = l * l + l + m, in = l * l + l - m;
        Y[ip] = K * qv * C[m];
        Y[in] = K * qv * S[m];
        if (Yd) {
          T a = K * qv * T(m);
          // +m: G = K (Q m C_{m-1}, -Q m S_{m-1}, Q' C_m)
          T G0 = a * C[m - 1], G1 = -a * S[m - 1], G2 = K * qd * C[m];
          T ug = ux * G0 + uy * G1 + uz * G2;
          Yd[3 * ip + 0] = (G0 - ux * ug) * ir;
          Yd[3 * ip + 1] = (G1 - uy * ug) * ir;
          Yd[3 * ip + 2] = (G2 - uz * ug) * ir;
          // -m: G = K (Q m S_{m-1}, Q m C_{m-1}, Q' S_m)
          G0 = a * S[m - 1]; G1 = a * C[m - 1]; G2 = K * qd * S[m];
          ug = ux * G0 + uy * G1 + uz * G2;
          Yd[3 * in + 0] = (G0 - ux * ug) * ir;
          Yd[3 * in + 1] = (G1 - uy * ug) * ir;
          Yd[3 * in + 2] = (G2 - uz * ug) * ir;
        }
      }
    }
    for (int l = 0; l <= L; l++) qnext[l] = qcur[l];
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
