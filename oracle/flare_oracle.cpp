// FP64 CPU oracle for FLARE's sparse-GP prediction path.
//
// TEST INFRASTRUCTURE ONLY.  This file is a loop-by-loop restatement of the
// reference's C++ (flare_pp) algorithms, used by the test-suite as the parity
// checker and by bench.py as the timed CPU baseline.  No product code path
// links or calls it.
//
// What is restated, and from where (paths inside mir-group/flare):
//   * cell algebra, wrapping, sweep      src/flare_pp/structure.cpp:7-43,120-165
//   * brute-force neighbour list          src/flare_pp/structure.cpp:52-118
//   * radial bases (all nine)             src/flare_pp/radial.cpp:6-336,381-408
//   * radial x cutoff product             src/flare_pp/radial.cpp:344-379
//   * cutoff functions                    src/flare_pp/cutoffs.cpp:7-85
//   * real spherical harmonics + grads    src/flare_pp/y_grad.cpp:667-2754
//       (restated by the associated-Legendre recurrence, not the closed
//        forms; values agree to rounding, pinned by tests/golden/)
//   * single-bond (A_nlm) accumulation    src/flare_pp/descriptors/b2.cpp:244-399
//   * B2 contraction + stored gradients   src/flare_pp/descriptors/b2.cpp:181-242
//   * envs_struc kernel scatter loop      src/flare_pp/kernels/normalized_dot_product.cpp:117-214
//   * self_kernel_struc (DTC prior)       src/flare_pp/kernels/normalized_dot_product.cpp:450-586
//   * struc_struc                         src/flare_pp/kernels/normalized_dot_product.cpp:216-448
//
// Canonical floating-point order: built with -ffp-contract=off so that no
// multiply-add is fused; wrapping and neighbour distances use the operation
// order written below, which the CUDA neighbour kernel repeats exactly.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

namespace {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------- cell algebra
// 3x3 inverse by cofactors: inv[i][j] = cof[j][i] / det, det by first-row
// expansion.  (The reference uses Eigen's inverse; the formula here is the
// documented canonical one shared with the CUDA host code.)
void inv3(const double *a, double *out) {
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

// c = a * b for row-major 3x3, k summed 0..2 left to right.
void mul3(const double *a, const double *b, double *c) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      c[3 * i + j] = (a[3 * i + 0] * b[0 + j] + a[3 * i + 1] * b[3 + j]) +
                     a[3 * i + 2] * b[6 + j];
}

}  // namespace

extern "C" {

// Cell matrices used by wrapping (structure.cpp:18-21) plus volume
// (structure.cpp:15) and the single-sweep cutoff (structure.cpp:135-165).
// out layout: [cellT(9), cellT_inv(9), cell_dot(9), cell_dot_inv(9),
//              volume, single_sweep_cutoff]
void orc_cell_setup(const double *cell, double *out) {
  double ct[9], cti[9], cd[9], cdi[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) ct[3 * i + j] = cell[3 * j + i];
  inv3(ct, cti);
  mul3(cell, ct, cd);
  inv3(cd, cdi);
  std::memcpy(out, ct, sizeof(ct));
  std::memcpy(out + 9, cti, sizeof(cti));
  std::memcpy(out + 18, cd, sizeof(cd));
  std::memcpy(out + 27, cdi, sizeof(cdi));
  double det = cell[0] * (cell[4] * cell[8] - cell[5] * cell[7]) +
               cell[1] * (cell[5] * cell[6] - cell[3] * cell[8]) +
               cell[2] * (cell[3] * cell[7] - cell[4] * cell[6]);
  out[36] = std::fabs(det);

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
  out[37] = s;
}

// Wrapped positions, structure.cpp:120-133:
//   frac = (pos * cellT) * cell_dot_inv ; frac -= floor(frac)
//   wrapped = (frac * cell_dot) * cellT_inv
void orc_wrap_positions(const double *cell, const double *pos, int n,
                        double *wrapped) {
  double setup[38];
  orc_cell_setup(cell, setup);
  const double *ct = setup, *cti = setup + 9, *cd = setup + 18,
               *cdi = setup + 27;
  for (int i = 0; i < n; i++) {
    const double *p = pos + 3 * i;
    double t[3], f[3], u[3];
    for (int k = 0; k < 3; k++)
      t[k] = (p[0] * ct[k] + p[1] * ct[3 + k]) + p[2] * ct[6 + k];
    for (int k = 0; k < 3; k++)
      f[k] = (t[0] * cdi[k] + t[1] * cdi[3 + k]) + t[2] * cdi[6 + k];
    for (int k = 0; k < 3; k++) f[k] = f[k] - std::floor(f[k]);
    for (int k = 0; k < 3; k++)
      u[k] = (f[0] * cd[k] + f[1] * cd[3 + k]) + f[2] * cd[6 + k];
    for (int k = 0; k < 3; k++)
      wrapped[3 * i + k] = (u[0] * cti[k] + u[1] * cti[3 + k]) + u[2] * cti[6 + k];
  }
}

// Brute-force neighbour list, structure.cpp:52-118.  Order: i, then j
// ascending, then s1, s2, s3 ascending from -sweep to +sweep; keep
// 0 < d < cutoff.  Two calls: with out arrays == nullptr it only counts and
// returns the total; otherwise it fills.
//   counts[n], rel[P*4] = (d, x, y, z), idx[P] = j, shift[P*3] = (s1,s2,s3)
long long orc_neighbors(const double *cell, const double *wrapped, int n,
                        double cutoff, int sweep, int *counts, double *rel,
                        int *idx, int *shift) {
  std::vector<long long> cnt(n, 0);
#pragma omp parallel for schedule(dynamic, 4)
  for (int i = 0; i < n; i++) {
    long long c = 0;
    const double *wi = wrapped + 3 * i;
    for (int j = 0; j < n; j++) {
      const double *wj = wrapped + 3 * j;
      double d0 = wj[0] - wi[0], d1 = wj[1] - wi[1], d2 = wj[2] - wi[2];
      for (int s1 = -sweep; s1 <= sweep; s1++)
        for (int s2 = -sweep; s2 <= sweep; s2++)
          for (int s3 = -sweep; s3 <= sweep; s3++) {
            double x = ((d0 + s1 * cell[0]) + s2 * cell[3]) + s3 * cell[6];
            double y = ((d1 + s1 * cell[1]) + s2 * cell[4]) + s3 * cell[7];
            double z = ((d2 + s1 * cell[2]) + s2 * cell[5]) + s3 * cell[8];
            double d = std::sqrt((x * x + y * y) + z * z);
            if (d < cutoff && d != 0) c++;
          }
    }
    cnt[i] = c;
  }
  std::vector<long long> off(n + 1, 0);
  for (int i = 0; i < n; i++) off[i + 1] = off[i] + cnt[i];
  if (counts)
    for (int i = 0; i < n; i++) counts[i] = (int)cnt[i];
  if (!rel) return off[n];
#pragma omp parallel for schedule(dynamic, 4)
  for (int i = 0; i < n; i++) {
    long long c = off[i];
    const double *wi = wrapped + 3 * i;
    for (int j = 0; j < n; j++) {
      const double *wj = wrapped + 3 * j;
      double d0 = wj[0] - wi[0], d1 = wj[1] - wi[1], d2 = wj[2] - wi[2];
      for (int s1 = -sweep; s1 <= sweep; s1++)
        for (int s2 = -sweep; s2 <= sweep; s2++)
          for (int s3 = -sweep; s3 <= sweep; s3++) {
            double x = ((d0 + s1 * cell[0]) + s2 * cell[3]) + s3 * cell[6];
            double y = ((d1 + s1 * cell[1]) + s2 * cell[4]) + s3 * cell[7];
            double z = ((d2 + s1 * cell[2]) + s2 * cell[5]) + s3 * cell[8];
            double d = std::sqrt((x * x + y * y) + z * z);
            if (d < cutoff && d != 0) {
              rel[4 * c + 0] = d; rel[4 * c + 1] = x;
              rel[4 * c + 2] = y; rel[4 * c + 3] = z;
              idx[c] = j;
              if (shift) {
                shift[3 * c + 0] = s1; shift[3 * c + 1] = s2;
                shift[3 * c + 2] = s3;
              }
              c++;
            }
          }
    }
  }
  return off[n];
}

// ------------------------------------------------------------ per-pair math
// Radial basis ids: 0 = chebyshev (radial.cpp:138-169).
// Cutoff ids: 0 quadratic, 1 hard, 2 cosine, 3 polynomial, 4 power
// (cutoffs.cpp:7-85).

static void cutoff_fn(int id, double r, double rc, const double *ch, int nch,
                      double *v, double *dv) {
  if (r > rc) { *v = 0; *dv = 0; return; }
  switch (id) {
    case 0: { double d = r - rc; *v = d * d; *dv = 2 * d; return; }
    case 1: { *v = 1; *dv = 0; return; }
    case 2: {
      *v = 0.5 * (std::cos(kPi * r / rc) + 1);
      *dv = -kPi * std::sin(kPi * r / rc) / (2 * rc);
      return;
    }
    case 3: {
      int p = (int)ch[0];
      double d = r / rc;
      double c1 = (p + 1) * (p + 2) / 2;  // integer division as in reference
      double c2 = p * (p + 2);
      double c3 = p * (p + 1) / 2;
      *v = 1 - c1 * std::pow(d, p) + c2 * std::pow(d, p + 1) -
           c3 * std::pow(d, p + 2);
      double c4 = c1 * p / rc, c5 = c2 * (p + 1) / rc, c6 = c3 * (p + 2) / rc;
      *dv = -c4 * std::pow(d, p - 1) + c5 * std::pow(d, p) -
            c6 * std::pow(d, p + 1);
      return;
    }
    case 4: {
      double pw = ch[0], rd = rc - r;
      *v = std::pow(rd, pw);
      *dv = -pw * std::pow(rd, pw - 1);
      return;
    }
  }
  *v = 0; *dv = 0;
}

// Radial bases (radial.cpp:6-336), ids in the order of set_radial_basis
// (radial.cpp:381-408): 0 chebyshev, 1 weighted_chebyshev,
// 2 equispaced_gaussians, 3 weighted_positive_chebyshev,
// 4 positive_chebyshev, 5 bessel, 6 fourier_quarter, 7 fourier_half,
// 8 fourier.  Hyperparameters (h0, r2, h2) are radial_hyps[0], the pair
// cutoff (the B2 descriptor overwrites radial_hyps[1] with it, b2.cpp:352)
// and radial_hyps[2].  Values and radial derivatives; zero outside the
// support [h0, r2] of every basis but the Gaussians.
static void radial_fn(int id, double r, int N, double r1, double r2,
                      double h2, double *g, double *dg) {
  for (int n = 0; n < N; n++) { g[n] = 0; dg[n] = 0; }
  if (id == 2) {
    // Gaussians of width h0 centred from radial_hyps[1] to radial_hyps[2]
    const double sigma = r1, first = r2, sep = h2 - r2;
    const double norm = 1 / (sigma * std::sqrt(2 * kPi));
    const double s2 = 1 / (sigma * sigma), hs2 = s2 / 2;
    for (int n = 0; n < N; n++) {
      const double mean = first + (n * sep / (N - 1));
      const double d = r - mean;
      g[n] = norm * std::exp(-hs2 * d * d);
      dg[n] = -s2 * g[n] * d;
    }
    return;
  }
  if (r < r1 || r > r2) return;
  if (id == 0 || id == 4) {
    // Chebyshev polynomials T_n(x), x = (r - r1)/(r2 - r1); the positive
    // variant is (1 - T_n)/2 with the reference's recurrence, which runs on
    // the transformed values themselves (radial.cpp:195-206)
    const double c = 1 / (r2 - r1), x = (r - r1) * c;
    for (int n = 0; n < N; n++) {
      if (n == 0) { g[n] = 1; dg[n] = 0; continue; }
      double t, dt;
      if (n == 1) { t = x; dt = c; }
      else {
        t = 2 * x * g[n - 1] - g[n - 2];
        dt = 2 * g[n - 1] * c + 2 * x * dg[n - 1] - dg[n - 2];
      }
      if (id == 0) { g[n] = t; dg[n] = dt; }
      else { g[n] = 0.5 * (1 - t); dg[n] = -0.5 * dt; }
    }
    return;
  }
  if (id == 1 || id == 3) {
    // Chebyshev polynomials of an exponentially weighted coordinate
    const double c = 1 / (r2 - r1), x = (r - r1) * c;
    const double e = std::exp(-h2 * (x - 1)), lc = std::exp(h2) - 1;
    const double xw = 1 - 2 * (e - 1) / lc, dxdr = 2 * c * h2 * e / lc;
    double t0 = 1, d0 = 0, t1 = xw, d1 = 1;
    for (int n = 0; n < N; n++) {
      double t, dt;
      if (n == 0) { g[n] = 1; dg[n] = 0; continue; }
      if (n == 1) { t = t1; dt = d1; }
      else {
        t = 2 * xw * t1 - t0;
        dt = 2 * t1 + 2 * xw * d1 - d0;
        t0 = t1; d0 = d1; t1 = t; d1 = dt;
      }
      if (id == 1) { g[n] = t; dg[n] = dt * dxdr; }
      else { g[n] = 0.5 * (1 - t); dg[n] = -0.5 * dt * dxdr; }
    }
    return;
  }
  if (id == 5) {
    // spherical Bessel functions of order zero, zeros at r2
    const double c = r2 - r1, c1 = std::sqrt(2 / c), d = r - r1;
    for (int n = 0; n < N; n++) {
      const double a = kPi * (n + 1) * d, b = a / c, e = c * d * d;
      g[n] = c1 * std::sin(b) / d;
      dg[n] = c1 * (a * std::cos(b) - c * std::sin(b)) / e;
    }
    return;
  }
  if (id >= 6 && id <= 8) {
    // 1, cos(k w x), sin(k w x), ... with w = pi/2, pi or pi h2
    const double c = 1 / (r2 - r1), x = (r - r1) * c;
    const double w = id == 6 ? kPi / 2 : (id == 7 ? kPi : kPi * h2);
    int kc = 1, ks = 1;
    for (int n = 0; n < N; n++) {
      if (n == 0) { g[n] = 1; dg[n] = 0; }
      else if (n % 2 == 1) {
        const double a = w * kc++;
        g[n] = std::cos(a * x); dg[n] = -std::sin(a * x) * a * c;
      } else {
        const double a = w * ks++;
        g[n] = std::sin(a * x); dg[n] = std::cos(a * x) * a * c;
      }
    }
  }
}

// Radial x cutoff with Cartesian gradients (radial.cpp:344-379).
// out: g[N], gx[N], gy[N], gz[N]
void orc_radial(int radial_id, int cutoff_id, double x, double y, double z,
                double r, double rc, int N, double r1, double h2,
                const double *ch, int nch, double *g, double *gx, double *gy,
                double *gz) {
  double fc, dfc;
  cutoff_fn(cutoff_id, r, rc, ch, nch, &fc, &dfc);
  std::vector<double> b(N), db(N);
  radial_fn(radial_id, r, N, r1, rc, h2, b.data(), db.data());
  double xr = x / r, yr = y / r, zr = z / r;
  for (int n = 0; n < N; n++) {
    g[n] = b[n] * fc;
    gx[n] = db[n] * xr * fc + b[n] * xr * dfc;
    gy[n] = db[n] * yr * fc + b[n] * yr * dfc;
    gz[n] = db[n] * zr * fc + b[n] * zr * dfc;
  }
}

// Real spherical harmonics Y_lm (l-major, m = -l..l; no Condon-Shortley
// phase), the convention of y_grad.cpp:667-2754, with Cartesian gradients.
// Method: u = r/|r|;  (ux + i uy)^m = C_m + i S_m;  Q_l^m(uz) = d^m P_l/dz^m
// by the standard three-term recurrence;  Y_l0 = K_l0 Q_l^0,
// Y_l,+m = sqrt2 K_lm Q_l^m C_m, Y_l,-m = sqrt2 K_lm Q_l^m S_m with
// K_lm = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!).  Gradient of Y(u(r)):
// (1/|r|)(G - u (u.G)) with G the gradient of the polynomial form in u,
// using dQ_l^m/dz = Q_l^{m+1}.
void orc_ylm(double x, double y, double z, int L, double *Y, double *Yx,
             double *Yy, double *Yz) {
  double r = std::sqrt(x * x + y * y + z * z);
  double ux = x / r, uy = y / r, uz = z / r;
  // C, S up to L
  std::vector<double> C(L + 2), S(L + 2);
  C[0] = 1; S[0] = 0;
  for (int m = 1; m <= L; m++) {
    C[m] = ux * C[m - 1] - uy * S[m - 1];
    S[m] = ux * S[m - 1] + uy * C[m - 1];
  }
  // Q[l][m] for 0<=m<=l+1 (Q_l^{l+1} = 0)
  std::vector<double> Q((L + 1) * (L + 2), 0.0);
  auto q = [&](int l, int m) -> double & { return Q[l * (L + 2) + m]; };
  double dfact = 1;  // (2m-1)!!
  for (int m = 0; m <= L; m++) {
    if (m > 0) dfact *= (2 * m - 1);
    q(m, m) = dfact;
    if (m + 1 <= L) q(m + 1, m) = (2 * m + 1) * uz * dfact;
    for (int l = m + 2; l <= L; l++)
      q(l, m) = ((2 * l - 1) * uz * q(l - 1, m) - (l + m - 1) * q(l - 2, m)) /
                (l - m);
  }
  const double sqrt2 = std::sqrt(2.0);
  for (int l = 0; l <= L; l++) {
    for (int mm = -l; mm <= l; mm++) {
      int m = mm < 0 ? -mm : mm;
      // K_lm
      double ratio = 1;  // (l-m)!/(l+m)!
      for (int k = l - m + 1; k <= l + m; k++) ratio /= k;
      double K = std::sqrt((2 * l + 1) / (4 * kPi) * ratio);
      double qv = q(l, m);
      double qd = (m + 1 <= l) ? q(l, m + 1) : 0.0;
      double val, G0, G1, G2;
      if (mm == 0) {
        val = K * qv;
        G0 = 0; G1 = 0; G2 = K * qd;
      } else if (mm > 0) {
        double f = sqrt2 * K;
        val = f * qv * C[m];
        G0 = f * qv * m * C[m - 1];
        G1 = -f * qv * m * S[m - 1];
        G2 = f * qd * C[m];
      } else {
        double f = sqrt2 * K;
        val = f * qv * S[m];
        G0 = f * qv * m * S[m - 1];
        G1 = f * qv * m * C[m - 1];
        G2 = f * qd * S[m];
      }
      double ug = ux * G0 + uy * G1 + uz * G2;
      int idx = l * l + (mm + l);
      Y[idx] = val;
      Yx[idx] = (G0 - ux * ug) / r;
      Yy[idx] = (G1 - uy * ug) / r;
      Yz[idx] = (G2 - uz * ug) / r;
    }
  }
}

// ------------------------------------------------------------------- B2
// single_bond_multiple_cutoffs (b2.cpp:244-399) + compute_b2 (b2.cpp:181-242)
// for one structure.  Inputs are the structure neighbour list in reference
// order.  Outputs (atom order, not species-sorted):
//   b2_count[n]               neighbours kept by the per-pair cutoff filter
//   b2_idx[Pb], b2_coords[Pb*3]
//   single_bond[n * nA], B2[n * nd], norms[n]
//   dervs[3Pb * nd] and force_dots[3Pb]   (only when dervs != nullptr)
// Two-phase: call with B2 == nullptr to get Pb (return value).
long long orc_b2(int n, const int *species, const int *counts,
                 const double *rel, const int *idx, int radial_id,
                 int cutoff_id, double r1, double h2, const double *cutoff_hyps,
                 int nch,
                 int S, int N, int L, const double *cutoffs, int *b2_count,
                 int *b2_idx, double *b2_coords, double *single_bond,
                 double *B2, double *norms, double *dervs,
                 double *force_dots) {
  std::vector<long long> off(n + 1, 0);
  for (int i = 0; i < n; i++) off[i + 1] = off[i] + counts[i];
  std::vector<long long> boff(n + 1, 0);
  std::vector<int> bc(n, 0);
  for (int i = 0; i < n; i++) {
    int si = species[i], c = 0;
    for (long long p = off[i]; p < off[i + 1]; p++) {
      int sj = species[idx[p]];
      if (rel[4 * p] <= cutoffs[si * S + sj]) c++;
    }
    bc[i] = c;
    boff[i + 1] = boff[i] + c;
  }
  if (b2_count)
    for (int i = 0; i < n; i++) b2_count[i] = bc[i];
  if (!B2) return boff[n];

  const int nh = (L + 1) * (L + 1);
  const int nr = S * N;
  const int nA = nr * nh;
  const int nd = nr * (nr + 1) / 2 * (L + 1);

#pragma omp parallel for schedule(dynamic, 2)
  for (int i = 0; i < n; i++) {
    int si = species[i];
    std::vector<double> g(N), gx(N), gy(N), gz(N);
    std::vector<double> h(nh), hx(nh), hy(nh), hz(nh);
    double *A = single_bond + (long long)i * nA;
    for (int k = 0; k < nA; k++) A[k] = 0;
    long long bp = boff[i];
    // local per-neighbour single-bond gradients (3 x nA per neighbour)
    std::vector<double> dA((size_t)bc[i] * 3 * nA, 0.0);
    int local = 0;
    for (long long p = off[i]; p < off[i + 1]; p++) {
      int j = idx[p];
      int sj = species[j];
      double rc = cutoffs[si * S + sj];
      double r = rel[4 * p];
      if (r > rc) continue;
      double x = rel[4 * p + 1], y = rel[4 * p + 2], z = rel[4 * p + 3];
      b2_idx[bp] = j;
      b2_coords[3 * bp + 0] = x;
      b2_coords[3 * bp + 1] = y;
      b2_coords[3 * bp + 2] = z;
      orc_radial(radial_id, cutoff_id, x, y, z, r, rc, N, r1, h2, cutoff_hyps,
                 nch, g.data(), gx.data(), gy.data(), gz.data());
      orc_ylm(x, y, z, L, h.data(), hx.data(), hy.data(), hz.data());
      int col = sj * N * nh;
      double *dl = dA.data() + (size_t)local * 3 * nA;
      for (int rn = 0; rn < N; rn++) {
        for (int a = 0; a < nh; a++) {
          A[col] += g[rn] * h[a];
          dl[col] += gx[rn] * h[a] + g[rn] * hx[a];
          dl[nA + col] += gy[rn] * h[a] + g[rn] * hy[a];
          dl[2 * nA + col] += gz[rn] * h[a] + g[rn] * hz[a];
          col++;
        }
      }
      bp++;
      local++;
    }
    // B2 contraction (b2.cpp:209-233).  The reference stores
    // B2_force_dervs column-major (Eigen), so its inner neighbour loop walks
    // contiguous memory; with row-major storage here the same arithmetic is
    // ordered neighbour-major so that the writes stay contiguous.
    double *b = B2 + (long long)i * nd;
    {
      int counter = 0;
      for (int n1 = 0; n1 < nr; n1++)
        for (int n2 = n1; n2 < nr; n2++)
          for (int l = 0; l < L + 1; l++) {
            double acc = 0;
            for (int m = 0; m < 2 * l + 1; m++) {
              int i1 = n1 * nh + l * l + m, i2 = n2 * nh + l * l + m;
              acc += A[i1] * A[i2];
            }
            b[counter++] = acc;
          }
    }
    if (dervs) {
      for (int nb = 0; nb < bc[i]; nb++)
        for (int comp = 0; comp < 3; comp++) {
          const double *dl = dA.data() + ((size_t)nb * 3 + comp) * nA;
          double *out = dervs + ((boff[i] + nb) * 3 + comp) * nd;
          int counter = 0;
          for (int n1 = 0; n1 < nr; n1++)
            for (int n2 = n1; n2 < nr; n2++)
              for (int l = 0; l < L + 1; l++) {
                double acc2 = 0;
                for (int m = 0; m < 2 * l + 1; m++) {
                  int i1 = n1 * nh + l * l + m, i2 = n2 * nh + l * l + m;
                  acc2 += A[i1] * dl[i2] + dl[i1] * A[i2];
                }
                out[counter++] = acc2;
              }
        }
    }
    double nn = 0;
    for (int k = 0; k < nd; k++) nn += b[k] * b[k];
    norms[i] = std::sqrt(nn);
    if (dervs) {
      for (int nb = 0; nb < bc[i]; nb++)
        for (int comp = 0; comp < 3; comp++) {
          const double *dv = dervs + ((boff[i] + nb) * 3 + comp) * nd;
          double acc = 0;
          for (int k = 0; k < nd; k++) acc += dv[k] * b[k];
          force_dots[(boff[i] + nb) * 3 + comp] = acc;
        }
    }
  }
  return boff[n];
}

// ------------------------------------------------------------ envs_struc
// NormalizedDotProduct::envs_struc scatter loop for ONE species block
// (normalized_dot_product.cpp:156-210).  dot_vals (Ms x Ns) and
// force_dot (Ms x 3Pb_s) are the two GEMMs of :145-146, computed by the
// caller.  kern is the full (M x (1 + 3 n_atoms + 6)) matrix, row-major;
// c_sparse is the first row of this species block.
void orc_envs_struc_block(int Ms, int Ns, int n_atoms, int c_sparse,
                          const double *sparse_norms, const double *struc_norms,
                          const double *dot_vals, const double *force_dot,
                          const double *struc_force_dots,
                          const int *neighbor_counts, const int *cum_neighbor,
                          const int *atom_indices, const int *neighbor_indices,
                          const double *neighbor_coords, double sig_sq,
                          double power, double vol_inv, double *kern) {
  const double empty_thresh = 1e-8;
  const long long ncol = 1 + 3LL * n_atoms + 6;
  long long fcols = 0;
  for (int j = 0; j < Ns; j++) fcols += neighbor_counts[j];
  fcols *= 3;
#pragma omp parallel for schedule(dynamic, 4)
  for (int i = 0; i < Ms; i++) {
    double norm_i = sparse_norms[i];
    if (norm_i < empty_thresh) continue;
    double *row = kern + (long long)(c_sparse + i) * ncol;
    for (int j = 0; j < Ns; j++) {
      double norm_j = struc_norms[j];
      double norm_ij = norm_i * norm_j;
      double norm_ij3 = norm_ij * norm_j * norm_j;
      if (norm_j < empty_thresh) continue;
      double dv = dot_vals[(long long)i * Ns + j];
      double norm_dot = dv / norm_ij;
      double dval = power * std::pow(norm_dot, power - 1);
      row[0] += sig_sq * std::pow(norm_dot, power);
      int n_neigh = neighbor_counts[j];
      int c_neigh = cum_neighbor[j];
      int atom_index = atom_indices[j];
      for (int k = 0; k < n_neigh; k++) {
        int neighbor_index = neighbor_indices[c_neigh + k];
        int stress_counter = 0;
        for (int comp = 0; comp < 3; comp++) {
          long long ind = c_neigh + k;
          long long fi = 3 * ind + comp;
          double f1 = force_dot[(long long)i * fcols + fi] / norm_ij;
          double f2 = dv * struc_force_dots[fi] / norm_ij3;
          double f3 = f1 - f2;
          double fk = sig_sq * dval * f3;
          row[1 + 3 * neighbor_index + comp] -= fk;
          row[1 + 3 * atom_index + comp] += fk;
          for (int comp2 = comp; comp2 < 3; comp2++) {
            double coord = neighbor_coords[ind * 3 + comp2];
            row[1 + 3 * n_atoms + stress_counter] -= fk * coord * vol_inv;
            stress_counter++;
          }
        }
      }
    }
  }
}

// Prior variances of one structure's energy, forces and stress for one
// species block (normalized_dot_product.cpp:450-586): every atom pair
// i <= j of the block (twice when i != j), every pair of their neighbour
// entries, the same force component on both sides.  dot_vals = D D^T
// (Ns x Ns), force_dot = dD D^T (3Ps x Ns), force_force = dD dD^T
// (3Ps x 3Ps), struc_force_dots (3Ps).  Rows are summed into `out` (1 + 3
// n_atoms + 6) in atom order after the per-atom rows are complete, as the
// reference reduces par_mat.  Returns -1 where a dot product is below the
// empty threshold and power < 2 (the reference throws invalid_argument).
int orc_self_kernel_block(int Ns, int n_atoms, const double *norms,
                          const double *dot_vals, const double *force_dot,
                          const double *force_force,
                          const double *struc_force_dots,
                          const int *neighbor_counts, const int *cum_neighbor,
                          const int *atom_indices, const int *neighbor_indices,
                          const double *neighbor_coords, double sig_sq,
                          double power, double vol_inv, double *out) {
  const double empty_thresh = 1e-8;
  const double vol_inv_sq = vol_inv * vol_inv;
  const long long ncol = 1 + 3LL * n_atoms + 6;
  long long fcols = 0;
  for (int j = 0; j < Ns; j++) fcols += neighbor_counts[j];
  fcols *= 3;
  std::vector<double> par((size_t)Ns * ncol, 0.0);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
  for (int i = 0; i < Ns; i++) {
    const double norm_i = norms[i];
    if (norm_i < empty_thresh) continue;
    const double norm_i2 = norm_i * norm_i;
    const double norm_i3 = norm_i2 * norm_i;
    double *row = par.data() + (size_t)i * ncol;
    for (int j = i; j < Ns; j++) {
      const double norm_j = norms[j];
      if (norm_j < empty_thresh) continue;
      const double mult_fac = i == j ? 1.0 : 2.0;
      const double norm_j2 = norm_j * norm_j;
      const double norm_j3 = norm_j2 * norm_j;
      const double norm_ij = norm_i * norm_j;
      const double norm_dot = dot_vals[(size_t)i * Ns + j] / norm_ij;
      const double c1 = (power - 1) * power * std::pow(norm_dot, power - 2);
      if (std::fabs(norm_dot) < empty_thresh && power < 2) { bad = 1; continue; }
      const double c2 = power * std::pow(norm_dot, power - 1);
      row[0] += sig_sq * mult_fac * std::pow(norm_dot, power);
      const int n1 = neighbor_counts[i], cn1 = cum_neighbor[i];
      const int ci1 = atom_indices[i];
      const int n2 = neighbor_counts[j], cn2 = cum_neighbor[j];
      const int ci2 = atom_indices[j];
      for (int k = 0; k < n1; k++) {
        const long long ind1 = cn1 + k;
        const int ni1 = neighbor_indices[ind1];
        for (int l = 0; l < n2; l++) {
          const long long ind2 = cn2 + l;
          const int ni2 = neighbor_indices[ind2];
          int stress_counter = 0;
          for (int m = 0; m < 3; m++) {
            const long long f1 = 3 * ind1 + m, f2 = 3 * ind2 + m;
            const double v1 = force_dot[f1 * Ns + j] / norm_ij -
                              norm_dot * struc_force_dots[f1] / norm_i2;
            const double v2 = force_dot[f2 * Ns + i] / norm_ij -
                              norm_dot * struc_force_dots[f2] / norm_j2;
            const double v3 = force_force[f1 * fcols + f2] / norm_ij;
            const double v4 = struc_force_dots[f1] * force_dot[f2 * Ns + i] /
                              (norm_i3 * norm_j);
            const double v5 = struc_force_dots[f2] * force_dot[f1 * Ns + j] /
                              (norm_i * norm_j3);
            const double v6 = struc_force_dots[f1] * struc_force_dots[f2] *
                              norm_dot / (norm_i2 * norm_j2);
            const double kv =
                sig_sq * mult_fac * (c1 * v1 * v2 + c2 * (v3 - v4 - v5 + v6));
            if (ci1 == ci2) row[1 + ci1 * 3 + m] += kv;
            if (ci1 == ni2) row[1 + ci1 * 3 + m] -= kv;
            if (ni1 == ci2) row[1 + ni1 * 3 + m] -= kv;
            if (ni1 == ni2) row[1 + ni1 * 3 + m] += kv;
            for (int n = m; n < 3; n++) {
              const double x1 = neighbor_coords[ind1 * 3 + n];
              const double x2 = neighbor_coords[ind2 * 3 + n];
              row[1 + 3 * n_atoms + stress_counter] += kv * x1 * x2 * vol_inv_sq;
              stress_counter++;
            }
          }
        }
      }
    }
  }
  if (bad) return -1;
  for (int i = 0; i < Ns; i++)
    for (long long c = 0; c < ncol; c++) out[c] += par[(size_t)i * ncol + c];
  return 0;
}

// Structure-structure kernel block of one species
// (normalized_dot_product.cpp:216-448): energy/energy, energy/force,
// energy/stress and their transposes, force/force, force/stress,
// stress/force and stress/stress entries of the (1 + 3 N1 + 6) x
// (1 + 3 N2 + 6) row-major matrix `out`, accumulated in the reference's
// loop order (i over structure 1, j over structure 2, then neighbour
// entries).  dot_vals = D1 D2^T, force_dot_1 = dD1 D2^T (3P1 x N2s),
// force_dot_2 = dD2 D1^T (3P2 x N1s), force_force = dD1 dD2^T (3P1 x 3P2).
// Returns -1 where a dot product is below the empty threshold and
// power < 2 (the reference throws invalid_argument).
int orc_struc_struc_block(
    int N1s, int N2s, int n_atoms_1, int n_atoms_2, const double *norms_1,
    const double *norms_2, const double *dot_vals, const double *force_dot_1,
    const double *force_dot_2, const double *force_force,
    const double *sfd_1, const double *sfd_2, const int *nc_1,
    const int *cn_1, const int *ai_1, const int *ni_1, const double *co_1,
    const int *nc_2, const int *cn_2, const int *ai_2, const int *ni_2,
    const double *co_2, double sig_sq, double power, double vol_inv_1,
    double vol_inv_2, double *out) {
  const double empty_thresh = 1e-8;
  const long long n2 = 1 + 3LL * n_atoms_2 + 6;
  const int stress_inds[3] = {0, 3, 5};
  long long fc2 = 0;
  for (int j = 0; j < N2s; j++) fc2 += nc_2[j];
  fc2 *= 3;
  auto K = [&](long long r, long long c) -> double & { return out[r * n2 + c]; };
  const long long s1 = 1 + 3LL * n_atoms_1, s2 = 1 + 3LL * n_atoms_2;
  for (int i = 0; i < N1s; i++) {
    const double norm_i = norms_1[i];
    if (norm_i < empty_thresh) continue;
    const double norm_i2 = norm_i * norm_i, norm_i3 = norm_i2 * norm_i;
    for (int j = 0; j < N2s; j++) {
      const double norm_j = norms_2[j];
      if (norm_j < empty_thresh) continue;
      const double norm_j2 = norm_j * norm_j, norm_j3 = norm_j2 * norm_j;
      const double norm_ij = norm_i * norm_j;
      const double dv = dot_vals[(long long)i * N2s + j];
      const double norm_dot = dv / norm_ij;
      const double c1 = (power - 1) * power * std::pow(norm_dot, power - 2);
      if (std::fabs(norm_dot) < empty_thresh && power < 2) return -1;
      const double c2 = power * std::pow(norm_dot, power - 1);
      K(0, 0) += sig_sq * std::pow(norm_dot, power);
      const int n_neigh_1 = nc_1[i], c_neigh_1 = cn_1[i], c_ind_1 = ai_1[i];
      const int n_neigh_2 = nc_2[j], c_neigh_2 = cn_2[j], c_ind_2 = ai_2[j];
      // energy / force and energy / stress
      for (int k = 0; k < n_neigh_2; k++) {
        const long long ind = c_neigh_2 + k;
        const int nb = ni_2[ind];
        int sc = 0;
        for (int comp = 0; comp < 3; comp++) {
          const long long fi = 3 * ind + comp;
          const double f1 = force_dot_2[fi * N1s + i] / norm_ij;
          const double f2 = dv * sfd_2[fi] / (norm_i * norm_j3);
          const double fk = sig_sq * c2 * (f1 - f2);
          K(0, 1 + 3 * nb + comp) -= fk;
          K(0, 1 + 3 * c_ind_2 + comp) += fk;
          for (int comp2 = comp; comp2 < 3; comp2++) {
            K(0, s2 + sc) -= fk * co_2[ind * 3 + comp2] * vol_inv_2;
            sc++;
          }
        }
      }
      // force / energy and stress / energy
      for (int k = 0; k < n_neigh_1; k++) {
        const long long ind = c_neigh_1 + k;
        const int nb = ni_1[ind];
        int sc = 0;
        for (int comp = 0; comp < 3; comp++) {
          const long long fi = 3 * ind + comp;
          const double f1 = force_dot_1[fi * N2s + j] / norm_ij;
          const double f2 = dv * sfd_1[fi] / (norm_j * norm_i3);
          const double fk = sig_sq * c2 * (f1 - f2);
          K(1 + 3 * nb + comp, 0) -= fk;
          K(1 + 3 * c_ind_1 + comp, 0) += fk;
          for (int comp2 = comp; comp2 < 3; comp2++) {
            K(s1 + sc, 0) -= fk * co_1[ind * 3 + comp2] * vol_inv_1;
            sc++;
          }
        }
      }
      // force / force, force / stress, stress / force, stress / stress
      for (int k = 0; k < n_neigh_1; k++) {
        const long long ind1 = c_neigh_1 + k;
        const int n_ind_1 = ni_1[ind1];
        for (int l = 0; l < n_neigh_2; l++) {
          const long long ind2 = c_neigh_2 + l;
          const int n_ind_2 = ni_2[ind2];
          for (int m = 0; m < 3; m++) {
            const long long f_ind_1 = 3 * ind1 + m;
            for (int n = 0; n < 3; n++) {
              const long long f_ind_2 = 3 * ind2 + n;
              const double v1 = force_dot_1[f_ind_1 * N2s + j] / norm_ij -
                                norm_dot * sfd_1[f_ind_1] / norm_i2;
              const double v2 = force_dot_2[f_ind_2 * N1s + i] / norm_ij -
                                norm_dot * sfd_2[f_ind_2] / norm_j2;
              const double v3 = force_force[f_ind_1 * fc2 + f_ind_2] / norm_ij;
              const double v4 = sfd_1[f_ind_1] * force_dot_2[f_ind_2 * N1s + i] /
                                (norm_i3 * norm_j);
              const double v5 = sfd_2[f_ind_2] * force_dot_1[f_ind_1 * N2s + j] /
                                (norm_i * norm_j3);
              const double v6 = sfd_1[f_ind_1] * sfd_2[f_ind_2] * norm_dot /
                                (norm_i2 * norm_j2);
              const double kv =
                  sig_sq * (c1 * v1 * v2 + c2 * (v3 - v4 - v5 + v6));
              K(1 + c_ind_1 * 3 + m, 1 + c_ind_2 * 3 + n) += kv;
              K(1 + c_ind_1 * 3 + m, 1 + n_ind_2 * 3 + n) -= kv;
              K(1 + n_ind_1 * 3 + m, 1 + c_ind_2 * 3 + n) -= kv;
              K(1 + n_ind_1 * 3 + m, 1 + n_ind_2 * 3 + n) += kv;
              int si = stress_inds[m];
              for (int p = m; p < 3; p++) {
                const double x1 = co_1[ind1 * 3 + p];
                K(s1 + si, 1 + c_ind_2 * 3 + n) -= kv * x1 * vol_inv_1;
                K(s1 + si, 1 + n_ind_2 * 3 + n) += kv * x1 * vol_inv_1;
                si++;
              }
              int sj = stress_inds[n];
              for (int p = n; p < 3; p++) {
                const double x2 = co_2[ind2 * 3 + p];
                K(1 + c_ind_1 * 3 + m, s2 + sj) -= kv * x2 * vol_inv_2;
                K(1 + n_ind_1 * 3 + m, s2 + sj) += kv * x2 * vol_inv_2;
                sj++;
              }
              si = stress_inds[m];
              for (int p = m; p < 3; p++) {
                const double x1 = co_1[ind1 * 3 + p];
                sj = stress_inds[n];
                for (int q = n; q < 3; q++) {
                  const double x2 = co_2[ind2 * 3 + q];
                  K(s1 + si, s2 + sj) += kv * x1 * x2 * vol_inv_1 * vol_inv_2;
                  sj++;
                }
                si++;
              }
            }
          }
        }
      }
    }
  }
  return 0;
}

}  // extern "C"
