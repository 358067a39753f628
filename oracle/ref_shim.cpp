// C entry points over the reference's own compiled per-pair math
// (src/flare_pp/radial.cpp, cutoffs.cpp, y_grad.cpp), used only to generate
// the golden vectors in tests/golden/ that pin the oracle's restatement.
#include <string>
#include <vector>
#include "cutoffs.h"
#include "radial.h"
#include "y_grad.h"

extern "C" {

void ref_get_Y(double x, double y, double z, int l, double *Y, double *Yx,
               double *Yy, double *Yz) {
  int n = (l + 1) * (l + 1);
  std::vector<double> a(n), b(n), c(n), d(n);
  get_Y(a, b, c, d, x, y, z, l);
  for (int i = 0; i < n; i++) {
    Y[i] = a[i]; Yx[i] = b[i]; Yy[i] = c[i]; Yz[i] = d[i];
  }
}

// calculate_radial (radial.cpp:344) for a named basis and cutoff.
void ref_calculate_radial(const char *basis, const char *cutoff, double x,
                          double y, double z, double r, double rcut, int N,
                          const double *radial_hyps, int n_rh,
                          const double *cutoff_hyps, int n_ch, double *g,
                          double *gx, double *gy, double *gz) {
  std::function<void(std::vector<double> &, std::vector<double> &, double, int,
                     std::vector<double>)> rp;
  std::function<void(std::vector<double> &, double, double,
                     std::vector<double>)> cp;
  set_radial_basis(basis, rp);
  set_cutoff(cutoff, cp);
  std::vector<double> a(N), b(N), c(N), d(N);
  std::vector<double> rh(radial_hyps, radial_hyps + n_rh);
  std::vector<double> ch(cutoff_hyps, cutoff_hyps + n_ch);
  calculate_radial(a, b, c, d, rp, cp, x, y, z, r, rcut, N, rh, ch);
  for (int i = 0; i < N; i++) {
    g[i] = a[i]; gx[i] = b[i]; gy[i] = c[i]; gz[i] = d[i];
  }
}
}
