// Uncertainty-aware molecular dynamics on the device (the ensemble workload
// an OTF learner runs with the sparse-GP forces; flare/learners/otf.py:
// 507-521 calls SGP_Calculator per step on the host, here every replica
// lives on the GPU and all of them are predicted in one batched call).
//
// R replicas of N atoms each (own cells and species), velocity Verlet:
//   v += F/m dt/2;  x += v dt;  F, var = model(x);  v += F/m dt/2
// Units: positions A, velocities A/fs, masses amu, forces eV/A, energies eV;
// F/m in A/fs^2 = F[eV/A] / m[amu] * 9.64853321e-3 (CODATA eV, amu).
// After each step the local std of every atom, sign(v) sqrt|v| / |sigma|
// (the reference calculator's normalisation, calculator.py:121), is compared
// with a threshold and counted per replica; kinetic energies are summed per
// replica.  Reductions run in a fixed order and counters are integers: a
// replica's trajectory is the same alone and in the ensemble.
#include "fgb_internal.h"
#include "fgb_model.h"

namespace fgb {
namespace {

constexpr double kAccel = 9.64853321e-3;   // (eV/A)/amu in A/fs^2

// v += F/m h;  if dt != 0 then x += v dt
__global__ void k_vv(long long n3, const int *__restrict__ species,
                     const double *__restrict__ inv_mass, double h, double dt,
                     const double *__restrict__ F, double *__restrict__ v,
                     double *__restrict__ x) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n3) return;
  const double a = F[e] * inv_mass[species[e / 3]] * kAccel;
  const double vn = v[e] + a * h;
  v[e] = vn;
  if (dt != 0.0) x[e] += vn * dt;
}

// Block per replica: atoms whose local std exceeds `thresh` (added to the
// replica's running count), kinetic energy, largest std of this state.
__global__ void k_observe(int N, const int *__restrict__ species,
                          const double *__restrict__ mass,
                          const double *__restrict__ v,
                          const double *__restrict__ var, double inv_sig,
                          double thresh, long long *__restrict__ flagged,
                          double *__restrict__ kinetic,
                          double *__restrict__ max_std) {
  __shared__ double red_k[256], red_m[256];
  __shared__ int red_c[256];
  const int r = blockIdx.x, t = threadIdx.x;
  const long long a0 = (long long)r * N;
  double ke = 0.0, mx = -1e300;
  int c = 0;
  for (int i = t; i < N; i += blockDim.x) {
    const long long a = a0 + i;
    const double m = mass[species[a]];
    const double vx = v[3 * a], vy = v[3 * a + 1], vz = v[3 * a + 2];
    ke += 0.5 * m * (vx * vx + vy * vy + vz * vz) / kAccel;
    const double s = var[a];
    const double sd = (s >= 0.0 ? sqrt(s) : -sqrt(-s)) * inv_sig;
    mx = fmax(mx, sd);
    c += sd > thresh ? 1 : 0;
  }
  red_k[t] = ke;
  red_m[t] = mx;
  red_c[t] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (t < s) {
      red_k[t] += red_k[t + s];
      red_m[t] = fmax(red_m[t], red_m[t + s]);
      red_c[t] += red_c[t + s];
    }
    __syncthreads();
  }
  if (t == 0) {
    flagged[r] += red_c[0];
    kinetic[r] = red_k[0];
    max_std[r] = red_m[0];
  }
}

}  // namespace
}  // namespace fgb

using namespace fgb;

struct fgb_md_s {
  fgb_model_s *model = nullptr;
  int R = 0, N = 0;
  double cutoff = 0.0;
  int precision = FGB_PREC_MIXED;
  std::vector<int> h_offsets;      // R + 1
  std::vector<double> h_cells;     // 9 R
  DevBuf pos, vel, force, species, mass, inv_mass, energy, var, flagged,
      kinetic, max_std;
  bool have_forces = false;
};

static int md_forces(fgb_md_s *md, cudaStream_t st) {
  const int want = FGB_WANT_ENERGY | FGB_WANT_FORCES | FGB_WANT_LOCAL_VAR;
  int rc = predict_impl(md->model, md->R, md->h_offsets.data(),
                        md->h_cells.data(), md->pos.as<double>(),
                        md->species.as<int>(), md->cutoff, want,
                        md->precision, md->energy.as<double>(),
                        md->force.as<double>(), nullptr, md->var.as<double>(),
                        st);
  if (rc) return rc;
  md->have_forces = true;
  return FGB_OK;
}

static int md_observe(fgb_md_s *md, double thresh, cudaStream_t st) {
  k_observe<<<md->R, 256, 0, st>>>(
      md->N, md->species.as<int>(), md->mass.as<double>(),
      md->vel.as<double>(), md->var.as<double>(),
      1.0 / std::fabs(md->model->sigma), thresh, md->flagged.as<long long>(),
      md->kinetic.as<double>(), md->max_std.as<double>());
  FGB_LAUNCH_CHECK("k_observe");
  return FGB_OK;
}

extern "C" int fgb_md_create(fgb_md_t *out, fgb_model_t model, int n_replicas,
                             int n_atoms, const double *h_cells,
                             const double *h_positions,
                             const double *h_velocities, const int *h_species,
                             const double *h_masses, double cutoff,
                             int precision) {
  if (!out || !model || n_replicas <= 0 || n_atoms <= 0 || !h_cells ||
      !h_positions || !h_velocities || !h_species || !h_masses) {
    set_error("fgb_md_create: invalid arguments");
    return FGB_EINVAL;
  }
  if (precision != FGB_PREC_FP64 && precision != FGB_PREC_MIXED) {
    set_error("fgb_md_create: unknown precision %d", precision);
    return FGB_EINVAL;
  }
  if ((long long)n_replicas * n_atoms > (1LL << 24)) {
    set_error("fgb_md_create: at most 2^24 atoms in an ensemble");
    return FGB_EINVAL;
  }
  const int S = model->b2.n_species;
  for (int s = 0; s < S; s++)
    if (!(h_masses[s] > 0.0) || !std::isfinite(h_masses[s])) {
      set_error("fgb_md_create: masses must be positive");
      return FGB_EINVAL;
    }
  const long long NT = (long long)n_replicas * n_atoms;
  for (long long a = 0; a < NT; a++)
    if (h_species[a] < 0 || h_species[a] >= S) {
      set_error("fgb_md_create: species must lie in [0, %d)", S);
      return FGB_EINVAL;
    }
  auto *md = new fgb_md_s();
  md->model = model;
  md->R = n_replicas;
  md->N = n_atoms;
  md->cutoff = cutoff;
  md->precision = precision;
  md->h_offsets.resize(n_replicas + 1);
  for (int r = 0; r <= n_replicas; r++) md->h_offsets[r] = r * n_atoms;
  md->h_cells.assign(h_cells, h_cells + 9 * (size_t)n_replicas);
  std::vector<double> inv(S);
  for (int s = 0; s < S; s++) inv[s] = 1.0 / h_masses[s];
  int rc;
  if ((rc = md->pos.ensure(sizeof(double) * 3 * NT)) ||
      (rc = md->vel.ensure(sizeof(double) * 3 * NT)) ||
      (rc = md->force.ensure(sizeof(double) * 3 * NT)) ||
      (rc = md->species.ensure(sizeof(int) * NT)) ||
      (rc = md->mass.ensure(sizeof(double) * S)) ||
      (rc = md->inv_mass.ensure(sizeof(double) * S)) ||
      (rc = md->energy.ensure(sizeof(double) * n_replicas)) ||
      (rc = md->var.ensure(sizeof(double) * NT)) ||
      (rc = md->flagged.ensure(sizeof(long long) * n_replicas)) ||
      (rc = md->kinetic.ensure(sizeof(double) * n_replicas)) ||
      (rc = md->max_std.ensure(sizeof(double) * n_replicas))) {
    delete md;
    return rc;
  }
  cudaError_t e;
  if ((e = cudaMemcpy(md->pos.p, h_positions, sizeof(double) * 3 * NT,
                      cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(md->vel.p, h_velocities, sizeof(double) * 3 * NT,
                      cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(md->species.p, h_species, sizeof(int) * NT,
                      cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(md->mass.p, h_masses, sizeof(double) * S,
                      cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(md->inv_mass.p, inv.data(), sizeof(double) * S,
                      cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(md->flagged.p, 0, sizeof(long long) * n_replicas)) !=
          cudaSuccess) {
    delete md;
    return cuda_status(e, "fgb_md_create");
  }
  *out = md;
  return FGB_OK;
}

extern "C" int fgb_md_destroy(fgb_md_t md) {
  delete md;
  return FGB_OK;
}

extern "C" int fgb_md_set_model(fgb_md_t md, fgb_model_t model) {
  if (!md || !model || model->b2.n_species != md->model->b2.n_species) {
    set_error("fgb_md_set_model: invalid arguments");
    return FGB_EINVAL;
  }
  md->model = model;
  md->have_forces = false;   // recomputed at the next step
  return FGB_OK;
}

extern "C" int fgb_md_step(fgb_md_t md, int n_steps, double dt,
                           double std_threshold, void *stream) {
  if (!md || n_steps < 0 || !(dt > 0.0) || !std::isfinite(dt)) {
    set_error("fgb_md_step: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const long long n3 = 3LL * md->R * md->N;
  const int T = 256;
  int rc;
  if (!md->have_forces && (rc = md_forces(md, st))) return rc;
  for (int k = 0; k < n_steps; k++) {
    k_vv<<<ceil_div(n3, T), T, 0, st>>>(n3, md->species.as<int>(),
                                        md->inv_mass.as<double>(), 0.5 * dt,
                                        dt, md->force.as<double>(),
                                        md->vel.as<double>(),
                                        md->pos.as<double>());
    FGB_LAUNCH_CHECK("k_vv");
    if ((rc = md_forces(md, st))) return rc;
    k_vv<<<ceil_div(n3, T), T, 0, st>>>(n3, md->species.as<int>(),
                                        md->inv_mass.as<double>(), 0.5 * dt,
                                        0.0, md->force.as<double>(),
                                        md->vel.as<double>(), nullptr);
    FGB_LAUNCH_CHECK("k_vv");
    if ((rc = md_observe(md, std_threshold, st))) return rc;
  }
  return FGB_OK;
}

extern "C" int fgb_md_read(fgb_md_t md, double *h_positions,
                           double *h_velocities, double *h_forces,
                           double *h_local_var, double *h_energy,
                           double *h_kinetic, double *h_max_std,
                           long long *h_flagged, void *stream) {
  if (!md) {
    set_error("fgb_md_read: null handle");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc;
  if (!md->have_forces && (rc = md_forces(md, st))) return rc;
  // kinetic energies and largest std of the current state (no flag counts)
  if ((rc = md_observe(md, HUGE_VAL, st))) return rc;
  const long long NT = (long long)md->R * md->N;
  struct Out { void *dst; const DevBuf *src; size_t bytes; };
  const Out outs[] = {
      {h_positions, &md->pos, sizeof(double) * 3 * NT},
      {h_velocities, &md->vel, sizeof(double) * 3 * NT},
      {h_forces, &md->force, sizeof(double) * 3 * NT},
      {h_local_var, &md->var, sizeof(double) * NT},
      {h_energy, &md->energy, sizeof(double) * md->R},
      {h_kinetic, &md->kinetic, sizeof(double) * md->R},
      {h_max_std, &md->max_std, sizeof(double) * md->R},
      {h_flagged, &md->flagged, sizeof(long long) * md->R}};
  for (const Out &o : outs)
    if (o.dst)
      FGB_CUDA(cudaMemcpyAsync(o.dst, o.src->p, o.bytes, cudaMemcpyDeviceToHost,
                               st));
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}
