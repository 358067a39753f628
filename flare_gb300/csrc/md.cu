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
//
// Replayed steps.  Atoms, species and cells do not change between steps, so
// after one full step the step is captured once as a CUDA graph (the
// prediction in its fixed form: neighbour list rebuilt into a reserved pair
// capacity, species permutation and geometry reused, no host
// synchronisation) and replayed.  Device error flags of every replayed
// step are ORed into a status word read once per chunk of steps; a chunk
// that overflowed the pair capacity or raised any flag is rolled back to a
// snapshot taken before it and redone with full, checked steps, after which
// the capacity is re-planned and the step captured again.  Replayed and
// full steps run the same kernels on the same data: the trajectories are
// identical.  The ensemble predicts with a private replica of the model, so
// the buffers a captured graph refers to belong to it alone.
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

// Sticky status of replayed steps: bit 0 neighbour-list flags (non-finite
// positions, fill or twin inconsistency), bit 1 pair capacity exceeded,
// bit 2 a bounded tensor-core wait ran out.
__global__ void k_collect(const int *__restrict__ nl_flag,
                          const int *__restrict__ ozerr,
                          int *__restrict__ status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int s = 0;
  if (nl_flag[0] | nl_flag[1] | nl_flag[2]) s |= 1;
  if (nl_flag[3]) s |= 2;
  if (ozerr[0]) s |= 4;
  if (s) atomicOr(status, s);
}

constexpr int kChunk = 50;   // replayed steps per status read

}  // namespace
}  // namespace fgb

using namespace fgb;

struct fgb_md_s {
  fgb_model_s *model = nullptr;    // private replica of the caller's model
  int R = 0, N = 0;
  double cutoff = 0.0;
  int precision = FGB_PREC_MIXED;
  std::vector<int> h_offsets;      // R + 1
  std::vector<double> h_cells;     // 9 R
  DevBuf pos, vel, force, species, mass, inv_mass, energy, var, flagged,
      kinetic, max_std;
  bool have_forces = false;
  // replayed steps
  bool graphs = true;
  double pair_margin = 0.25;       // capacity = pairs of the last full step x (1 + margin) + 4096
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  double g_dt = 0.0, g_thresh = 0.0;
  unsigned long long g_allocs = 0;  // allocation count when captured
  FixedPlan plan;
  bool planned = false;
  DevBuf status, s_pos, s_vel, s_force, s_energy, s_var, s_flagged, s_kinetic,
      s_max_std;
  long long n_replayed = 0, n_full = 0, n_captures = 0, n_rollbacks = 0;

  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
  ~fgb_md_s() {
    drop_graph();
    if (cap_stream) cudaStreamDestroy(cap_stream);
    delete model;
  }
};

// Forces, energies and variances at the current positions: the full,
// checked prediction, or (plan given) the fixed one.
static int md_forces(fgb_md_s *md, cudaStream_t st,
                     const FixedPlan *plan = nullptr) {
  const int want = FGB_WANT_ENERGY | FGB_WANT_FORCES | FGB_WANT_LOCAL_VAR;
  int rc = predict_impl(md->model, md->R, md->h_offsets.data(),
                        md->h_cells.data(), md->pos.as<double>(),
                        md->species.as<int>(), md->cutoff, want,
                        md->precision, md->energy.as<double>(),
                        md->force.as<double>(), nullptr, md->var.as<double>(),
                        st, plan);
  if (rc) return rc;
  if (!plan) md->planned = false;   // a full build may have moved buffers
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
  int rc = FGB_OK;
  if (!(md->model = model_replicate(model, rc))) {
    delete md;
    return rc;
  }
  md->R = n_replicas;
  md->N = n_atoms;
  md->cutoff = cutoff;
  md->precision = precision;
  md->h_offsets.resize(n_replicas + 1);
  for (int r = 0; r <= n_replicas; r++) md->h_offsets[r] = r * n_atoms;
  md->h_cells.assign(h_cells, h_cells + 9 * (size_t)n_replicas);
  std::vector<double> inv(S);
  for (int s = 0; s < S; s++) inv[s] = 1.0 / h_masses[s];
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
      (rc = md->max_std.ensure(sizeof(double) * n_replicas)) ||
      (rc = md->status.ensure(sizeof(int)))) {
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
  int rc = FGB_OK;
  fgb_model_s *rep = model_replicate(model, rc);
  if (!rep) return rc;
  md->drop_graph();
  delete md->model;
  md->model = rep;
  md->planned = false;
  md->have_forces = false;   // recomputed at the next step
  return FGB_OK;
}

extern "C" int fgb_md_set_graphs(fgb_md_t md, int enable, double pair_margin) {
  if (!md || !(pair_margin > -0.5) || !(pair_margin <= 16.0)) {
    set_error("fgb_md_set_graphs: invalid arguments");
    return FGB_EINVAL;
  }
  md->graphs = enable != 0;
  md->pair_margin = pair_margin;
  md->planned = false;
  md->drop_graph();
  return FGB_OK;
}

extern "C" int fgb_md_stats(fgb_md_t md, long long *out4) {
  if (!md || !out4) {
    set_error("fgb_md_stats: invalid arguments");
    return FGB_EINVAL;
  }
  out4[0] = md->n_replayed;
  out4[1] = md->n_full;
  out4[2] = md->n_captures;
  out4[3] = md->n_rollbacks;
  return FGB_OK;
}

// One velocity-Verlet step; `plan` selects the fixed prediction (then the
// step's device flags are collected into md->status).
static int md_step_once(fgb_md_s *md, double dt, double thresh,
                        cudaStream_t st, const FixedPlan *plan) {
  const long long n3 = 3LL * md->R * md->N;
  const int T = 256;
  int rc;
  if (plan)
    FGB_CUDA(cudaMemsetAsync(md->model->ws.ozerr.p, 0, sizeof(int), st));
  k_vv<<<ceil_div(n3, T), T, 0, st>>>(n3, md->species.as<int>(),
                                      md->inv_mass.as<double>(), 0.5 * dt, dt,
                                      md->force.as<double>(),
                                      md->vel.as<double>(),
                                      md->pos.as<double>());
  FGB_LAUNCH_CHECK("k_vv");
  if ((rc = md_forces(md, st, plan))) return rc;
  if (plan) {
    k_collect<<<1, 32, 0, st>>>(md->model->nl.flag.as<int>(),
                                md->model->ws.ozerr.as<int>(),
                                md->status.as<int>());
    FGB_LAUNCH_CHECK("k_collect");
  }
  k_vv<<<ceil_div(n3, T), T, 0, st>>>(n3, md->species.as<int>(),
                                      md->inv_mass.as<double>(), 0.5 * dt, 0.0,
                                      md->force.as<double>(),
                                      md->vel.as<double>(), nullptr);
  FGB_LAUNCH_CHECK("k_vv");
  return md_observe(md, thresh, st);
}

// Pair capacity and buffers for fixed steps, from the last full step.
static int md_plan(fgb_md_s *md) {
  fgb_model_s *m = md->model;
  const long long P = m->nl.n_pairs;
  long long cap = (long long)std::ceil((double)P * (1.0 + md->pair_margin));
  if (md->pair_margin >= 0.0) cap += 4096;
  cap = std::max(cap, 1LL);
  int rc;
  if ((rc = nlist_reserve(&m->nl, cap)) ||
      (rc = m->ws.pair_grad.ensure(sizeof(double3) * (cap + 1))) ||
      (rc = m->ws.ozerr.ensure(sizeof(int))))
    return rc;
  const long long NT = (long long)md->R * md->N;
  const struct { DevBuf *b; size_t n; } snaps[] = {
      {&md->s_pos, sizeof(double) * 3 * NT},
      {&md->s_vel, sizeof(double) * 3 * NT},
      {&md->s_force, sizeof(double) * 3 * NT},
      {&md->s_energy, sizeof(double) * md->R},
      {&md->s_var, sizeof(double) * NT},
      {&md->s_flagged, sizeof(long long) * md->R},
      {&md->s_kinetic, sizeof(double) * md->R},
      {&md->s_max_std, sizeof(double) * md->R}};
  for (const auto &q : snaps)
    if ((rc = q.b->ensure(q.n))) return rc;
  md->plan.pair_cap = cap;
  md->plan.counts = m->last_species_counts;
  md->planned = true;
  md->drop_graph();
  return FGB_OK;
}

// Capture one fixed step on the ensemble's own stream.
static int md_capture(fgb_md_s *md, double dt, double thresh) {
  if (!md->cap_stream)
    FGB_CUDA(cudaStreamCreateWithFlags(&md->cap_stream, cudaStreamNonBlocking));
  md->drop_graph();
  for (int attempt = 0; attempt < 2; attempt++) {
    const unsigned long long a0 = devbuf_allocations();
    FGB_CUDA(cudaStreamBeginCapture(md->cap_stream,
                                    cudaStreamCaptureModeRelaxed));
    const int rc = md_step_once(md, dt, thresh, md->cap_stream, &md->plan);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(md->cap_stream, &g);
    if (rc || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      if (rc) return rc;
      return cuda_status(e, "fgb_md_step: graph capture");
    }
    if (devbuf_allocations() != a0) {   // a buffer moved while recording
      cudaGraphDestroy(g);
      continue;
    }
    const cudaError_t ei = cudaGraphInstantiate(&md->exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      md->exec = nullptr;
      return cuda_status(ei, "fgb_md_step: graph instantiation");
    }
    md->g_dt = dt;
    md->g_thresh = thresh;
    md->g_allocs = a0;
    md->n_captures++;
    return FGB_OK;
  }
  set_error("fgb_md_step: buffers kept growing during graph capture");
  return FGB_ECUDA;
}

// Copies between the state and its snapshot (to_snap: state -> snapshot).
static int md_snapshot(fgb_md_s *md, bool to_snap, cudaStream_t st) {
  const long long NT = (long long)md->R * md->N;
  const struct { DevBuf *a, *b; size_t n; } pairs[] = {
      {&md->pos, &md->s_pos, sizeof(double) * 3 * NT},
      {&md->vel, &md->s_vel, sizeof(double) * 3 * NT},
      {&md->force, &md->s_force, sizeof(double) * 3 * NT},
      {&md->energy, &md->s_energy, sizeof(double) * md->R},
      {&md->var, &md->s_var, sizeof(double) * NT},
      {&md->flagged, &md->s_flagged, sizeof(long long) * md->R},
      {&md->kinetic, &md->s_kinetic, sizeof(double) * md->R},
      {&md->max_std, &md->s_max_std, sizeof(double) * md->R}};
  for (const auto &q : pairs)
    FGB_CUDA(cudaMemcpyAsync(to_snap ? q.b->p : q.a->p,
                             to_snap ? q.a->p : q.b->p, q.n,
                             cudaMemcpyDeviceToDevice, st));
  return FGB_OK;
}

extern "C" int fgb_md_step(fgb_md_t md, int n_steps, double dt,
                           double std_threshold, void *stream) {
  if (!md || n_steps < 0 || !(dt > 0.0) || !std::isfinite(dt)) {
    set_error("fgb_md_step: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc;
  if (!md->have_forces && (rc = md_forces(md, st))) return rc;
  int k = 0;
  while (k < n_steps) {
    if (!md->graphs) {
      if ((rc = md_step_once(md, dt, std_threshold, st, nullptr))) return rc;
      md->n_full++;
      k++;
      continue;
    }
    if (!md->planned && (rc = md_plan(md))) return rc;
    if (!md->exec || md->g_dt != dt || md->g_thresh != std_threshold ||
        md->g_allocs != devbuf_allocations())
      if ((rc = md_capture(md, dt, std_threshold))) return rc;
    const int c = std::min(kChunk, n_steps - k);
    if ((rc = md_snapshot(md, true, st))) return rc;
    FGB_CUDA(cudaMemsetAsync(md->status.p, 0, sizeof(int), st));
    for (int q = 0; q < c; q++) FGB_CUDA(cudaGraphLaunch(md->exec, st));
    int h = 0;
    FGB_CUDA(cudaMemcpyAsync(&h, md->status.p, sizeof(int),
                             cudaMemcpyDeviceToHost, st));
    FGB_CUDA(cudaStreamSynchronize(st));
    if (h == 0) {
      md->n_replayed += c;
      k += c;
      continue;
    }
    // redo the chunk with full, checked steps from the snapshot
    md->n_rollbacks++;
    if ((rc = md_snapshot(md, false, st))) return rc;
    for (int q = 0; q < c; q++) {
      if ((rc = md_step_once(md, dt, std_threshold, st, nullptr))) return rc;
      md->n_full++;
    }
    k += c;
    if ((rc = md_plan(md))) return rc;   // capacity from the latest pairs
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
