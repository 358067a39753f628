/*
 * libflaregb — GB300-native (sm_103a) sparse-GP prediction for FLARE's
 * B2 / NormalizedDotProduct / SparseGP path, behind a plain C ABI.
 *
 * Every entry point returns an int status (FGB_OK = 0) and never aborts;
 * fgb_last_error() returns the message of the last failure on this thread.
 * Pointers named d_* are device pointers on the current CUDA device, h_* are
 * host pointers.  `stream` is a cudaStream_t passed as void* (NULL = legacy
 * default stream).  No entry point takes or returns framework (torch) types.
 *
 * Reference interfaces replaced (paths inside mir-group/flare):
 *   Structure(cell, species, positions, cutoff, descriptors)
 *       src/flare_pp/structure.cpp:27-118, bound at src/ace_binding.cpp:30-35
 *   B2(radial_basis, cutoff_function, radial_hyps, cutoff_hyps, settings[, cutoffs])
 *       src/flare_pp/descriptors/b2.cpp:13-50,76-242, bound at src/ace_binding.cpp:125-138
 *   NormalizedDotProduct(sigma, power).envs_struc / envs_envs
 *       src/flare_pp/kernels/normalized_dot_product.cpp:15-214, bound at src/ace_binding.cpp:168-176
 *   SparseGP.update_matrices_QR / predict_{mean,SOR,local_uncertainties}
 *       src/flare_pp/bffs/sparse_gp.cpp:607-757, bound at src/ace_binding.cpp:195-213
 */
#ifndef FLAREGB_H
#define FLAREGB_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- status */
enum {
  FGB_OK = 0,
  FGB_EINVAL = 1,   /* bad argument (reference: std::invalid_argument)     */
  FGB_ENOMEM = 2,   /* device allocation failed                            */
  FGB_ECUDA = 3,    /* CUDA runtime / library error                        */
  FGB_ETIMEOUT = 4, /* a bounded device wait ran out                       */
  FGB_ESTALE = 5,   /* model weights not solved (reference: runtime_error
                       "L_inv must be up to date", sparse_gp.cpp:644-649)  */
  FGB_ENOTSUP = 6   /* valid in the reference but not built here           */
};

/* radial bases (radial.cpp:381-408) and cutoffs (cutoffs.cpp:87-103) */
enum {
  FGB_RADIAL_CHEBYSHEV = 0,
  FGB_RADIAL_WEIGHTED_CHEBYSHEV = 1,          /* radial_hyps[2] = lambda */
  FGB_RADIAL_EQUISPACED_GAUSSIANS = 2,        /* [sigma, first, final]   */
  FGB_RADIAL_WEIGHTED_POSITIVE_CHEBYSHEV = 3, /* radial_hyps[2] = lambda */
  FGB_RADIAL_POSITIVE_CHEBYSHEV = 4,
  FGB_RADIAL_BESSEL = 5,
  FGB_RADIAL_FOURIER_QUARTER = 6,
  FGB_RADIAL_FOURIER_HALF = 7,
  FGB_RADIAL_FOURIER = 8                      /* radial_hyps[2] = factor */
};
enum {
  FGB_CUTOFF_QUADRATIC = 0,
  FGB_CUTOFF_HARD = 1,
  FGB_CUTOFF_COSINE = 2,
  FGB_CUTOFF_POLYNOMIAL = 3,
  FGB_CUTOFF_POWER = 4
};

/* prediction precision */
enum {
  FGB_PREC_FP64 = 0,  /* FP64 adjoint path                                   */
  FGB_PREC_MIXED = 1  /* double-float descriptors, tensor-core kernel and
                         variance GEMMs by exact slicing to 54 down to 42
                         and 36 bits (fgb_model_slice_plan), FP32-level
                         tensor-core force GEMM and FP32 adjoint; models
                         whose largest folded coefficient exceeds 200
                         (fgb_model_fold_guard) get the force stage at
                         FP64 level instead                                  */
};

/* prediction outputs */
enum {
  FGB_WANT_ENERGY = 1,
  FGB_WANT_FORCES = 2,
  FGB_WANT_STRESS = 4,
  FGB_WANT_LOCAL_VAR = 8
};

const char *fgb_last_error(void);
int fgb_version(void);

/* ------------------------------------------------------ stage profiler
 * When enabled, every kernel launch of the prediction pipeline is bracketed
 * by CUDA events on its launch stream.  fgb_profile_read synchronises those
 * events and returns, per stage, the summed device time (ms) and the launch
 * count since the last reset.  Stage names: fgb_profile_stage_name(i). */
int fgb_profile_enable(int on);
int fgb_profile_reset(void);
int fgb_profile_n_stages(void);
const char *fgb_profile_stage_name(int stage);
int fgb_profile_read(double *ms, long long *launches, int n);

/* ----------------------------------------------------- neighbour list
 * Cell-list neighbour build for a batch of periodic structures.  Replaces
 * Structure::compute_neighbors (structure.cpp:52-118): the same pairs
 * (0 < d < cutoff, image shifts |s| <= sweep with sweep from
 * get_single_sweep_cutoff, structure.cpp:35,135-165), in the reference's
 * order (i, then j ascending, then s1, s2, s3 ascending), with relative
 * vectors computed in the same FP64 operation order, so the lists are
 * bit-exact against the reference.  Structures are packed: structure s owns
 * atoms [h_atom_offsets[s], h_atom_offsets[s+1]).
 */
typedef struct fgb_nlist_s *fgb_nlist_t;
int fgb_nlist_create(fgb_nlist_t *out);
int fgb_nlist_destroy(fgb_nlist_t nl);
int fgb_nlist_build(fgb_nlist_t nl, int n_struc, const int *h_atom_offsets,
                    const double *h_cells, const double *d_positions,
                    double cutoff, void *stream);
/* total pairs and atoms of the last build (fgb_nlist_build returns after
 * its checks, so the count is exact; the build fills per-atom slots in one
 * pass and falls back to a counting pass when an atom has more pairs than
 * its slots) */
int fgb_nlist_size(fgb_nlist_t nl, long long *n_pairs, int *n_atoms);
/* Copy out in the reference's Structure layout (device pointers; any may be
 * NULL): neighbor_count[N], structure_indices[P] (index within the
 * structure), shifts[P*3], relative_positions[P*4] = (d, x, y, z),
 * wrapped_positions[N*3]. */
int fgb_nlist_export(fgb_nlist_t nl, int *d_neighbor_count,
                     int *d_structure_indices, int *d_shifts,
                     double *d_relative_positions, double *d_wrapped,
                     void *stream);

/* The neighbour list of ONE structure written into caller-owned device
 * buffers, with no device allocation at all.  No counterpart in the
 * reference; it serves callers that cannot allocate device memory (for
 * example a host program that owns a fixed device-memory budget, or a loop
 * that must not allocate between steps).  Working memory is a fixed
 * FGB_NOALLOC_SCRATCH_BYTES array that every GPU loading the library holds
 * until exit.  Limits: n_atoms <= FGB_NOALLOC_MAX_ATOMS and at most
 * FGB_NOALLOC_MAX_PAIRS pairs; larger inputs return FGB_EINVAL with a
 * message.  Outputs as in fgb_nlist_export (d_shifts may be NULL;
 * d_relative_positions 16-byte aligned); *h_n_pairs receives the pair count
 * (also when it exceeds max_pairs, so the caller can grow its buffers).
 * Each call looks up the array's device address in the current context;
 * the first call on each device also loads the module, so make that first
 * call before any stream capture.  The call synchronises `stream` twice (to
 * read the pair count, and to read the consistency flags at the end), so
 * it returns with its outputs complete.  Calls share the array, so calls
 * that overlap on the GPU race and must be serialised (for example on one
 * stream); calls in sequence are independent. */
#define FGB_NOALLOC_MAX_ATOMS 8192
#define FGB_NOALLOC_MAX_PAIRS 262144
#define FGB_NOALLOC_SCRATCH_BYTES (24u << 20)
int fgb_nlist_build_noalloc(const double *h_cell, const double *d_positions,
                            int n_atoms, double cutoff, long long max_pairs,
                            int *d_neighbor_count, int *d_structure_indices,
                            int *d_shifts, double *d_relative_positions,
                            long long *h_n_pairs, void *stream);

/* ------------------------------------------------------- B2 descriptor
 * B2(radial_basis, cutoff_function, radial_hyps, cutoff_hyps,
 *    [n_species, n_max, l_max], cutoffs[n_species^2]) — b2.cpp:13-50.
 * radial_hyps = [r1, r2(, ...)]; cutoffs == NULL means r2 for every pair.
 */
typedef struct fgb_b2_s *fgb_b2_t;
int fgb_b2_create(fgb_b2_t *out, int radial_basis, int cutoff_function,
                  const double *radial_hyps, int n_radial_hyps,
                  const double *cutoff_hyps, int n_cutoff_hyps, int n_species,
                  int n_max, int l_max, const double *h_cutoffs);
int fgb_b2_destroy(fgb_b2_t b2);
int fgb_b2_size(fgb_b2_t b2, int *n_descriptors, int *n_single_bond);

/* B2 values and norms in atom order (B2::compute_struc values,
 * b2.cpp:181-242 without the stored gradients): d_B2[N * n_d], d_norms[N].
 * d_species[N] are the coded species (0..n_species-1). */
int fgb_b2_forward(fgb_b2_t b2, fgb_nlist_t nl, const int *d_species,
                   double *d_B2, double *d_norms, void *stream);

/* Stored forward-mode gradients, the reference's algorithm (b2.cpp:181-242):
 * over the neighbour list of `nl` (pairs filtered by the per-pair cutoff
 * get zero rows): d_dB2[3P * n_d] with row 3p+c = dB2_i/dr_ij,c and
 * d_force_dots[3P] = dB2/dr . B2. */
int fgb_b2_forward_dervs(fgb_b2_t b2, fgb_nlist_t nl, const int *d_species,
                         double *d_B2, double *d_norms, double *d_dB2,
                         double *d_force_dots, void *stream);

/* ------------------------------------------------------------- model
 * Device-resident sparse GP: B2 settings, NormalizedDotProduct(sigma,
 * power), sparse set grouped by species (sparse_gp.cpp sparse_descriptors),
 * alpha and L_inv (sparse_gp.cpp:607-641).
 */
typedef struct fgb_model_s *fgb_model_t;
int fgb_model_create(fgb_model_t *out, fgb_b2_t b2, double sigma,
                     double power);
int fgb_model_destroy(fgb_model_t m);
/* h_counts[n_species]: sparse environments per species; h_desc[M * n_d]
 * species-grouped rows (species 0 first); h_alpha[M]; h_L_inv[M * M]
 * row-major (the kernel's block of L_inv).  h_alpha/h_L_inv may be NULL to
 * load only the sparse set (model is then stale for prediction). */
int fgb_model_set(fgb_model_t m, const int *h_counts, const double *h_desc,
                  const double *h_alpha, const double *h_L_inv);

/* R_inv (sparse_gp.cpp:635, upper triangular, row-major M x M) for the SOR
 * variance. */
int fgb_model_set_R_inv(fgb_model_t m, const double *h_R_inv);

/* SparseGP::predict_SOR (sparse_gp.cpp:667-692) for ONE structure in FP64:
 * mean_efs = K^T alpha and variance_efs = diag(K^T R_inv R_inv^T K) with K
 * from envs_struc.  d_mean_efs, d_variance_efs: [1 + 3N + 6]. */
int fgb_predict_sor(fgb_model_t m, fgb_nlist_t nl, const int *d_species,
                    double *d_mean_efs, double *d_variance_efs, void *stream);

/* SparseGP::predict_DTC (sparse_gp.cpp:694-729) for ONE structure in FP64:
 * mean_efs = K^T alpha and variance_efs = K_self - diag(K^T Kuu^-1 K) +
 * diag(K^T Sigma K), Kuu^-1 = L_inv^T L_inv, Sigma = R_inv R_inv^T, K_self
 * from fgb_self_kernel_struc.  Needs fgb_model_set_R_inv.  d_mean_efs,
 * d_variance_efs: [1 + 3N + 6]. */
int fgb_predict_dtc(fgb_model_t m, fgb_nlist_t nl, const int *d_species,
                    double *d_mean_efs, double *d_variance_efs, void *stream);

/* Full prediction for a packed batch of structures (device pointers):
 * neighbours (cutoff = Structure cutoff), B2, kernel against the sparse set,
 * mean energy / forces / stress by the reverse-mode adjoint and the local
 * variance sigma^2 - |L_inv k|^2 (sparse_gp.cpp:94-139, 731-757).
 * Outputs (any may be NULL if not wanted):
 *   d_energy[n_struc], d_forces[N*3] (atom order),
 *   d_stress[n_struc*6] (flare order xx, xy, xz, yy, yz, zz: mean_efs[-6:]),
 *   d_local_var[N] (atom order; the calculator's sort_variances applied). */
int fgb_predict(fgb_model_t m, int n_struc, const int *h_atom_offsets,
                const double *h_cells, const double *d_positions,
                const int *d_species, double cutoff, int want, int precision,
                double *d_energy, double *d_forces, double *d_stress,
                double *d_local_var, void *stream);

/* Same with HOST input/output buffers: copies in, predicts, copies out on
 * `stream` and synchronises it once (the species are counted and range-
 * checked on the host; results are queued for copy-back before that
 * synchronisation).  fgb_predict waits twice: for the species counts
 * (queued before the descriptor, waited for while it runs), then for the
 * deferred checks. */
int fgb_predict_host(fgb_model_t m, int n_struc, const int *h_atom_offsets,
                     const double *h_cells, const double *h_positions,
                     const int *h_species, double cutoff, int want,
                     int precision, double *h_energy, double *h_forces,
                     double *h_stress, double *h_local_var, void *stream);

/* --------------------------------------------------- MD ensemble
 * Uncertainty-aware molecular dynamics on the device: R replicas of N atoms
 * (own cells and species, packed replica by replica) advanced together by
 * velocity Verlet with the model's forces, every replica predicted in one
 * batched call per step (precision as in fgb_predict).  No counterpart in
 * flare_pp: the reference's OTF learner (flare/learners/otf.py:507-521)
 * drives an ASE integrator on the host and calls SGP_Calculator once per
 * structure per step.  Units: A, A/fs, amu, eV; dt in fs.  After each step
 * the local std of every atom, sign(v) sqrt|v| / |sigma| (calculator.py:121),
 * is compared with std_threshold and counted per replica.  The ensemble
 * predicts with its own replica of the model (weights copied at creation
 * and at fgb_md_set_model), so the model handle stays free for other use.
 *
 * Steps after the first are captured once as a CUDA graph and replayed
 * (neighbour list rebuilt into a reserved pair capacity, no host
 * synchronisation inside a step); device error flags are read once per
 * chunk of up to 50 steps, and a chunk that exceeded the capacity or
 * raised a flag is rolled back and redone with full, checked steps.
 * Replayed and full steps give identical trajectories. */
typedef struct fgb_md_s *fgb_md_t;
int fgb_md_create(fgb_md_t *out, fgb_model_t model, int n_replicas,
                  int n_atoms, const double *h_cells, const double *h_positions,
                  const double *h_velocities, const int *h_species,
                  const double *h_masses, double cutoff, int precision);
int fgb_md_destroy(fgb_md_t md);
/* Switch to another (re-solved) model with the same species; forces are
 * recomputed at the next step. */
int fgb_md_set_model(fgb_md_t md, fgb_model_t model);
int fgb_md_step(fgb_md_t md, int n_steps, double dt, double std_threshold,
                void *stream);
/* Replayed steps on (enable != 0, the default) or off; pair capacity of a
 * replayed step = pairs of the last full step x (1 + pair_margin), plus
 * 4096 when pair_margin >= 0 (default 0.25; -0.5 < pair_margin <= 16). */
int fgb_md_set_graphs(fgb_md_t md, int enable, double pair_margin);
/* Counters since creation: replayed steps, full steps, graph captures,
 * rolled-back chunks. */
int fgb_md_stats(fgb_md_t md, long long *out4);
/* Current state to host buffers (any may be NULL): positions, velocities,
 * forces [R*N*3], local variances [R*N], potential and kinetic energies
 * [R], largest std [R], flagged atom-steps since creation [R]. */
int fgb_md_read(fgb_md_t md, double *h_positions, double *h_velocities,
                double *h_forces, double *h_local_var, double *h_energy,
                double *h_kinetic, double *h_max_std, long long *h_flagged,
                void *stream);

/* ------------------------------------------------------- mapped models
 * The mapping coefficients of a solved power-1 or power-2 model
 * (SparseGP::write_mapping_coefficients, sparse_gp.cpp:1199-1264, with
 * compute_map_coeff_pow1/pow2, normalized_dot_product.cpp:653-767): per
 * species sigma^2 sum_t alpha_t s^_t s^_t^T (power 2; n_d x n_d row-major,
 * symmetric) or sigma^2 sum_t alpha_t s^_t (power 1; n_d), FP64. */
int fgb_model_mapping(fgb_model_t m, double *h_beta, void *stream);

/* The mixed path's force-precision guard for a solved power-1 or power-2
 * model: h_fold_max = the largest |sigma^2 sum_t alpha_t s^_t s^_t^T| entry
 * (power 1: of the vector), h_fp64_forces = 1 when it exceeds 200 and the
 * mixed path's descriptor and force stage (force product, mapped gradient,
 * B2 adjoint) therefore run at FP64 level, 0 when they run in double-float
 * and at FP32 level.  Either may be NULL. */
int fgb_model_fold_guard(fgb_model_t m, double *h_fold_max,
                         int *h_fp64_forces, void *stream);

/* The mixed path's precision plan for a solved model: h_kernel_slices =
 * BF16 slices of the kernel GEMM (9, 8 or 7: 54, 48 or 42 bits) and
 * h_slice_err_est = the largest energy difference to 9 slices measured on
 * the model's sparse environments (fgb_model_slice_plan gives the variance
 * GEMM's count too); h_fold_max and h_fp64_forces as fgb_model_fold_guard.
 * Powers other than 1 and 2 run the mixed path's kernel stages in FP64 (9
 * reported).  Any output may be NULL. */
int fgb_model_mixed_plan(fgb_model_t m, int *h_kernel_slices,
                         double *h_slice_err_est, double *h_fold_max,
                         int *h_fp64_forces, void *stream);

/* The mixed path's slice counts for a solved model: h_kernel_slices (9, 8
 * or 7: the kernel GEMM c = d^ . s^, whose energies must stay within 1e-6
 * eV/atom) and h_variance_slices (9, 8, 7 or 6: the variance GEMM
 * z = L_inv k, whose local variances must stay within 1e-8 sigma^2), each
 * the fewest for which the model's own sparse environments differ from 9
 * slices by at most a tenth of the energy budget (1e-7 eV/atom) and half
 * the variance budget (5e-9 sigma^2), with those largest differences in
 * h_energy_err_est and h_var_err_est (measured once per model, before its
 * first mixed prediction; 0 when a count is forced).  Any output may be
 * NULL.  No reference counterpart. */
int fgb_model_slice_plan(fgb_model_t m, int *h_kernel_slices,
                         int *h_variance_slices, double *h_energy_err_est,
                         double *h_var_err_est, void *stream);
/* Force the slice counts (kernel 7..9, variance 6..9; 0 = chosen by the
 * probes above); kept across new weights.  No reference counterpart. */
int fgb_model_set_slices(fgb_model_t m, int kernel_slices,
                         int variance_slices);

/* Self-check of the tensor-core GEMMs' give-up path: one CTA waits (at
 * most `polls` polls, 1 <= polls <= 2^22) on a barrier that nothing arrives
 * at, raises its abort flag and reports the time-out as a GEMM does; a
 * second warp on the same barrier leaves through the abort flag.  Returns
 * FGB_ETIMEOUT (the expected outcome; h_how[2] = 2 and 1: timed out, left on
 * abort) with the context still usable, or another status on failure. */
int fgb_wait_expiry_check(long long polls, int *h_how, void *stream);

/* Thin Q (rows x cols, column-major) of the Householder QR of A (rows x
 * cols, column-major, rows >= cols), device buffers; the varmap
 * coefficients (normalized_dot_product.cpp:769-830) are its leading rows. */
int fgb_qr_thin_q(int rows, int cols, const double *d_A, double *d_Q,
                  void *stream);

/* Evaluation from mapping coefficients, the model a LAMMPS run loads from
 * an lmp.flare file (pair_flare.cpp:68-175, lammps_descriptor.cpp:250-326):
 * E_i = B2.beta_s B2/|B2|^2 (power 2) or beta_s.B2/|B2| (power 1) for the
 * NormalizedDotProduct kernel (normalized != 0; the DotProduct forms
 * without the norms), zero where |B2|^2 < 1e-8, forces and stresses by the
 * reverse-mode adjoint.  h_beta as returned by fgb_model_mapping.  An
 * optional variance map h_varmap (n_species x n_d x n_d row-major Q_s, the
 * map_unc file of compute flare/std/atom, compute_flare_std_atom.cpp:
 * 179-193) gives v_i = 1 - |Q_s^T B2/|B2||^2 per atom (FGB_WANT_LOCAL_VAR;
 * the std is sign(v) sqrt|v|).  Outputs as in fgb_predict, plus per-atom
 * energies (any output may be NULL); precision FGB_PREC_FP64, or
 * FGB_PREC_MIXED (descriptor in double-float, adjoint in FP32 unless the
 * largest |beta| exceeds 200, the beta product still FP64-level). */
typedef struct fgb_mapped_s *fgb_mapped_t;
int fgb_mapped_create(fgb_mapped_t *out, fgb_b2_t b2, int power,
                      int normalized, const double *h_beta,
                      const double *h_varmap);
int fgb_mapped_destroy(fgb_mapped_t m);
int fgb_mapped_predict(fgb_mapped_t m, int n_struc, const int *h_atom_offsets,
                       const double *h_cells, const double *d_positions,
                       const int *d_species, double cutoff, int want,
                       double *d_energy, double *d_forces, double *d_stress,
                       double *d_atom_energy, double *d_local_var,
                       int precision, void *stream);

/* ------------------------------------------------------------ autotuner
 * Tile shapes of the sliced tensor-core GEMMs (kernel, variance and force
 * GEMMs of the mixed path) are chosen per problem shape: at the first call
 * with a new (operation, rows rounded up to a power of two, columns, depth)
 * every candidate shape is timed with CUDA events and the fastest is kept
 * (process-wide; appended to the file named by FGB_TUNE_CACHE when that is
 * set, and read from it at start).  All candidates give identical results.
 * FGB_AUTOTUNE=0 in the environment starts with tuning off.  No counterpart
 * in flare_pp (CPU code with fixed loops). */
enum {
  FGB_TUNE_KERNEL_GEMM = 0,     /* candidates: B tiles of 48, 32 rows      */
  FGB_TUNE_VARIANCE_GEMM = 1,   /* candidates: B tiles of 48, 32 rows      */
  FGB_TUNE_FORCE_GEMM = 2       /* candidates: 128 rows x 2 epilogue warps,
                                   128 x 4, 64 x 2                          */
};
/* 1: tune at first use (default); 0: always the first candidate. */
int fgb_tune_set_mode(int mode);
/* Force candidate `candidate` for operation `op` (-1: back to tuning). */
int fgb_tune_force(int op, int candidate);
/* Forget every tuned shape. */
int fgb_tune_clear(void);
/* Tuned shapes so far, and entry i: key5 = {op, rows bucket, columns,
 * depth, chosen candidate}, ms4 = best timed launch per candidate (0 for
 * entries read from the cache file). */
int fgb_tune_count(void);
int fgb_tune_entry(int i, int *key5, double *ms4);

/* ------------------------------------------------------------ serving
 * Continuous batching over a solved model.  fgb_serve_start launches
 * n_workers host threads; each owns a replica of the model (same weights,
 * its own device workspace) and a CUDA stream.  Submitted structures queue
 * in arrival order; a free worker takes the longest prefix of the queue
 * whose device-memory footprint (atoms x the model's bytes per atom) fits
 * what the budget has left, predicts it as one batch (fgb_predict_host),
 * and hands each result back.  Batches of different workers run
 * concurrently on the GPU.  A structure alone or in any batch gives the same
 * bits (no float atomics, fixed reduction orders).  A request whose own
 * footprint exceeds the budget is refused at submit (FGB_EINVAL). */
typedef struct fgb_server_s *fgb_server_t;
int fgb_serve_start(fgb_server_t *out, fgb_model_t model, int n_workers,
                    long long memory_budget_bytes, int max_structures,
                    double cutoff, int want, int precision);
/* copies the inputs; returns the request id in *request_id */
int fgb_serve_submit(fgb_server_t s, int n_atoms, const double *h_cell,
                     const double *h_positions, const int *h_species,
                     long long *request_id);
/* *done = 1 when finished: results are copied out (any pointer may be NULL)
 * and the request is released; *latency_ms = submit-to-completion time.
 * A failed request returns its error status here. */
int fgb_serve_poll(fgb_server_t s, long long request_id, int *done,
                   double *h_energy, double *h_forces, double *h_stress,
                   double *h_local_var, double *latency_ms);
/* completed requests, batches run, bytes of the model's per-atom footprint */
int fgb_serve_stats(fgb_server_t s, long long *completed, long long *batches,
                    long long *bytes_per_atom);
int fgb_serve_stop(fgb_server_t s);

/* NormalizedDotProduct::envs_envs (normalized_dot_product.cpp:28-89) for
 * one species block in FP64: d_kern[n1 * n2] (row-major) =
 * sig2 * (d1.d2 / (norm1 norm2))^power, zero where either norm < 1e-8.
 * d_desc1[n1 * n_desc], d_norm1[n1], d_desc2[n2 * n_desc], d_norm2[n2]. */
int fgb_envs_envs(const double *d_desc1, const double *d_norm1, int n1,
                  const double *d_desc2, const double *d_norm2, int n2,
                  int n_desc, double sig2, double power, double *d_kern,
                  void *stream);

/* NormalizedDotProduct::envs_struc (normalized_dot_product.cpp:117-214) on
 * the GPU in FP64, the reference algorithm with stored forward-mode
 * descriptor gradients: the sparse set (h_counts[n_species] environments per
 * species, d_sparse[M * n_d] species-grouped raw descriptors) against ONE
 * structure (an n_struc == 1 build of `nl`, coded species d_species[N]).
 * d_kern[M * (1 + 3N + 6)] row-major: energy, force and stress columns. */
int fgb_envs_struc(fgb_b2_t b2, double sigma, double power,
                   const int *h_counts, const double *d_sparse,
                   fgb_nlist_t nl, const int *d_species, double *d_kern,
                   void *stream);

/* NormalizedDotProduct::self_kernel_struc (normalized_dot_product.cpp:
 * 450-586) in FP64: the prior variances of ONE structure's energy, forces
 * and stress, d_out[1 + 3N + 6] (energy, 3N force components, stress xx xy
 * xz yy yz zz).  Computed without the reference's 3P x 3P force_force
 * matrix: force entries as local sums over each atom's neighbourhood,
 * energy and stress over atom pairs.  FGB_EINVAL with the reference's
 * message where a descriptor dot product is below 1e-8 and power < 2. */
int fgb_self_kernel_struc(fgb_b2_t b2, double sigma, double power,
                          fgb_nlist_t nl, const int *d_species, double *d_out,
                          void *stream);

/* NormalizedDotProduct::struc_struc (normalized_dot_product.cpp:216-448)
 * in FP64: the kernel between every output of structure 1 (energy, 3 N1
 * force components, 6 stress components) and every output of structure 2,
 * d_out[(1 + 3 N1 + 6) x (1 + 3 N2 + 6)] row-major.  Both lists are
 * single-structure builds with the same B2 settings.  Errors as
 * fgb_self_kernel_struc. */
int fgb_struc_struc(fgb_b2_t b2, double sigma, double power, fgb_nlist_t nl1,
                    const int *d_species1, fgb_nlist_t nl2,
                    const int *d_species2, double *d_out, void *stream);

/* Plain FP64 form of SparseGP::predict_local_uncertainties for one
 * structure: envs_struc (stored gradients), mean_efs = K^T alpha, and the
 * local variances via the envs_envs route.  d_mean_efs[1+3N+6],
 * d_local_var[N] (atom order). */
int fgb_predict_plain(fgb_model_t m, fgb_nlist_t nl, const int *d_species,
                      double *d_mean_efs, double *d_local_var, void *stream);

/* C = A B^T in FP64 accuracy on the BF16 tensor cores (tcgen05), by exact
 * integer slicing of A and B (9 slices of 6 bits per row, 45 slice products
 * accumulated exactly in FP32 over K segments of at most 1472, summed and
 * recombined in 64-bit integers, rounded once to FP64).  A[M x K] (lda),
 * B[N x K] (ldb), C[M x N] (ldc), row-major device pointers.  The kernel
 * used for the sparse-GP kernel and variance products. */
int fgb_oz_dgemm_nt(int M, int N, int K, const double *d_A, long long lda,
                    const double *d_B, long long ldb, double *d_C,
                    long long ldc, void *stream);
/* The same product at `slices` = 9, 8 or 7 BF16 slices per operand (54,
 * 48 or 42 bits: the precisions the mixed path's kernel and variance GEMMs
 * run at); the dropped digit products and slice residuals stay below
 * 2^(-6 slices) of the row maxima.  No reference counterpart. */
int fgb_oz_dgemm_nt_slices(int slices, int M, int N, int K, const double *d_A,
                           long long lda, const double *d_B, long long ldb,
                           double *d_C, long long ldc, void *stream);

/* C = A B^T in FP32 accuracy on the same tensor-core kernel with 4 slices
 * (10 slice products, exact accumulation), FP64 inputs, FP32 output
 * C[M x N] (ldc).  The kernel used for the force GEMM of the
 * mixed-precision path.  No reference counterpart (an internal product). */
int fgb_oz_sgemm_nt(int M, int N, int K, const double *d_A, long long lda,
                    const double *d_B, long long ldb, float *d_C,
                    long long ldc, void *stream);

/* SparseGP::update_matrices_QR (sparse_gp.cpp:607-641) in FP64 on the GPU:
 * Cholesky of Kuu + jitter I and L_inv (fgb_cholesky, fgb_trtri_lower), the
 * QR of [diag(sqrt(noise)) Kuf^T ; L^T] by shifted Cholesky QR with two
 * refinement passes (R_inv and Q^T b; R agrees with the reference's
 * Householder R up to row signs, so alpha and Sigma are the same
 * quantities), alpha = R_inv (Q^T b)[:M]; the O(n M^2) and O(M^3) products
 * as FP64-level tensor-core products.  All device pointers, row-major.
 * d_Kuu[M*M], d_Kuf[M*n_labels], d_y[n_labels], d_noise[n_labels] ->
 * d_alpha[M], d_L_inv[M*M], d_R_inv[M*M] (may be NULL).  A Kuu + jitter
 * that is not positive definite returns FGB_EINVAL with the reference's
 * kind of message. */
int fgb_solve_qr(int M, int n_labels, const double *d_Kuu,
                 const double *d_Kuf, const double *d_y,
                 const double *d_noise, double jitter, double *d_alpha,
                 double *d_L_inv, double *d_R_inv, void *stream);

/* The LLT step of update_matrices_QR (sparse_gp.cpp:610-615, Eigen's LLT in
 * the reference): d_A (M x M, row-major, symmetric; the lower triangle is
 * read) is replaced by its lower Cholesky factor, strict upper part zeroed.
 * Blocked: 128 x 128 diagonal blocks factored in shared memory, the panel
 * and trailing updates as FP64-level tensor-core products.  FGB_EINVAL if a
 * leading minor is not positive definite. */
int fgb_cholesky(int M, double *d_A, void *stream);
/* Inverse of a lower-triangular M x M matrix (row-major; the reference's
 * triangularView<Lower>().solve(Kuu_eye), sparse_gp.cpp:616-618, and the
 * R_inv solve through R^T, :636-638), recursive over diagonal halves with
 * FP64-level tensor-core products; d_X's strict upper part zeroed; d_L and
 * d_X distinct. */
int fgb_trtri_lower(int M, const double *d_L, double *d_X, void *stream);
/* Kuu_inverse = L_inv^T L_inv and Sigma = R_inv R_inv^T (sparse_gp.cpp:619,
 * 640) as FP64-level tensor-core products (M x M, row-major; either output
 * may be NULL). */
int fgb_solve_products(int M, const double *d_L_inv, const double *d_R_inv,
                       double *d_Kuu_inverse, double *d_Sigma, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FLAREGB_H */
