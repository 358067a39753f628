// Device-resident sparse-GP model and its prediction workspace.
#pragma once
#include <functional>
#include <memory>
#include <vector>

#include "fgb_internal.h"
#include "fgb_ozaki.h"

// Page-locked species counts (and range flag) of the species permutation
// and the event recorded after their copy, so that the host can wait for
// them after queueing more work.
struct fgb_pinned_counts {
  int *h = nullptr;
  cudaEvent_t ev = nullptr;
  fgb_pinned_counts() = default;
  fgb_pinned_counts(const fgb_pinned_counts &) = delete;
  fgb_pinned_counts &operator=(const fgb_pinned_counts &) = delete;
  ~fgb_pinned_counts() {
    if (h) cudaFreeHost(h);
    if (ev) cudaEventDestroy(ev);
  }
};

struct fgb_workspace {
  fgb_pinned_counts counts;
  fgb::DevBuf perm, flags, pos, scal, scan_tmp, flag;
  fgb::DevBuf A, B2, norms, e_atom, var, volume, atom_off;
  fgb::DevBuf rowmax;   // largest |B2| per row (tensor-core row scales)
  fgb::DevBuf gB2, pair_grad, forces, virial;
  fgb::DevBuf kmat, wmat, erows, part;
  fgb::DevBuf b2f, yf;           // mixed path: FP32 normalised rows, D^ B
  fgb::DevBuf dB2, fdots, fdot, dots, kern;  // plain (stored-gradient) form
  fgb::oz::Sliced ozA, ozK;      // tensor-core path: sliced rows per call
  fgb::DevBuf ozerr;
};

struct fgb_io {
  fgb::DevBuf pos, species, energy, forces, stress, var;
};

struct fgb_model_s {
  fgb::B2Params b2;
  double sigma = 1.0, power = 2.0;
  int M = 0;
  bool solved = false;
  std::vector<int> h_counts, h_offsets;       // sparse envs per species
  std::vector<double> h_desc, h_snorm, h_alpha;
  std::vector<int> h_panel_rows;
  std::vector<long long> h_panel_off;
  std::vector<double> h_L_inv;   // host copy (replicas for serving workers)
  fgb::DevBuf S;        // normalised sparse descriptors, M x n_d (FP64)
  fgb::DevBuf Sraw;     // raw sparse descriptors, M x n_d (FP64)
  fgb::DevBuf snorm;    // sparse norms
  fgb::DevBuf svalid;   // uint8 norm >= 1e-8
  fgb::DevBuf alpha;    // M
  fgb::DevBuf Lp;       // per-species L_inv panels
  fgb::DevBuf RinvT;    // R_inv^T (M x M, lower triangular) for SOR
  bool has_rinv = false;
  fgb::DevBuf Lfull;    // L_inv (M x M, lower triangular) for DTC, on demand
  bool lfull_ready = false;
  fgb::DevBuf Bmap;     // mixed path: per species n_d x n_d FP32 folded matrix
  fgb::DevBuf Bfold;    // the folded matrices in FP64 (power 2), per species
  // the folded matrices in FP32-level slices (tensor-core force GEMM), one
  // set per B tile height of the autotuner's candidates
  std::vector<std::unique_ptr<fgb::oz::Sliced>> ozB[fgb::oz::kF32Sets];
  bool ozB_ready[fgb::oz::kF32Sets] = {};
  bool bmap_ready = false;
  // largest folded coefficient sigma^2 |B_s| and the guard it sets: forces
  // at FP64 level (product, gradient, adjoint) when it is large
  double fold_max = 0.0;
  bool force_f64 = false;
  std::vector<std::unique_ptr<fgb::oz::Sliced>> ozB64;   // FP64-level B_s rows
  // mixed path: sliced sparse set and L_inv panels per species (tensor
  // cores), one set per variant (slice count x B tile width of the
  // autotuner's candidates), each sliced the first time it runs
  std::vector<std::unique_ptr<fgb::oz::Sliced>> ozS[fgb::oz::kF64Variants],
      ozL[fgb::oz::kF64Variants];
  bool ozS_ready[fgb::oz::kF64Variants] = {};
  bool ozL_ready[fgb::oz::kF64Variants] = {};
  // slices of the kernel GEMM (9, 8 or 7) and of the variance GEMM (9, 8,
  // 7 or 6) with the largest energy (eV/atom) and local-variance
  // differences to 9 slices measured on the sparse set when they were
  // chosen (choose_kernel_slices); forced counts (fgb_model_set_slices,
  // 0 = chosen by the probes) outlive new weights
  int oz_S = fgb::oz::kS;
  int oz_Sv = fgb::oz::kS;
  double oz_err_est = 0.0;
  double oz_var_err_est = 0.0;
  int oz_S_forced = 0, oz_Sv_forced = 0;
  bool slices_chosen = false;
  fgb_nlist_s nl;
  fgb_workspace ws;
  fgb_io io;
  std::vector<int> last_species_counts;   // atoms per species, last full call
};

namespace fgb {
// Above this largest folded coefficient the mixed path's force stage runs
// at FP64 level (the FP32-level stage errs by ~2.5e-7 eV/A per unit).
constexpr double kFoldMaxF32 = 200.0;

// A prediction repeated on the atoms, species and cells of the model's last
// full call at new positions (a molecular-dynamics step).  The geometry, the
// species permutation and the workspace of that call are reused, the
// neighbour list is rebuilt into a reserved pair capacity, and nothing is
// read back, synchronised or allocated: the launches can be captured in a
// CUDA graph.  Error flags stay on the device for the caller: nl.flag (and
// flag[3] = pair capacity exceeded) and ws.ozerr (bounded tensor-core
// waits), which the caller clears before the call.
struct FixedPlan {
  long long pair_cap = 0;
  std::vector<int> counts;   // atoms per species (last_species_counts)
};
}  // namespace fgb

// A model with the same weights and its own device workspace (predict.cu);
// nullptr with rc set on failure.
fgb_model_s *model_replicate(const fgb_model_s *src, int &rc);

// Host side of a prediction whose inputs and results live in host memory
// (fgb_predict_host): the host copy of the species (species counts without
// a device read-back) and the result buffers, copied back on the stream
// before the call's final synchronisation (any may be null).
struct PredictHostIO {
  const int *species = nullptr;
  double *energy = nullptr, *forces = nullptr, *stress = nullptr,
         *local_var = nullptr;
};

// One batched prediction on device positions (predict.cu): the body of
// fgb_predict, also driven by the MD ensemble (with `fixed` for the steps
// it replays) and by fgb_predict_host (with `hio`).
int predict_impl(fgb_model_s *m, int n_struc, const int *h_atom_offsets,
                 const double *h_cells, const double *d_positions,
                 const int *d_species, double cutoff, int want, int precision,
                 double *d_energy, double *d_forces, double *d_stress,
                 double *d_local_var, cudaStream_t st,
                 const fgb::FixedPlan *fixed = nullptr,
                 const PredictHostIO *hio = nullptr);

namespace fgb {
int kernel_stage_fp64(fgb_model_s *m, int N, const std::vector<int> &counts,
                      bool want_grad, bool want_var, double *d_e_atom,
                      double *d_gB2, double *d_var, cudaStream_t st);
// Bounded tensor-core waits report into ws.ozerr, which the caller clears
// before and reads after; `fixed`: prepare nothing (operands must be ready).
// `after_chunk(s, Mr, perm)` runs after each row chunk's kernel and
// variance GEMMs, with the chunk's rows still sliced in ws.ozA (the force
// stage of the mixed path).
using ChunkHook = std::function<int(int, int, const int *)>;
int kernel_stage_oz(fgb_model_s *m, int N, const std::vector<int> &counts,
                    bool want_w, bool want_var, double *d_e_atom, double *d_var,
                    cudaStream_t st, bool fixed = false,
                    const ChunkHook *after_chunk = nullptr);
// Slice count of the mixed path's kernel and variance GEMMs, measured on
// the model's sparse set (ozaki.cu; synchronises).
int choose_kernel_slices(fgb_model_s *m, cudaStream_t st);
// The folded matrices and the fold guard (force_f64) of a power-1/2 model,
// built once before its first mixed prediction (synchronises).
int prepare_mixed(fgb_model_s *m, cudaStream_t st);
int kernel_stage_mixed(fgb_model_s *m, int N, const std::vector<int> &counts,
                       bool want_grad, bool want_var, double *d_e_atom,
                       double *d_gB2, double *d_var, cudaStream_t st,
                       bool fixed = false);
int species_permutation(fgb_model_s *m, const int *d_species, int N,
                        std::vector<int> &counts, cudaStream_t st,
                        const int *h_species = nullptr);
// The same on any workspace: perm = atoms of species 0 (ascending), then
// 1, ...; one host synchronisation (counts and the species range check),
// none when the host copy of the species is given (counted and checked on
// the host).
int species_permutation(int S, fgb_workspace &ws, const int *d_species, int N,
                        std::vector<int> &counts, cudaStream_t st,
                        const int *h_species = nullptr);
// The same in two halves: start queues the kernels and the counts' copy
// to page-locked memory (pending = true when finish must wait for it);
// finish waits for the stream up to that copy, not for what was queued
// after it (so work queued in between keeps the GPU busy meanwhile), and
// checks the species range.
int species_permutation_start(int S, fgb_workspace &ws, const int *d_species,
                              int N, std::vector<int> &counts, cudaStream_t st,
                              const int *h_species, bool &pending);
int species_permutation_finish(int S, fgb_workspace &ws,
                               std::vector<int> &counts);
int envs_struc_impl(const B2Params &p, double sigma, double power,
                    const int *h_counts, const double *d_sparse,
                    fgb_nlist_s *nl, const int *d_species, double *d_kern,
                    fgb_workspace &ws, cudaStream_t st);
// self_kernel_struc of one structure into d_out[1 + 3N + 6] (struc_kernels.cu); with
// have_dervs the workspace already holds B2, norms and dB2 of this list.
int self_kernel_impl(const B2Params &p, double sigma, double power,
                     fgb_nlist_s *nl, const int *d_species, double *d_out,
                     fgb_workspace &ws, cudaStream_t st, bool have_dervs);
// struc_struc of two structures into d_out[(1 + 3 N1 + 6) x (1 + 3 N2 + 6)]
// row-major (struc_kernels.cu).
int struc_struc_impl(const B2Params &p, double sigma, double power,
                     fgb_nlist_s *nl1, const int *d_species1,
                     fgb_nlist_s *nl2, const int *d_species2, double *d_out,
                     cudaStream_t st);
}  // namespace fgb
