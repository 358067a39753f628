// Internal host-side types shared by the libflaregb translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <vector>

#include "fgb_common.cuh"

namespace fgb {

// Grow-only device buffer.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  int ensure(size_t n);            // FGB_OK or FGB_ENOMEM
  void release();
  ~DevBuf() { release(); }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

// Device allocations made by DevBuf::ensure so far (process-wide): a graph
// captured while this number changed may refer to freed buffers.
unsigned long long devbuf_allocations();

// Per-structure geometry for the cell-list build (device copy).
struct StrucGeom {
  double cell[9];
  double ct[9], cti[9], cd[9], cdi[9];   // cell^T, inverse, cell cell^T, inverse
  double volume;
  int nb[3];        // bins per axis
  int kk[3];        // bin search half-width per axis
  int sweep;        // reference image sweep (structure.cpp:35)
  int atom0, natoms;
  int bin0;         // first global bin
  // FP32 candidate prefilter: cell rows in FP32 and squared-distance bounds
  // that bracket the FP64 test with a margin above the FP32 rounding error
  float cell32[9];
  float d2_out;     // FP32 d^2 above this: certainly outside the cutoff
  float d2_in;      // FP32 d^2 below this (and above d2_zero): certainly inside
  float d2_zero;    // FP32 d^2 at or below this: d may be 0, test in FP64
  // Integer division without the FP64/conversion pipe: n / d = (n m) >> 32
  // with m = floor(2^32 / d) + 1, exact for n, d < 2^16 and for n < 2^24,
  // d < 2^8 (the image counts and bins here are within both).
  unsigned long long m_nb[3];    // for nb[k]
  unsigned long long m_n1, m_n2; // for 2 kk[1] + 1 and 2 kk[2] + 1
  int wrap_c[3];    // floordiv(t, nb) = (t + wrap_c nb) / nb - wrap_c, t > -kk
};

// Host-side cell algebra in the canonical operation order (no FMA).
void cell_setup(const double *cell, double *ct, double *cti, double *cd,
                double *cdi, double *volume, double *single_sweep_cutoff);

// Device exclusive scan helpers (two-level, deterministic).
int scan_int_to_int(const int *d_in, int *d_out, int n, int *d_total,
                    DevBuf &tmp, cudaStream_t st);
int scan_int_to_ll(const int *d_in, long long *d_out, int n,
                   long long *d_total, DevBuf &tmp, cudaStream_t st);
// Variants with caller-provided block sums (ceil(n/1024) + 1 elements).
int scan_int_to_int_raw(const int *d_in, int *d_out, int n, int *d_total,
                        int *d_sums, cudaStream_t st);
int scan_int_to_ll_raw(const int *d_in, long long *d_out, int n,
                       long long *d_total, long long *d_sums,
                       cudaStream_t st);

}  // namespace fgb

struct fgb_nlist_s;
namespace fgb {
// fgb_nlist_build on a stream.  With `check` false the device flags
// (non-finite positions, fill and twin consistency, single-pass overflow)
// are left for the caller, who reads them after its own synchronisation
// and passes them to nlist_finish; a single-pass build then does not
// synchronise at all, and n_pairs is an upper bound until nlist_finish.
int nlist_build(fgb_nlist_s *nl, int n_struc, const int *h_atom_offsets,
                const double *h_cells, const double *d_positions,
                double cutoff, cudaStream_t st, bool check);
// The deferred checks of a build with `check` false, from its four device
// flags read after the stream synchronised: FGB_OK (and the exact pair
// count in n_pairs), an error, or kNlistRetry when an atom had more pairs
// than its single-pass slots (the caller repeats its work with
// count_pass set).
constexpr int kNlistRetry = 1000;
int nlist_finish(fgb_nlist_s *nl, const int *hflag);
// Per-pair buffers for at least `cap` pairs (neighbors.cu).
int nlist_reserve(fgb_nlist_s *nl, long long cap);
// The list of the last full build's structures (same atoms, cells, bins) at
// new positions, with no host synchronisation and no allocation: pairs go
// into the capacity reserved by nlist_reserve; more pairs than that set
// flag[3] and truncate every list at the capacity (the caller discards the
// result).  Flags are cleared first and left on the device for the caller.
int nlist_rebuild_fixed(fgb_nlist_s *nl, const double *d_positions,
                        double cutoff, long long cap, cudaStream_t st);
}  // namespace fgb

struct fgb_nlist_s {
  int n_struc = 0;
  int n_atoms = 0;
  long long n_pairs = 0;
  long long n_bins = 0;       // bins of the last full build
  std::vector<int> h_atom_offsets;
  std::vector<double> h_cells;
  std::vector<double> h_volume;
  fgb::DevBuf geom;          // StrucGeom[n_struc]
  fgb::DevBuf atom_struct;   // int[N]
  fgb::DevBuf wrapped;       // double[N*3]
  fgb::DevBuf wrapped32;     // float4[N]: FP32 wrapped position, image flags
  fgb::DevBuf raw_bin;       // int[N*3]
  fgb::DevBuf home_bin;      // int[N]
  fgb::DevBuf bin_slot;      // int[N]
  fgb::DevBuf bin_count;     // int[n_bins]
  fgb::DevBuf bin_start;     // int[n_bins+1]
  fgb::DevBuf bin_atoms;     // int[N]
  fgb::DevBuf counts;        // int[N]
  fgb::DevBuf offsets;       // long long[N+1]
  fgb::DevBuf tmp_key;       // unsigned long long[P]
  fgb::DevBuf tmp_rel;       // double4_16a[P]
  fgb::DevBuf nbr_j;         // int[P]  (batch-global atom index)
  fgb::DevBuf nbr_shift;     // int[P]  packed (s0+128)<<16|(s1+128)<<8|(s2+128)
  fgb::DevBuf nbr_rel;       // double4_16a[P] (d, x, y, z)
  fgb::DevBuf nbr_twin;      // long long[P] index of (j -> i, -s)
  fgb::DevBuf flag;          // int[4] device error flags: non-finite
                             // positions, fill or twin inconsistency, pair
                             // capacity exceeded (fixed rebuild)
  fgb::DevBuf scan_tmp;
  fgb::DevBuf scalars;       // long long[4]
  // single-pass builds: slots per atom of the last one and the least the
  // next may take (raised after an overflow), the pinned pair total the
  // build copies back, whether n_pairs still waits for it, and a request
  // for a count pass (set by callers repeating a build that overflowed)
  long long last_slots = 0, min_slots = 0;
  int last_launches = 0;     // kernels the last build or rebuild launched
  long long *h_total = nullptr;
  bool total_pending = false;
  bool count_pass = false;
  fgb_nlist_s() = default;
  fgb_nlist_s(const fgb_nlist_s &) = delete;
  fgb_nlist_s &operator=(const fgb_nlist_s &) = delete;
  ~fgb_nlist_s() {
    if (h_total) cudaFreeHost(h_total);
  }
};

struct fgb_b2_s {
  fgb::B2Params p;
};
