// Tile-shape autotuner for the sliced tensor-core GEMMs (tune.cu).
//
// Each GEMM of the prediction has a few candidate tile shapes that give the
// same result bit for bit (the products are exact integer sums, and every
// candidate writes its row partial sums into the same 16-column slots).
// The first time a problem shape (operation, rows rounded up to a power of
// two, columns, depth) is met, every candidate runs once untimed and twice
// timed with CUDA events on the caller's stream and the fastest is kept for
// the rest of the process (and in the file named by FGB_TUNE_CACHE, when
// set).  Calls that are being captured into a CUDA graph, or that must not
// synchronise, take the cached choice or candidate 0.
#pragma once
#include <functional>

#include "fgb_internal.h"

namespace fgb {
namespace tune {

enum Op {
  kOpKernelGemm = 0,     // FP64-level kernel GEMM (energy, K slices)
  kOpVarianceGemm = 1,   // FP64-level triangular variance GEMM
  kOpForceGemm = 2,      // FP32-level force GEMM of the mixed path
  kNumOps
};
constexpr int kMaxCand = 4;

// Launch one GEMM of shape (M, N, K) for `op`: `run(c)` launches candidate
// c on `st` (preparing its operands if needed) and returns a status.
// `frozen`: no timing and no preparation; the cached choice is taken when
// `usable(c)` says its operands are ready, else candidate 0.  The candidate
// launched last is returned in *chosen.
int run(int op, int M, int N, int K, int n_cand,
        const std::function<int(int)> &run,
        const std::function<bool(int)> &usable, cudaStream_t st, bool frozen,
        int *chosen);

}  // namespace tune
}  // namespace fgb
