// FP64- and FP32-accurate tensor-core GEMMs by exact BF16 slicing (ozaki.cu).
#pragma once
#include "fgb_internal.h"

namespace fgb {
namespace oz {

constexpr int kS = 9;        // slices per operand
constexpr int kBeta = 6;     // bits per slice
constexpr int kG = kS;       // groups a + b = 2 .. kS + 1
constexpr int kTM = 128;     // A rows per tile (TMEM lanes)
constexpr int kTN = 48;      // B rows per tile (columns per group), default
constexpr int kKC = 16;      // k per pipeline stage (one MMA k-step)
constexpr int kStages = 4;   // shared-memory pipeline depth
constexpr int kEpiWarps = 3; // epilogue warps per TMEM lane quarter (16 columns
                             // each); partial sums per row: B tiles x kEpiWarps
// K segment: the largest K whose group sums stay below 2^24 (exact FP32
// accumulation in TMEM); the biggest group (a + b = 10) sums to at most
// 11264 * K.  Longer K runs in segments summed in 64-bit integers.
constexpr int kMaxK = 1472;
// FP32-level configuration (force GEMM of the mixed path): 4 slices, B tiles
// of 128 rows; the biggest group (a + b = 5) sums to at most 6144 * K.
constexpr int kSF32 = 4;
constexpr int kTNF32 = 128;
constexpr int kMaxKF32 = 2720;

// Tile shapes the autotuner chooses from (fgb_tune.h).  FP64 level: B tiles
// of kTNF64v[v] rows, one 16-column chunk per epilogue warp, so row partial
// sums land in the same 16-column slots whatever the tile.  FP32 level: B
// tiles of kTNF32v[v] rows drained by kEWF32v[v] epilogue warps per TMEM
// lane quarter.  All candidates give the same results bit for bit.
// The mixed path's kernel GEMM takes 9, 8 or 7 slices (54, 48 or 42 bits)
// and its variance GEMM 9, 8, 7 or 6 (36 bits), each the fewest that the
// model's error probes allow (choose_kernel_slices); variant v =
// kF64PerS x (slice set) + (tile choice).  Tile candidates per slice count:
// B tiles of 48 and 32 rows, and of 64 rows where S x 64 accumulator
// columns fit TMEM (S <= 8).
constexpr int kNumSF64 = 4;
constexpr int kSF64set[kNumSF64] = {9, 8, 7, 6};
constexpr int kF64PerS = 3;
constexpr int kF64Variants = kNumSF64 * kF64PerS;
constexpr int kTNF64v[kF64Variants] = {48, 32, 48, 48, 32, 64,
                                       48, 32, 64, 48, 32, 64};
constexpr int kSF64v[kF64Variants] = {9, 9, 9, 8, 8, 8, 7, 7, 7, 6, 6, 6};
constexpr int s_index(int S) { return 9 - S; }
constexpr int n_cand_s(int S) { return S == 9 ? 2 : 3; }
// slice counts each GEMM may take
constexpr int kMinKernelSlices = 7;
constexpr int kMinVarianceSlices = 6;
constexpr int kF32Variants = 3;
constexpr int kTNF32v[kF32Variants] = {128, 128, 64};
constexpr int kEWF32v[kF32Variants] = {2, 4, 2};
// B operand slice sets of the FP32 level (one per distinct tile height)
constexpr int kF32Sets = 2;
constexpr int kTNF32set[kF32Sets] = {128, 64};
constexpr int f32_set(int v) { return kTNF32v[v] == 128 ? 0 : 1; }

struct SliceSpec {
  int rows, K, TR;
  const double *src;
  long long ld;
  const int *perm;         // optional row gather
  const double *rownorm;   // optional: divide row by its norm (0 if < 1e-8)
  // optional: each source row's largest |value| (indexed like src rows);
  // the row scales then come from it instead of a pass over the rows
  const double *rowmax = nullptr;
};

struct Sliced {
  int rows = 0, K = 0, TR = 0, RP = 0, KP = 0, S = 0;
  DevBuf q;       // bf16 slices, tiled canonical layout
  DevBuf scale;   // per-row 2^e
};

int pad_to(int x, int m);
// Size `out` for rows x K in S slices (no conversion).
int prepare(int rows, int K, int TR, int S, Sliced &out);
// Slice rows into S = kS (FP64-level), 8, 7 or 6 (the mixed path's kernel
// and variance GEMMs) or kSF32 (FP32-level) digits.
int slice(const SliceSpec &sp, Sliced &out, cudaStream_t st, int S = kS);

// Product of S-slice operands (S = 9, 8, 7 or 6; B.S == S, A.S >= S); the
// tile shape follows B.TR (one of kTNF64v).
template <int S, class Epi>
int gemm_s(const Sliced &A, const Sliced &B, bool tri, const Epi &epi,
           int *err, cudaStream_t st);
// FP64-level product of kS-slice operands.
template <class Epi>
int gemm(const Sliced &A, const Sliced &B, bool tri, const Epi &epi, int *err,
         cudaStream_t st);
// C (A.rows x B.rows, leading dimension ldc) = A B^T in FP64 from kS-slice
// operands (A tiles of kTM rows, B tiles of kTN rows): exact integer sums,
// one rounding.
int gemm_store(const Sliced &A, const Sliced &B, double *C, long long ldc,
               int *err, cudaStream_t st);
// C = a (A B^T) + b C in FP64 from kS-slice operands (b = 0: C is only
// written), the same exact integer sums and one rounding of the product.
int gemm_axpby(const Sliced &A, const Sliced &B, double *C, long long ldc,
               double a, double b, int *err, cudaStream_t st);
// Y (A.rows x B.rows, leading dimension ldy) = A B^T rounded to FP32, from
// kSF32-slice operands (A tiles of kTM rows, B tiles of 128 or 64 rows;
// `ew` epilogue warps per lane quarter, 2 or 4 for 128-row tiles).  A may
// be sliced with more digits (kS): its first kSF32 slices are used.
int gemm_f32(const Sliced &A, const Sliced &B, float *Y, long long ldy,
             int *err, cudaStream_t st, int ew = 2);

}  // namespace oz
}  // namespace fgb
