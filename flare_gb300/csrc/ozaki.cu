// FP64-accurate (and FP32-accurate) GEMMs on the BF16 tensor cores
// (tcgen05), by exact integer slicing (the Ozaki scheme).
//
// Each row of A (M x K) and of B (N x K) is scaled by a power of two so its
// entries lie in (-1, 1), then split into S slices of BETA = 6 bits:
// x = sum_a q_a 2^(-6a) + r, |q_1| <= 64, |q_a| <= 32 (a > 1), each q an
// integer held exactly in BF16.  The products q_a q_b are exact in FP32 and,
// for K up to the configuration's limit, every partial sum of a group (all
// pairs with the same t = a + b) stays below 2^24, so the tensor core's FP32
// accumulation is exact too.  The S (S + 1) / 2 pairs with a + b <= S + 1 are
// accumulated into S group accumulators held in TMEM (S x TN FP32 columns
// per 128-row tile), and the epilogue recombines
// C = 2^(e_row + e_col) sum_t 2^(-6t) group_t exactly in 64-bit integers,
// rounding once to FP64 or FP32.  The dropped terms (a + b > S + 1) and the
// slice residuals are below 2^(-6S) of each row's largest entry.
//   S = 9, TN = 48:  FP64-level (2^-54); kernel and variance products of the
//                    sparse GP (energy 4e-12 eV/atom, std 4e-13 against FP64)
//   S = 4, TN = 128: FP32-level (2^-24); the alpha-folded force GEMM
//
// Data movement: slices are written by k_oz_slice8 directly in the tensor
// core's no-swizzle K-major canonical layout (8 x 16-byte core matrices),
// tiled so that the S slices of every (row tile, 16-wide k chunk) are one
// contiguous block.  One thread streams each chunk with two cp.async.bulk
// copies into a shared-memory ring (mbarrier transaction counts), another
// issues the chunk's pair products as tcgen05.mma with the B slices stacked
// along N (mma_kstep) and commits them to the stage's "consumed" mbarrier;
// every wait is bounded and reports through `err`.
#include <cuda_bf16.h>

#include <cmath>
#include <type_traits>

#include "fgb_internal.h"
#include "fgb_ozaki.h"
#include "fgb_tc.cuh"

namespace fgb {
namespace oz {

namespace {

constexpr uint32_t kTmemCols = 512;
constexpr long long kWaitLimit = 1LL << 22;

// Largest per-k contribution to one group: sum over its pairs of
// max|q_a| max|q_b| (64 for the first digit, 32 for the others).
__host__ __device__ constexpr int max_group_weight(int S) {
  int best = 0;
  for (int t = 2; t <= S + 1; t++) {
    int w = 0;
    for (int a = 1; a <= S; a++) {
      const int b = t - a;
      if (b < 1 || b > S) continue;
      w += (a == 1 ? 64 : 32) * (b == 1 ? 64 : 32);
    }
    best = w > best ? w : best;
  }
  return best;
}

// A tile configuration: S slices, TN columns of B per CTA, STAGES ring
// depth, EW epilogue warps per TMEM lane quarter (each takes TN / EW columns).
template <int S_, int TN_, int STAGES_, int MAXK_, int EW_>
struct Cfg {
  static constexpr int S = S_, TN = TN_, STAGES = STAGES_, MAXK = MAXK_;
  static constexpr int EW = EW_;
  static constexpr int THREADS = 32 * (2 + 4 * EW);
  static constexpr int MMA_WARP = 1 + 4 * EW;   // after the epilogue warps
  static constexpr int WCOLS = TN / EW;   // columns per epilogue warp
  // K segment: chunks accumulated in TMEM before the epilogue adds the exact
  // group sums into its 64-bit registers (any K, exact)
  static constexpr int SEGC = MAXK / kKC;
  static constexpr uint32_t TileA = kTM * kKC * 2;   // bytes per slice
  static constexpr uint32_t TileB = TN * kKC * 2;
  static constexpr uint32_t Stage = S * (TileA + TileB);
  static constexpr uint32_t Smem = STAGES * Stage + 256;
  // groups t = 2 .. TSPLIT go to the high integer, the rest to the low one
  static constexpr int TSPLIT = S + 1 < 6 ? S + 1 : 6;
  static constexpr bool HAS_LO = TSPLIT < S + 1;
  static_assert(S * TN <= (int)kTmemCols, "group accumulators exceed TMEM");
  static_assert(Smem <= 227 * 1024, "stages exceed shared memory");
  static_assert(TN % 16 == 0 && TN <= 256, "MMA N");
  static_assert((long long)MAXK * max_group_weight(S) < (1LL << 24),
                "group sums must stay exact in FP32");
  static_assert(TN % (16 * EW) == 0, "epilogue warps take whole 16-column chunks");
};
using CfgF64 = Cfg<kS, 48, kStages, kMaxK, 3>;
using CfgF64n = Cfg<kS, 32, kStages, kMaxK, 2>;
// fewer slices: smaller stages, so a deeper ring fits; B tiles of 64 rows
// take four epilogue warps per lane quarter (576 threads)
constexpr int ring_depth(int S, int TN) {
  return 5 * S * (kTM * kKC * 2 + TN * kKC * 2) + 256 <= 227 * 1024 ? 5 : 4;
}
template <int S, int TN>
using CfgS = typename std::conditional<
    S == kS, typename std::conditional<TN == 48, CfgF64, CfgF64n>::type,
    Cfg<S, TN, ring_depth(S, TN), kMaxK, TN / 16>>::type;
static_assert(CfgS<8, 48>::EW == 3 && CfgS<8, 32>::EW == 2 &&
                  CfgS<8, 64>::EW == 4 && CfgS<7, 48>::WCOLS == 16 &&
                  CfgS<7, 32>::WCOLS == 16 && CfgS<7, 64>::WCOLS == 16,
              "every FP64-level candidate: one 16-column chunk per epilogue warp");
using CfgF32 = Cfg<kSF32, 128, 6, kMaxKF32, 2>;
using CfgF32w = Cfg<kSF32, 128, 6, kMaxKF32, 4>;
using CfgF32n = Cfg<kSF32, 64, 8, kMaxKF32, 2>;
static_assert(CfgF64::TN == kTNF64v[0] && CfgF64n::TN == kTNF64v[1] &&
                  CfgF64::WCOLS == 16 && CfgF64n::WCOLS == 16,
              "FP64-level candidates: one 16-column chunk per epilogue warp");
static_assert(CfgF64::TN == kTN && CfgF64::EW == kEpiWarps, "default shape");
static_assert(CfgF32::TN == kTNF32v[0] && CfgF32::EW == kEWF32v[0] &&
                  CfgF32w::TN == kTNF32v[1] && CfgF32w::EW == kEWF32v[1] &&
                  CfgF32n::TN == kTNF32v[2] && CfgF32n::EW == kEWF32v[2],
              "FP32-level candidates");
static_assert(kKC % 16 == 0, "a chunk is whole MMA k-steps");
static_assert(kBeta == 6, "digits of 6 bits");

// One tcgen05.mma covering the pairs (A, B0) .. (A, B0 + NB - 1).  The B
// slices of a stage sit one after another in shared memory (each TN rows of
// 8-row core-matrix groups, 256 bytes apart), so NB consecutive slices are a
// single N = TN NB operand; their products belong to the consecutive groups
// A + B0 .. A + B0 + NB - 1, whose accumulators are consecutive TN-column
// blocks of TMEM.  An M = 128 MMA costs max(64, N / 2) cycles, so stacking
// slices keeps instructions wide.
template <class C, int A, int B0, int NB>
__device__ __forceinline__ void mma_span(uint32_t tmem, uint64_t ad0,
                                         uint64_t bd0, bool first) {
  static_assert(A >= 0 && B0 >= 0 && NB >= 1 && A + B0 + NB <= C::S,
                "span outside the pairs with a + b <= S + 1");
  static_assert(NB * C::TN <= 256, "an M = 128 MMA takes N <= 256");
  // descriptor start addresses are in 16-byte units in the low bits
  tc::mma_bf16(tmem + (uint32_t)((A + B0) * C::TN),
               ad0 + (uint64_t)((A * C::TileA) >> 4),
               bd0 + (uint64_t)((B0 * C::TileB) >> 4),
               tc::idesc_bf16_f32(kTM, NB * C::TN),
               (A == 0 && first) ? 0u : 1u);
}

// All pairs of one 16-deep k-step.  A slice a pairs with B slices
// 0 .. S-1-a, split into the fewest spans of at most 256 / TN slices, of
// near-equal width (S = 9, TN = 48: 13 MMAs; S = 4, TN = 128: 6).  The a = 0
// spans together cover every group, so with `first` set they initialise all
// accumulators.
template <class C, int A = 0, int B0 = 0>
__device__ __forceinline__ void mma_kstep(uint32_t tmem, uint64_t ad0,
                                          uint64_t bd0, bool first) {
  if constexpr (A < C::S) {
    constexpr int total = C::S - A;               // B slices for this A
    constexpr int maxnb = 256 / C::TN;
    constexpr int nspans = (total + maxnb - 1) / maxnb;
    constexpr int width = (total + nspans - 1) / nspans;
    constexpr int rem = total - B0;
    if constexpr (rem > 0) {
      constexpr int nb = rem < width ? rem : width;
      mma_span<C, A, B0, nb>(tmem, ad0, bd0, first);
      mma_kstep<C, A, B0 + nb>(tmem, ad0, bd0, first);
    } else {
      mma_kstep<C, A + 1, 0>(tmem, ad0, bd0, first);
    }
  }
}

// Slice storage, chunk-major: the S slices of one (row tile, 16-wide k chunk)
// are one contiguous block (S tiles of TR x 16 in the canonical layout), so a
// pipeline stage is filled by a single bulk copy per operand.  Returns the
// element index of (m, k) in slice 0; slice a sits a * TR * 16 further on.
template <int S>
__device__ __forceinline__ size_t tiled_index(int m, int k, int KP, int TR) {
  return ((size_t)(m / TR) * (KP / kKC) + k / kKC) * (size_t)(S * TR * kKC) +
         (size_t)(((m % TR) / 8) * (kKC / 8) + (k % kKC) / 8) * 64 +
         (m % 8) * 8 + (k % 8);
}

// ---------------------------------------------------------------------------
// Integer helpers.  FP64 arithmetic runs at about 2 operations per clock per
// SM on this GPU, so the slicing and recombination build and take apart
// doubles with integer instructions; the results are the same doubles the
// FP64 expressions give.

// e for a power-of-two scale 2^e.
__device__ __forceinline__ int pow2_exp(double s) {
  return (int)((__double_as_longlong(s) >> 52) & 0x7FF) - 1023;
}

// Out of line so that its FP64 instructions stay off the common path.
static __device__ __noinline__ double scaled_rare(long long x, int sc) {
  return ldexp((double)x, sc);
}

// x 2^sc as a double: exact for |x| < 2^53 and a normal result (the common
// case), else rounded once.
__device__ __forceinline__ double exact_scaled(long long x, int sc) {
  if (x == 0) return 0.0;
  const unsigned long long a = x < 0 ? 0ULL - (unsigned long long)x
                                     : (unsigned long long)x;
  const int p = 63 - __clzll((long long)a);            // leading bit
  const int field = p + sc + 1023;
  if (p > 52 || field < 1 || field > 2046) return scaled_rare(x, sc);
  unsigned long long bits = ((unsigned long long)field << 52) |
                            ((a << (52 - p)) & 0xFFFFFFFFFFFFFULL);
  if (x < 0) bits |= 1ULL << 63;
  return __longlong_as_double(bits);
}

static __device__ __noinline__ float scaled_float_rare(long long x, int sc) {
  return ldexpf(__ll2float_rn(x), sc);
}

// x 2^sc rounded once to FP32 (nearest, ties to even: the value of
// __ll2float_rn(x) scaled exactly), built with integer instructions.
__device__ __forceinline__ float scaled_float(long long x, int sc) {
  if (x == 0) return 0.f;
  const unsigned long long a = x < 0 ? 0ULL - (unsigned long long)x
                                     : (unsigned long long)x;
  const int p = 63 - __clzll((long long)a);            // leading bit
  unsigned long long q;
  int lead = p;                                        // weight of q's top bit
  if (p > 23) {
    const int r = p - 23;
    q = a >> r;
    const unsigned long long rem = a & ((1ULL << r) - 1), half = 1ULL << (r - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
    if (q == (1ULL << 24)) { q >>= 1; lead++; }
  } else {
    q = a << (23 - p);
  }
  const int field = lead + sc + 127;
  if (field < 1 || field > 254) return scaled_float_rare(x, sc);
  return __uint_as_float((x < 0 ? 0x80000000u : 0u) | ((unsigned)field << 23) |
                         ((unsigned)q & 0x7FFFFFu));
}

// rn(d 2^sh) as a 64-bit integer (nearest, ties to even, as __double2ll_rn
// of the exactly scaled value), for |d 2^sh| < 2^62.
__device__ __forceinline__ long long fixed_rn(double d, int sh) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(d);
  const int field = (int)((bits >> 52) & 0x7FF);
  const int s = field - 1075 + sh;   // value = mant 2^s
  if (field == 0 || s > 9) return __double2ll_rn(ldexp(d, sh));  // rare
  const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  unsigned long long q;
  if (s >= 0) {
    q = mant << s;
  } else {
    const int r = -s;
    if (r > 53) {
      q = 0;
    } else {
      q = mant >> r;
      const unsigned long long rem = mant & ((1ULL << r) - 1);
      const unsigned long long half = 1ULL << (r - 1);
      q += (rem > half || (rem == half && (q & 1))) ? 1 : 0;
    }
  }
  return (bits >> 63) ? -(long long)q : (long long)q;
}

// The S base-64 digits of X (|X| < 2^(6S)) for 8 consecutive k, stored as
// 16-byte rows of the canonical layout: slice a at out + a * stride.  The
// digits are balanced: U = X + sum_{a >= 2} 32 2^(6(S-a)) has plain base-64
// digits u_2..u_S below its top one, d_a = u_a - 32 in [-32, 31] and d_1 =
// U >> 6(S-1) in [-64, 64]; X = sum_a d_a 2^(6(S-a)) exactly.  U is held as
// two 32-bit words, so a digit is one funnel shift (or word shift) and a
// mask.  Its float (exact: |d| <= 64) is the bits of 1.5 * 2^23 + d minus
// 1.5 * 2^23, one FP32 subtraction (an integer-to-float conversion would
// run on the FP64/conversion pipe, which this GPU runs slowly); its BF16 is
// that float's upper half, and one byte permute packs two of them.
template <int S>
__device__ __forceinline__ void store_digits8(long long (&X)[8],
                                              __nv_bfloat16 *out,
                                              size_t stride) {
  constexpr long long kBias = [] {
    long long b = 0;
    for (int a = 2; a <= S; a++) b += 32LL << (kBeta * (S - a));
    return b;
  }();
  uint32_t lo[8], hi[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const unsigned long long u = (unsigned long long)(X[j] + kBias);
    lo[j] = (uint32_t)u;
    hi[j] = (uint32_t)(u >> 32);
  }
#pragma unroll
  for (int a = 1; a <= S; a++) {
    const int sh = kBeta * (S - a);
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      float f[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        // bits [sh, ...) of U: the low word of U >> sh (U >> sh fits it)
        const uint32_t v = sh >= 32 ? hi[j + h] >> (sh - 32)
                                    : __funnelshift_r(lo[j + h], hi[j + h], sh);
        const int q = a == 1
                          ? (sh >= 32 ? (int)hi[j + h] >> (sh - 32) : (int)v)
                          : (int)(v & 63u) - 32;
        f[h] = __fsub_rn(__int_as_float(0x4B400000 + q), 12582912.0f);
      }
      // BF16 of each (their exact floats' upper halves), low digit first
      w[j / 2] = __byte_perm(__float_as_uint(f[0]), __float_as_uint(f[1]),
                             0x7632);
    }
    *reinterpret_cast<uint4 *>(out + (size_t)(a - 1) * stride) =
        make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Row scales: 2^e with e from the row's largest magnitude (after the
// optional division by the row norm), one warp per row; rows past R and
// empty rows get 2^0.  Written to `scale` for k_oz_slice8.
__global__ void __launch_bounds__(256)
k_oz_rowscale(int R, int K, int RP, const double *__restrict__ src,
              long long ld, const int *__restrict__ perm,
              const double *__restrict__ rownorm, double thresh,
              double *__restrict__ scale) {
  const int m = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (m >= RP) return;
  bool valid = m < R;
  long long row = 0;
  double inv = 1.0;
  if (valid) {
    row = perm ? (long long)perm[m] : (long long)m;
    if (rownorm) {
      const double n = rownorm[row];
      if (n >= thresh) inv = 1.0 / n;
      else valid = false;
    }
  }
  unsigned long long mb = 0;
  if (valid) {
    const double *sr = src + row * ld;
    for (int k = lane; k < K; k += 32)
      mb = max(mb, (unsigned long long)__double_as_longlong(sr[k]) &
                       0x7FFFFFFFFFFFFFFFULL);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    mb = max(mb, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)mb, off));
  const double mx = __longlong_as_double((long long)mb) * inv;
  const int e = mx > 0.0 ? ilogb(mx) + 1 : 0;
  if (lane == 0) scale[m] = ldexp(1.0, e);
}

// The same scales from each source row's largest |value| given up front
// (`rowmax`, indexed like the source rows): a thread per row.
__global__ void k_oz_scale_from_max(int R, int RP, const int *__restrict__ perm,
                                    const double *__restrict__ rownorm,
                                    double thresh,
                                    const double *__restrict__ rowmax,
                                    double *__restrict__ scale) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= RP) return;
  double mx = 0.0;
  if (m < R) {
    const long long row = perm ? (long long)perm[m] : (long long)m;
    double inv = 1.0;
    bool valid = true;
    if (rownorm) {
      const double n = rownorm[row];
      if (n >= thresh) inv = 1.0 / n;
      else valid = false;
    }
    if (valid) mx = rowmax[row] * inv;
  }
  const int e = mx > 0.0 ? ilogb(mx) + 1 : 0;
  scale[m] = ldexp(1.0, e);
}

// Row slicing: each row scaled to (-1, 1) by its power of two 2^e
// (k_oz_rowscale), the scaled value y taken as the integer X = rn(y 2^(6S))
// (exact for |y| >= 2^-1 of the row's top binade, rounded at 2^(-6S) below
// that) and its S balanced base-64 digits stored (store_digits8).  A warp
// takes 8 rows (one core-matrix row group) and one part of kSlicePart
// columns, 32 consecutive k at a time, lane = row + 8 x (k group of 8), so
// that the 16-byte row pieces a store instruction writes for one slice are
// two contiguous 256-byte blocks (one 16-k chunk each) rather than 32
// scattered pieces; the parts let a few thousand rows fill the GPU.
constexpr int kSlicePart = 128;
static_assert(kSlicePart % 32 == 0, "a part is whole 32-column steps");
template <int S>
__global__ void __launch_bounds__(256)
k_oz_slice8(int R, int K, int RP, int KP, int TR, int nparts,
            const double *__restrict__ src, long long ld, int vec,
            const int *__restrict__ perm, const double *__restrict__ rownorm,
            double thresh, __nv_bfloat16 *__restrict__ out,
            const double *__restrict__ scale) {
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int part = (int)(gw % nparts);
  const int m0 = (int)(gw / nparts) * 8;
  if (m0 >= RP) return;
  const int r = lane & 7, g = lane >> 3;
  const int m = m0 + r;
  bool valid = m < R;
  long long row = 0;
  double inv = 1.0;
  if (valid) {
    row = perm ? (long long)perm[m] : (long long)m;
    if (rownorm) {
      const double n = rownorm[row];
      if (n >= thresh) inv = 1.0 / n;
      else valid = false;
    }
  }
  const double *sr = src + row * ld;
  const int e = pow2_exp(scale[m]);
  const size_t stride = (size_t)TR * kKC;
  const int kend = min(KP, (part + 1) * kSlicePart);
  for (int k0 = part * kSlicePart + g * 8; k0 < kend; k0 += 32) {
    // the lane's 8 values: four 16-byte loads when the source rows allow
    // (vec: 16-byte aligned rows) and all 8 lie inside the row
    double v[8];
    if (vec && valid && k0 + 8 <= K) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const double2 t = reinterpret_cast<const double2 *>(sr + k0)[q];
        v[2 * q] = t.x;
        v[2 * q + 1] = t.y;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) v[j] = (valid && k0 + j < K) ? sr[k0 + j] : 0.0;
    }
    long long X[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int k = k0 + j;
      X[j] = (valid && k < K)
                 ? fixed_rn(rownorm ? v[j] * inv : v[j], kBeta * S - e)
                 : 0;
    }
    store_digits8<S>(X, out + tiled_index<S>(m, k0, KP, TR), stride);
  }
}

// n / d for 32-bit n and d >= 1 without the FP64/conversion pipe (which
// run-time integer division uses, and which this GPU runs slowly): m =
// floor((2^64 - 1) / d) + 1, q = high 64 bits of n m (exact: the excess
// n (m - 2^64/d) / 2^64 < 2^-32 stays below 1/d).
struct FastDiv {
  unsigned d;
  unsigned long long m;
};
inline FastDiv make_fastdiv(int d) {
  return {(unsigned)d, d > 1 ? ~0ULL / (unsigned long long)d + 1ULL : 0ULL};
}
__device__ __forceinline__ int fdiv(int n, FastDiv f) {
  return f.d == 1 ? n : (int)__umul64hi((unsigned long long)(unsigned)n, f.m);
}

// Wait for a phase, giving up when `abort_flag` is raised or after `limit`
// polls: 0 done, 1 aborted elsewhere, 2 timed out.
__device__ __forceinline__ int wait_or_abort(uint64_t *bar, uint32_t phase,
                                             volatile int *abort_flag,
                                             long long limit = kWaitLimit) {
  for (long long i = 0; i < limit; i++) {
    if (tc::mbar_try_wait(bar, phase)) return 0;
    if (*abort_flag) return 1;
  }
  return 2;
}

// The GEMMs' give-up path on a barrier that nothing arrives at: warp 0
// waits (bounded by `limit` polls) for a phase that never completes, raises
// the CTA's abort flag and reports the time-out in *err, as a GEMM's
// producer does; warp 1 waits on the same barrier and leaves through the
// abort flag.  Nothing faults and every wait ends.
__global__ void k_wait_expiry(long long limit, int *__restrict__ err,
                              int *__restrict__ how) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    abort_flag = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (lane == 0) {
    const int w = wait_or_abort(&bar, 0, &abort_flag,
                                warp == 0 ? limit : 64 * limit);
    if (w == 2) {
      abort_flag = 1;
      atomicExch(err, 1);
    }
    how[warp] = w;
  }
  __syncthreads();
}

// Persistent, warp-specialised GEMM: one CTA per SM walks the tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... (B tiles fastest).
//   warp 0, lane 0  streams chunks into the shared-memory ring: a stage is
//                   refilled as soon as the MMAs that read it complete; the
//                   ring runs on across tile boundaries.
//   last warp, lane 0  issues the MMAs of each chunk as soon as its copies
//                   land (so the tensor pipe never waits on the copy issue),
//                   commits the stage back to the loader and, after a tile's
//                   (or K segment's) last chunk, the accumulator to the
//                   epilogue.
//   warps 1..4 EW   the epilogue: warp w reads TMEM lanes 32 (w % 4) ...
//                   (the hardware's lane quarter for that warp) and columns
//                   [sub WCOLS, (sub + 1) WCOLS) with sub = (w - 1) / 4.
//                   Phase 1 drains its part of the accumulator into registers
//                   (exact integer recombination) and releases it
//                   (acc_empty); phase 2 (the functor's arithmetic and
//                   stores, latency-bound) then overlaps the next tile's MMAs,
//                   with EW warps per quarter to hide its latency.
// Barriers: load_full / load_empty per ring stage (transaction bytes; MMA
// commit), acc_full (commit after a tile's last MMAs), acc_empty (one arrive
// per epilogue warp).  Every wait is bounded; a thread that gives up raises
// the CTA's abort flag, which every other wait polls; the copies and MMAs
// in flight are waited for (bounded) before TMEM is freed and the CTA
// exits, and `err` reports it.  Energy and variance partials are written
// per (tile, epilogue warp): NTt * EW slots per row.
template <class C, class Epi>
__global__ void __launch_bounds__(C::THREADS, 1)
k_oz_gemm(int M, int N, int K, int KP, int MT, int NTt, FastDiv divNT,
          int SA, const __nv_bfloat16 *__restrict__ Asl,
          const double *__restrict__ Ascale,
          const __nv_bfloat16 *__restrict__ Bsl,
          const double *__restrict__ Bscale, int tri, Epi epi,
          int *__restrict__ err) {
  constexpr int S = C::S, TN = C::TN, NST = C::STAGES, NCH = C::WCOLS / 16;
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *bar_load = reinterpret_cast<uint64_t *>(smem + NST * C::Stage);
  uint64_t *bar_mma = bar_load + NST;
  uint64_t *acc_full = bar_mma + NST;
  uint64_t *acc_empty = acc_full + 1;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  long long *issued = reinterpret_cast<long long *>(tmem_slot + 2);
  long long *consumed = issued + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = MT * NTt;
  const int KCH = KP / kKC;

  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int b = 0; b < NST; b++) {
      tc::mbar_init(&bar_load[b], 1);
      tc::mbar_init(&bar_mma[b], 1);
    }
    tc::mbar_init(acc_full, 1);
    tc::mbar_init(acc_empty, 4 * C::EW);
    tc::mbar_fence_init();
    *abort_flag = 0;
    *issued = 0;
    *consumed = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  // row and column tile of tile t; chunks of a tile (triangular B: columns
  // n0 .. n0+TN-1 need k < n0 + TN)
  // Tiles row-major (a row tile's column tiles run together and share its A
  // operand in L2), with the column order rotated by the row tile: a
  // persistent CTA's tiles t, t + grid, ... then visit every column tile
  // instead of a few (with a triangular B the column tiles differ in cost).
  auto tile_rc = [&](int t, int &mt, int &nt) {
    mt = fdiv(t, divNT);
    const int rot = mt - fdiv(mt, divNT) * NTt;
    nt = t - mt * NTt + rot;
    if (nt >= NTt) nt -= NTt;
  };
  auto tile_nch = [&](int nt) {
    const int n0 = nt * TN;
    const int kmax = tri ? min(K, n0 + TN) : K;
    return (kmax + kKC - 1) / kKC;
  };
  auto give_up = [&](int why) {   // why: 1 aborted elsewhere, 2 timed out
    if (why == 2) {
      *abort_flag = 1;
      atomicExch(err, 1);
    }
  };

  if (warp == 0) {
    if (lane == 0) {
      long long g = 0;   // chunks issued
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        int mt, nt;
        tile_rc(t, mt, nt);
        const int nch = tile_nch(nt);
        // A blocks hold SA >= S slices per chunk; the first S (the most
        // significant digits) are this product's operand
        const __nv_bfloat16 *a = Asl + (size_t)mt * KCH * (SA * kTM * kKC);
        const __nv_bfloat16 *bsrc = Bsl + (size_t)nt * KCH * (S * TN * kKC);
        for (int c = 0; c < nch; c++, g++) {
          const int b = (int)(g % NST);
          if (g >= NST) {
            // stage b last held chunk g - NST: its MMAs must be done
            const int w = wait_or_abort(&bar_mma[b],
                                        (uint32_t)(((g / NST) - 1) & 1),
                                        abort_flag);
            if (w) { give_up(w); ok = false; break; }
          }
          unsigned char *st = smem + b * C::Stage;
          tc::mbar_expect_tx(&bar_load[b], C::Stage);
          tc::bulk_g2s(st, a + (size_t)c * (SA * kTM * kKC), S * C::TileA,
                       &bar_load[b]);
          tc::bulk_g2s(st + S * C::TileA, bsrc + (size_t)c * (S * TN * kKC),
                       S * C::TileB, &bar_load[b]);
        }
      }
      *issued = g;
    }
  } else if (warp == C::MMA_WARP) {
    if (lane == 0) {
      long long g = 0;   // chunks consumed
      int sg = 0;        // K segments accumulated so far (acc_full phases)
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        int mt, nt;
        tile_rc(t, mt, nt);
        const int nch = tile_nch(nt);
        for (int c = 0; c < nch; c++) {
          const bool seg_first = c % C::SEGC == 0;
          if (seg_first && sg > 0) {
            // the previous segment's accumulator must be drained first
            const int w = wait_or_abort(acc_empty, (sg - 1) & 1, abort_flag);
            if (w) { give_up(w); ok = false; break; }
            tc::fence_after_sync();
          }
          const int b = (int)(g % NST);
          const int w = wait_or_abort(&bar_load[b], (uint32_t)((g / NST) & 1),
                                      abort_flag);
          if (w) { give_up(w); ok = false; break; }
          tc::fence_after_sync();
          const uint32_t aBase = tc::smem_u32(smem + b * C::Stage);
          const uint64_t ad0 = tc::smem_desc(aBase, 128, (kKC / 8) * 128);
          const uint64_t bd0 = tc::smem_desc(aBase + S * C::TileA, 128,
                                             (kKC / 8) * 128);
          // k-steps of 16 are two core matrices (256 bytes) apart along K
#pragma unroll
          for (int kk = 0; kk < kKC / 16; kk++)
            mma_kstep<C>(tmem, ad0 + (uint64_t)((kk * 256) >> 4),
                         bd0 + (uint64_t)((kk * 256) >> 4),
                         seg_first && kk == 0);
          tc::mma_commit(&bar_mma[b]);
          if (c == nch - 1 || (c + 1) % C::SEGC == 0) {
            tc::mma_commit(acc_full);
            sg++;
          }
          g++;
        }
      }
      *consumed = g;
      if (!ok && g > 0)   // MMAs finish before TMEM is freed (bounded)
        tc::mbar_wait(&bar_mma[(g - 1) % NST], (uint32_t)(((g - 1) / NST) & 1),
                      kWaitLimit);
    }
  } else {
    const int q = warp & 3;            // TMEM lane quarter of this warp
    const int sub = (warp - 1) >> 2;   // its column range within the tile
    const int c_lo = sub * C::WCOLS;
    const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16);
    int sg = 0;   // K segments drained so far
    bool alive = true;
    for (int t = blockIdx.x; t < ntiles && alive; t += gridDim.x) {
      int mt, nt;
      tile_rc(t, mt, nt);
      const int m0 = mt * kTM, n0 = nt * TN;
      const int m = m0 + q * 32 + lane;
      const bool row_ok = m < M;
      const int nseg = (tile_nch(nt) + C::SEGC - 1) / C::SEGC;
      // Phase 1, per K segment.  Group sums are exact integers below 2^24;
      // add them exactly into 64-bit integers, hi = sum_{t <= TSPLIT} g_t
      // 2^(6(TSPLIT-t)) and lo = sum_{t > TSPLIT} g_t 2^(6(S+1-t)), and
      // release the accumulator after each segment.
      long long hi[NCH][16], lo[NCH][16];
#pragma unroll
      for (int ch = 0; ch < NCH; ch++)
#pragma unroll
        for (int j = 0; j < 16; j++) { hi[ch][j] = 0; lo[ch][j] = 0; }
      for (int seg = 0; seg < nseg; seg++, sg++) {
        const int w = wait_or_abort(acc_full, sg & 1, abort_flag);
        if (w) {
          give_up(w);
          alive = false;
          break;
        }
        tc::fence_after_sync();
        // (chunk, group) loads in sequence, two register buffers: the load
        // of the next pair is in flight while this one is added up, and the
        // accumulator is released as soon as the last load has landed
        uint32_t rb[2][16];
        tc::tmem_ld16(trow + c_lo, rb[0]);
        tc::tmem_ld_wait(rb[0]);
#pragma unroll
        for (int it = 0; it < NCH * S; it++) {
          const int ch = it / S, g = it % S, cur = it & 1;
          if (it + 1 < NCH * S) {
            const int ch1 = (it + 1) / S, g1 = (it + 1) % S;
            tc::tmem_ld16(trow + g1 * TN + c_lo + ch1 * 16, rb[cur ^ 1]);
          } else {
            // the accumulator may now take the next segment or tile
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(acc_empty);
          }
          const int tg = g + 2;
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const long long qv =
                (long long)__float2int_rn(__uint_as_float(rb[cur][j]));
            if (tg <= C::TSPLIT) hi[ch][j] += qv << (6 * (C::TSPLIT - tg));
            else lo[ch][j] += qv << (6 * (S + 1 - tg));
          }
          if (it + 1 < NCH * S) tc::tmem_ld_wait(rb[cur ^ 1]);
        }
      }
      if (!alive) break;
      // C = (hi 2^(-6 TSPLIT) + lo 2^(-6(S+1))) 2^(e_row + e_col): exact
      // doubles built from the integers and one correctly rounded addition
      // (FP64 results), or one rounding of hi (FP32 results, no low part).
      // Rows past M (tile padding) still run so that functors can write
      // zero padding.
      const int er = pow2_exp(Ascale[m]);
      using V = typename Epi::Value;
      V v[NCH][16];
#pragma unroll
      for (int ch = 0; ch < NCH; ch++) {
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int e = er + pow2_exp(Bscale[n0 + c_lo + ch * 16 + j]);
          if constexpr (Epi::kFloat) {
            static_assert(!C::HAS_LO, "FP32 results take at most 5 slices");
            v[ch][j] = scaled_float(hi[ch][j], e - 6 * C::TSPLIT);
          } else {
            double x = exact_scaled(hi[ch][j], e - 6 * C::TSPLIT);
            if constexpr (C::HAS_LO)
              x += exact_scaled(lo[ch][j], e - 6 * (S + 1));
            v[ch][j] = x;
          }
        }
      }
      // Phase 2
      double acc = 0.0;
#pragma unroll
      for (int ch = 0; ch < NCH; ch++)
        acc = epi.chunk(m, row_ok, n0 + c_lo + ch * 16, v[ch], acc);
      epi.finish(m, row_ok, nt * C::EW + sub, acc);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (tid == 0 && *abort_flag) {
    // copies issued but never consumed land before the CTA exits (bounded)
    for (long long g = *consumed; g < *issued; g++)
      tc::mbar_wait(&bar_load[g % NST], (uint32_t)((g / NST) & 1), kWaitLimit);
  }
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// Plain product C = A B^T (FP64).
struct EpiStore {
  using Value = double;
  static constexpr bool kFloat = false;
  double *C;
  long long ldc;
  int N;
  __device__ double chunk(int m, bool row_ok, int n0, const double (&v)[16],
                          double acc) const {
    if (!row_ok) return acc;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      int n = n0 + j;
      if (n < N) C[(long long)m * ldc + n] = v[j];
    }
    return acc;
  }
  __device__ void finish(int, bool, int, double) const {}
};

// C = a (A B^T) + b C (b = 0: C is not read), FP64; the dense
// factorizations' updates (C -= L21 L21^T, X21 = -X22 T, ...).
struct EpiAxpby {
  using Value = double;
  static constexpr bool kFloat = false;
  double *C;
  long long ldc;
  int N;
  double a, b;
  __device__ double chunk(int m, bool row_ok, int n0, const double (&v)[16],
                          double acc) const {
    if (!row_ok) return acc;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int n = n0 + j;
      if (n < N) {
        double *c = C + (long long)m * ldc + n;
        *c = b == 0.0 ? a * v[j] : fma(b, *c, a * v[j]);
      }
    }
    return acc;
  }
  __device__ void finish(int, bool, int, double) const {}
};

// Plain product Y = A B^T rounded to FP32.
struct EpiStoreF32 {
  using Value = float;
  static constexpr bool kFloat = true;
  float *Y;
  long long ldy;
  int N;
  __device__ double chunk(int m, bool row_ok, int n0, const float (&v)[16],
                          double acc) const {
    if (!row_ok) return acc;
    float *y = Y + (long long)m * ldy + n0;
    if (n0 + 16 <= N && (reinterpret_cast<uintptr_t>(y) & 15) == 0) {
      // a full chunk on a 16-byte boundary: four vector stores
      float4 *y4 = reinterpret_cast<float4 *>(y);
#pragma unroll
      for (int q = 0; q < 4; q++)
        y4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      return acc;
    }
#pragma unroll
    for (int j = 0; j < 16; j++)
      if (n0 + j < N) y[j] = v[j];
    return acc;
  }
  __device__ void finish(int, bool, int, double) const {}
};

}  // namespace

int pad_to(int x, int m) { return (x + m - 1) / m * m; }

int prepare(int rows, int K, int TR, int S, Sliced &out) {
  out.rows = rows;
  out.K = K;
  out.TR = TR;
  out.S = S;
  out.RP = pad_to(std::max(rows, 1), TR);
  out.KP = pad_to(std::max(K, 1), kKC);
  int rc;
  if ((rc = out.q.ensure(sizeof(__nv_bfloat16) * (size_t)S * out.RP * out.KP)) ||
      (rc = out.scale.ensure(sizeof(double) * (size_t)out.RP)))
    return rc;
  return FGB_OK;
}

template <int S>
static int slice_s(const SliceSpec &sp, Sliced &out, cudaStream_t st) {
  int rc;
  if ((rc = prepare(sp.rows, sp.K, sp.TR, S, out))) return rc;
  if (sp.rowmax) {
    k_oz_scale_from_max<<<ceil_div(out.RP, 256), 256, 0, st>>>(
        sp.rows, out.RP, sp.perm, sp.rownorm, kEmptyThresh, sp.rowmax,
        out.scale.as<double>());
    FGB_LAUNCH_CHECK("k_oz_scale_from_max");
  } else {
    k_oz_rowscale<<<ceil_div((long long)out.RP * 32, 256), 256, 0, st>>>(
        sp.rows, sp.K, out.RP, sp.src, sp.ld, sp.perm, sp.rownorm,
        kEmptyThresh, out.scale.as<double>());
    FGB_LAUNCH_CHECK("k_oz_rowscale");
  }
  const int nparts = ceil_div(out.KP, kSlicePart);
  const long long threads = (long long)(out.RP / 8) * nparts * 32;  // RP % 8 == 0
  // 16-byte loads need every row start 16-byte aligned
  const int vec = (sp.ld % 2 == 0 &&
                   reinterpret_cast<uintptr_t>(sp.src) % 16 == 0) ? 1 : 0;
  k_oz_slice8<S><<<ceil_div(threads, 256), 256, 0, st>>>(
      sp.rows, sp.K, out.RP, out.KP, sp.TR, nparts, sp.src, sp.ld, vec,
      sp.perm, sp.rownorm, kEmptyThresh, out.q.as<__nv_bfloat16>(),
      out.scale.as<double>());
  FGB_LAUNCH_CHECK("k_oz_slice8");
  return FGB_OK;
}

int slice(const SliceSpec &sp, Sliced &out, cudaStream_t st, int S) {
  if (S == kS) return slice_s<kS>(sp, out, st);
  if (S == 8) return slice_s<8>(sp, out, st);
  if (S == 7) return slice_s<7>(sp, out, st);
  if (S == 6) return slice_s<6>(sp, out, st);
  if (S == kSF32) return slice_s<kSF32>(sp, out, st);
  set_error("ozaki slice: unsupported slice count %d", S);
  return FGB_EINVAL;
}


template <class C, class Epi>
static int gemm_c(const Sliced &A, const Sliced &B, bool tri, const Epi &epi,
                  int *err, cudaStream_t st) {
  // A may carry more (less significant) slices than the product uses
  if (A.K != B.K || A.KP != B.KP || A.TR != kTM || B.TR != C::TN ||
      A.S < C::S || B.S != C::S) {
    set_error("ozaki gemm: operand layouts disagree");
    return FGB_EINVAL;
  }
  if (A.rows == 0 || B.rows == 0) return FGB_OK;
  FGB_CUDA(cudaFuncSetAttribute(k_oz_gemm<C, Epi>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)C::Smem));
  int dev = 0, sms = 0;
  FGB_CUDA(cudaGetDevice(&dev));
  FGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int MT = A.RP / kTM, NTt = B.RP / C::TN;
  const int grid = std::max(1, std::min(MT * NTt, sms));
  k_oz_gemm<C, Epi><<<grid, C::THREADS, C::Smem, st>>>(
      A.rows, B.rows, A.K, A.KP, MT, NTt, make_fastdiv(NTt), A.S,
      A.q.as<__nv_bfloat16>(),
      A.scale.as<double>(), B.q.as<__nv_bfloat16>(), B.scale.as<double>(),
      tri ? 1 : 0, epi, err);
  FGB_LAUNCH_CHECK("k_oz_gemm");
  return FGB_OK;
}

template <int S, class Epi>
int gemm_s(const Sliced &A, const Sliced &B, bool tri, const Epi &epi,
           int *err, cudaStream_t st) {
  if (B.TR == 32) return gemm_c<CfgS<S, 32>>(A, B, tri, epi, err, st);
  if constexpr (S < kS)
    if (B.TR == 64) return gemm_c<CfgS<S, 64>>(A, B, tri, epi, err, st);
  return gemm_c<CfgS<S, 48>>(A, B, tri, epi, err, st);
}

template <class Epi>
int gemm(const Sliced &A, const Sliced &B, bool tri, const Epi &epi, int *err,
         cudaStream_t st) {
  return gemm_s<kS>(A, B, tri, epi, err, st);
}

int gemm_store(const Sliced &A, const Sliced &B, double *C, long long ldc,
               int *err, cudaStream_t st) {
  return gemm(A, B, false, EpiStore{C, ldc, B.rows}, err, st);
}

int gemm_axpby(const Sliced &A, const Sliced &B, double *C, long long ldc,
               double a, double b, int *err, cudaStream_t st) {
  return gemm(A, B, false, EpiAxpby{C, ldc, B.rows, a, b}, err, st);
}

int gemm_f32(const Sliced &A, const Sliced &B, float *Y, long long ldy,
             int *err, cudaStream_t st, int ew) {
  const EpiStoreF32 epi{Y, ldy, B.rows};
  if (B.TR == CfgF32n::TN) return gemm_c<CfgF32n>(A, B, false, epi, err, st);
  if (ew == CfgF32w::EW) return gemm_c<CfgF32w>(A, B, false, epi, err, st);
  return gemm_c<CfgF32>(A, B, false, epi, err, st);
}

}  // namespace oz
}  // namespace fgb

using namespace fgb;

extern "C" int fgb_oz_dgemm_nt(int M, int N, int K, const double *d_A,
                               long long lda, const double *d_B, long long ldb,
                               double *d_C, long long ldc, void *stream) {
  return fgb_oz_dgemm_nt_slices(oz::kS, M, N, K, d_A, lda, d_B, ldb, d_C, ldc,
                                stream);
}

extern "C" int fgb_oz_dgemm_nt_slices(int slices, int M, int N, int K,
                                      const double *d_A, long long lda,
                                      const double *d_B, long long ldb,
                                      double *d_C, long long ldc,
                                      void *stream) {
  if (M < 0 || N < 0 || K < 0 || (M && N && (!d_A || !d_B || !d_C)) ||
      (slices != 9 && slices != 8 && slices != 7)) {
    set_error("fgb_oz_dgemm_nt: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (M == 0 || N == 0) return FGB_OK;
  if (K == 0) {
    for (int m = 0; m < M; m++)
      FGB_CUDA(cudaMemsetAsync(d_C + (long long)m * ldc, 0,
                               sizeof(double) * N, st));
    return FGB_OK;
  }
  oz::Sliced A, B;
  DevBuf err;
  int rc;
  if ((rc = err.ensure(sizeof(int)))) return rc;
  FGB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  if ((rc = oz::slice({M, K, oz::kTM, d_A, lda, nullptr, nullptr}, A, st,
                      slices)) ||
      (rc = oz::slice({N, K, oz::kTN, d_B, ldb, nullptr, nullptr}, B, st,
                      slices)))
    return rc;
  const oz::EpiStore epi{d_C, ldc, N};
  rc = slices == 9 ? oz::gemm_s<9>(A, B, false, epi, err.as<int>(), st)
       : slices == 8 ? oz::gemm_s<8>(A, B, false, epi, err.as<int>(), st)
                     : oz::gemm_s<7>(A, B, false, epi, err.as<int>(), st);
  if (rc) return rc;
  int h = 0;
  FGB_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error("fgb_oz_dgemm_nt: a bounded device wait ran out");
    return FGB_ETIMEOUT;
  }
  return FGB_OK;
}

extern "C" int fgb_oz_sgemm_nt(int M, int N, int K, const double *d_A,
                               long long lda, const double *d_B, long long ldb,
                               float *d_C, long long ldc, void *stream) {
  if (M < 0 || N < 0 || K < 0 || (M && N && (!d_A || !d_B || !d_C))) {
    set_error("fgb_oz_sgemm_nt: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (M == 0 || N == 0) return FGB_OK;
  if (K == 0) {
    for (int m = 0; m < M; m++)
      FGB_CUDA(cudaMemsetAsync(d_C + (long long)m * ldc, 0, sizeof(float) * N,
                               st));
    return FGB_OK;
  }
  oz::Sliced A, B;
  DevBuf err;
  int rc;
  if ((rc = err.ensure(sizeof(int)))) return rc;
  FGB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  if ((rc = oz::slice({M, K, oz::kTM, d_A, lda, nullptr, nullptr}, A, st,
                      oz::kSF32)) ||
      (rc = oz::slice({N, K, oz::kTNF32, d_B, ldb, nullptr, nullptr}, B, st,
                      oz::kSF32)))
    return rc;
  if ((rc = oz::gemm_f32(A, B, d_C, ldc, err.as<int>(), st))) return rc;
  int h = 0;
  FGB_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error("fgb_oz_sgemm_nt: a bounded device wait ran out");
    return FGB_ETIMEOUT;
  }
  return FGB_OK;
}

extern "C" int fgb_wait_expiry_check(long long polls, int *h_how,
                                     void *stream) {
  if (polls < 1 || polls > oz::kWaitLimit) {
    set_error("fgb_wait_expiry_check: polls must be in [1, %lld]",
              oz::kWaitLimit);
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf err, how;
  int rc;
  if ((rc = err.ensure(sizeof(int))) || (rc = how.ensure(2 * sizeof(int))))
    return rc;
  FGB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  FGB_CUDA(cudaMemsetAsync(how.p, 0, 2 * sizeof(int), st));
  oz::k_wait_expiry<<<1, 64, 0, st>>>(polls, err.as<int>(), how.as<int>());
  FGB_LAUNCH_CHECK("k_wait_expiry");
  int h = 0, hw[2] = {0, 0};
  FGB_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaMemcpyAsync(hw, how.p, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                           st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (h_how) { h_how[0] = hw[0]; h_how[1] = hw[1]; }
  if (h) {
    set_error("fgb_wait_expiry_check: a bounded device wait ran out");
    return FGB_ETIMEOUT;
  }
  return FGB_OK;
}

// ------------------------------------------------------------------------
// Sparse-GP stages on the tensor cores (mixed precision mode).
#include "fgb_gemm64.cuh"
#include "fgb_kernels.h"
#include "fgb_model.h"
#include "fgb_profile.h"
#include "fgb_tune.h"

namespace fgb {
namespace oz {
namespace {

// k (16 values of one row) as SO BF16 slices at a fixed scale 2^eK, stored
// at (m, n0) of a 128-row-tile operand of K extent KPv.
template <int SO>
__device__ __forceinline__ void store_k_slices(const double (&k)[16], int eK,
                                               __nv_bfloat16 *Ksl, int m,
                                               int n0, int KPv) {
#pragma unroll
  for (int h = 0; h < 2; h++) {
    long long X[8];
#pragma unroll
    for (int j = 0; j < 8; j++) X[j] = fixed_rn(k[8 * h + j], kBeta * SO - eK);
    store_digits8<SO>(X, Ksl + tiled_index<SO>(m, n0 + 8 * h, KPv, kTM),
                      (size_t)kTM * kKC);
  }
}

// Kernel GEMM epilogue: c = d^ . s^ -> k = sig^2 c^xi, zero for empty
// environments and invalid sparse rows (the same expressions as the FP64
// path).  Per row and tile it keeps sum_n alpha_n k_n (the energy partial,
// finished in a fixed order by k_energy_final) and, for the variance GEMM,
// writes k directly as SO BF16 slices (the variance GEMM's slice count; A
// operand layout, 128-row tiles, K = N padded to 16) under the fixed scale
// 2^eK > sig^2 >= |k|; the FP64 matrix is written only when the variance
// runs in FP64.
template <int S>
struct EpiKernel {
  using Value = double;
  static constexpr bool kFloat = false;
  double *Kd;                 // optional M x N FP64 kernel matrix
  __nv_bfloat16 *Ksl;         // optional slices of K (variance A operand)
  double *Kscale;             // their row scales (all 2^eK)
  int KPv, eK;
  int SO;                     // slices of K written (9, 8, 7 or 6)
  double *epart;              // M x nslots energy partials
  int nslots;                 // B tiles x epilogue warps per quarter
  const double *alpha;
  const unsigned char *valid;
  const int *perm;
  const double *norms;
  double sig2, xi;
  int N;
  __device__ double chunk(int m, bool row_ok, int n0, const double (&v)[16],
                          double acc) const {
    const bool dok = row_ok && norms[perm[m]] >= kEmptyThresh;
    double k[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int n = n0 + j;
      const bool ok = dok && n < N && valid[n];
      k[j] = ok ? sig2 * gemm64::powx(v[j], xi) : 0.0;
      if (n < N && row_ok) acc = fma(alpha[n], k[j], acc);
      if (Kd && n < N && row_ok) Kd[(long long)m * N + n] = k[j];
    }
    if (Ksl && n0 < KPv) {
      // 16 columns = one k chunk of the variance operand: two core-matrix
      // rows of 8 (SO is uniform across the launch)
      switch (SO) {
        case 9: store_k_slices<9>(k, eK, Ksl, m, n0, KPv); break;
        case 8: store_k_slices<8>(k, eK, Ksl, m, n0, KPv); break;
        case 7: store_k_slices<7>(k, eK, Ksl, m, n0, KPv); break;
        default: store_k_slices<6>(k, eK, Ksl, m, n0, KPv); break;
      }
    }
    return acc;
  }
  __device__ void finish(int m, bool row_ok, int slot, double acc) const {
    if (row_ok) epart[(long long)m * nslots + slot] = acc;
    if (Ksl && slot == 0) Kscale[m] = ldexp(1.0, eK);
  }
};

// Variance GEMM epilogue: per-row sum of z^2 over this tile's columns.
struct EpiZsq {
  using Value = double;
  static constexpr bool kFloat = false;
  double *part;
  int nslots, R;   // slots: B tiles x epilogue warps per quarter
  __device__ double chunk(int m, bool row_ok, int n0, const double (&v)[16],
                          double acc) const {
    if (!row_ok) return acc;
#pragma unroll
    for (int j = 0; j < 16; j++)
      if (n0 + j < R) acc = fma(v[j], v[j], acc);
    return acc;
  }
  __device__ void finish(int m, bool row_ok, int slot, double acc) const {
    if (row_ok) part[(long long)m * nslots + slot] = acc;
  }
};

// E_atom = sum of the row's energy partials (fixed order, row_slots_sum).
__global__ void k_energy_final(int M, int ntiles, const double *__restrict__ part,
                               const int *__restrict__ perm,
                               double *__restrict__ e_atom) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int m = (int)(gt / kRowLanes), q = (int)(gt % kRowLanes);
  if (m >= M) return;   // whole lane groups
  const double s = row_slots_sum(part, m, ntiles, q);
  if (q == 0) e_atom[perm[m]] = s;
}

}  // namespace
}  // namespace oz


// Slice the model operands for variant v (slice count and B tile height),
// per species: the normalised sparse rows (B of the kernel GEMM) or the
// L_inv panels (B of the variance GEMM).  Each is done once per variant,
// the first time the variant runs.
static int build_oz_S(fgb_model_s *m, int v, cudaStream_t st) {
  const int S = m->b2.n_species, nd = m->b2.n_d, TN = oz::kTNF64v[v];
  const int SL = oz::kSF64v[v];
  m->ozS[v].clear();
  int rc;
  for (int s = 0; s < S; s++) {
    m->ozS[v].emplace_back(new oz::Sliced());
    const int Ms = m->h_counts[s];
    if (Ms == 0) continue;
    if ((rc = oz::slice({Ms, nd, TN,
                         m->S.as<double>() + (size_t)m->h_offsets[s] * nd, nd,
                         nullptr, nullptr},
                        *m->ozS[v][s], st, SL)))
      return rc;
  }
  m->ozS_ready[v] = true;
  return FGB_OK;
}

static int build_oz_L(fgb_model_s *m, int v, cudaStream_t st) {
  const int S = m->b2.n_species, TN = oz::kTNF64v[v];
  const int SL = oz::kSF64v[v];
  m->ozL[v].clear();
  int rc;
  for (int s = 0; s < S; s++) {
    m->ozL[v].emplace_back(new oz::Sliced());
    const int Ms = m->h_counts[s];
    if (Ms == 0) continue;
    if ((rc = oz::slice({m->h_panel_rows[s], Ms, TN,
                         m->Lp.as<double>() + m->h_panel_off[s], Ms, nullptr,
                         nullptr},
                        *m->ozL[v][s], st, SL)))
      return rc;
  }
  m->ozL_ready[v] = true;
  return FGB_OK;
}

// The slice count as a compile-time constant.
template <class F>
static int with_slices(int S, F &&f) {
  if (S == 8) return f(std::integral_constant<int, 8>{});
  if (S == 7) return f(std::integral_constant<int, 7>{});
  if (S == 6) return f(std::integral_constant<int, 6>{});
  return f(std::integral_constant<int, oz::kS>{});
}

// The sparse set's own environments through the mixed path's kernel and
// variance GEMMs (48-row B tiles), one row per sparse environment: energies
// sum_t alpha_t k(s_i, s_t) with the kernel GEMM at Sk slices and, when
// Sv > 0, local variances k_self - |L_inv k_i|^2 with k written as Sv
// slices and the variance GEMM at Sv slices.  Every sparse row meets
// itself (c = 1, its own alpha), and its variance is the smallest the
// model gives (about the jitter): the largest cancellation.
static int probe_sparse(fgb_model_s *m, int Sk, int Sv, std::vector<double> &E,
                        std::vector<double> &V, cudaStream_t st) {
  const int vk = oz::s_index(Sk) * oz::kF64PerS;
  const int vv = oz::s_index(Sv > 0 ? Sv : oz::kS) * oz::kF64PerS;
  int rc;
  if (!m->ozS_ready[vk] && (rc = build_oz_S(m, vk, st))) return rc;
  if (Sv > 0 && !m->ozL_ready[vv] && (rc = build_oz_L(m, vv, st))) return rc;
  const int M = m->M, nd = m->b2.n_d;
  int maxMs = 0;
  for (int s = 0; s < m->b2.n_species; s++) maxMs = std::max(maxMs, m->h_counts[s]);
  std::vector<int> id(maxMs);
  for (int i = 0; i < maxMs; i++) id[i] = i;
  DevBuf ident, erows, eout, vout, part, err;
  oz::Sliced A, Ksl;
  if ((rc = ident.ensure(sizeof(int) * (maxMs + 1))) ||
      (rc = eout.ensure(sizeof(double) * (M + 1))) ||
      (rc = vout.ensure(sizeof(double) * (M + 1))) ||
      (rc = err.ensure(sizeof(int))))
    return rc;
  FGB_CUDA(cudaMemcpyAsync(ident.p, id.data(), sizeof(int) * maxMs,
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemsetAsync(eout.p, 0, sizeof(double) * (M + 1), st));
  FGB_CUDA(cudaMemsetAsync(vout.p, 0, sizeof(double) * (M + 1), st));
  FGB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  const double sig2 = m->sigma * m->sigma;
  const int eK = std::ilogb(sig2) + 1;
  for (int s = 0; s < m->b2.n_species; s++) {
    const int Ms = m->h_counts[s], off = m->h_offsets[s];
    if (Ms == 0) continue;
    if ((rc = oz::slice({Ms, nd, oz::kTM, m->S.as<double>() + (size_t)off * nd,
                         nd, nullptr, nullptr},
                        A, st, Sk)))
      return rc;
    if (Sv > 0 && (rc = oz::prepare(Ms, Ms, oz::kTM, Sv, Ksl))) return rc;
    const oz::Sliced &B = *m->ozS[vk][s];
    const int slots = B.RP / 16;
    if ((rc = erows.ensure(sizeof(double) * (size_t)Ms * slots))) return rc;
    rc = with_slices(Sk, [&](auto sc) -> int {
      constexpr int S_ = decltype(sc)::value;
      oz::EpiKernel<S_> epi{nullptr,
                            Sv > 0 ? Ksl.q.as<__nv_bfloat16>() : nullptr,
                            Sv > 0 ? Ksl.scale.as<double>() : nullptr,
                            Ksl.KP, eK, Sv, erows.as<double>(), slots,
                            m->alpha.as<double>() + off,
                            m->svalid.as<unsigned char>() + off, ident.as<int>(),
                            m->snorm.as<double>() + off, sig2, m->power, Ms};
      return oz::gemm_s<S_>(A, B, false, epi, err.as<int>(), st);
    });
    if (rc) return rc;
    oz::k_energy_final<<<
        ceil_div((long long)Ms * kRowLanes, 128), 128, 0, st>>>(
        Ms, slots, erows.as<double>(), ident.as<int>(),
        eout.as<double>() + off);
    FGB_LAUNCH_CHECK("k_energy_final");
    if (Sv > 0) {
      const oz::Sliced &L = *m->ozL[vv][s];
      const int vslots = L.RP / 16;
      if ((rc = part.ensure(sizeof(double) * (size_t)Ms * vslots))) return rc;
      oz::EpiZsq zepi{part.as<double>(), vslots, m->h_panel_rows[s]};
      rc = with_slices(Sv, [&](auto sc) -> int {
        return oz::gemm_s<decltype(sc)::value>(Ksl, L, true, zepi,
                                               err.as<int>(), st);
      });
      if (rc) return rc;
      if ((rc = launch_variance_final(Ms, vslots, part.as<double>(),
                                      ident.as<int>(),
                                      m->snorm.as<double>() + off, sig2,
                                      m->power, vout.as<double>() + off, st)))
        return rc;
    }
  }
  E.assign(M, 0.0);
  V.assign(M, 0.0);
  int h = 0;
  if (M > 0) {
    FGB_CUDA(cudaMemcpyAsync(E.data(), eout.p, sizeof(double) * M,
                             cudaMemcpyDeviceToHost, st));
    FGB_CUDA(cudaMemcpyAsync(V.data(), vout.p, sizeof(double) * M,
                             cudaMemcpyDeviceToHost, st));
  }
  FGB_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error("slice-count probe: a bounded device wait ran out");
    return FGB_ETIMEOUT;
  }
  return FGB_OK;
}

static double max_abs_diff(const std::vector<double> &a,
                           const std::vector<double> &b) {
  double e = 0.0;
  for (size_t i = 0; i < a.size(); i++) e = std::max(e, std::fabs(a[i] - b[i]));
  return e;
}

// Slice counts of the kernel and variance GEMMs, chosen per model from the
// sparse set's own environments (probe_sparse) against 9 slices:
//   kernel GEMM: the fewest of 7, 8, 9 whose energies differ by at most
//     kEnergyProbe = 1e-7 eV/atom, a tenth of the mixed path's energy
//     budget of 1e-6 eV/atom;
//   variance GEMM: the fewest of 6, 7, 8, 9 whose local variances differ
//     by at most kVarProbe sigma^2 = 5e-9 sigma^2, half the stated
//     local-variance budget of 1e-8 sigma^2 (local std sqrt|var| / sigma
//     then errs by under 1e-4 anywhere, 1e-7 at std 0.05).
// On held-out structures of the 2-species alloy model the errors track
// these probes to within a factor of two (exact CPU emulation of the
// slicing: energy 4.7e-8 eV/atom at 7 slices against a probe of 6.6e-8;
// variance 9.4e-9 at 6 slices against 1.4e-8), the variance error coming
// almost entirely from the variance GEMM's own slicing.  Forced counts
// (fgb_model_set_slices) skip the probes.  Measured once per model, before
// its first mixed prediction.
int choose_kernel_slices(fgb_model_s *m, cudaStream_t st) {
  constexpr double kEnergyProbe = 1e-7;   // eV/atom
  constexpr double kVarProbe = 5e-9;      // x sigma^2
  m->oz_S = m->oz_S_forced ? m->oz_S_forced : oz::kS;
  m->oz_Sv = m->oz_Sv_forced ? m->oz_Sv_forced : oz::kS;
  m->oz_err_est = 0.0;
  m->oz_var_err_est = 0.0;
  m->slices_chosen = true;
  if (m->M == 0) return FGB_OK;
  int rc;
  std::vector<double> E9, V9, E, V;
  if (!m->oz_S_forced) {
    if ((rc = probe_sparse(m, oz::kS, 0, E9, V9, st))) return rc;
    for (int S = oz::kMinKernelSlices; S < oz::kS; S++) {
      if ((rc = probe_sparse(m, S, 0, E, V, st))) return rc;
      const double e = max_abs_diff(E, E9);
      if (e <= kEnergyProbe) {
        m->oz_S = S;
        m->oz_err_est = e;
        break;
      }
    }
  }
  if (!m->oz_Sv_forced) {
    const double vmax = kVarProbe * m->sigma * m->sigma;
    if ((rc = probe_sparse(m, m->oz_S, oz::kS, E9, V9, st))) return rc;
    for (int S = oz::kMinVarianceSlices; S < oz::kS; S++) {
      if ((rc = probe_sparse(m, m->oz_S, S, E, V, st))) return rc;
      const double e = max_abs_diff(V, V9);
      if (e <= vmax) {
        m->oz_Sv = S;
        m->oz_var_err_est = e;
        break;
      }
    }
  }
  return FGB_OK;
}

int kernel_stage_oz(fgb_model_s *m, int N, const std::vector<int> &counts,
                    bool want_w, bool want_var, double *d_e_atom, double *d_var,
                    cudaStream_t st, bool fixed, const ChunkHook *after_chunk) {
  int rc;
  if (want_w) {
    set_error("tensor-core kernel stage: adjoint weights are not produced");
    return FGB_ENOTSUP;
  }
  // the model's slice counts; each GEMM's tile candidates are variants
  // sb + q (kernel GEMM, sparse rows at SL slices) and vb + q (variance
  // GEMM, L_inv panels at SV slices)
  const int SL = m->oz_S, SV = m->oz_Sv;
  const int sb = oz::s_index(SL) * oz::kF64PerS;
  const int vb = oz::s_index(SV) * oz::kF64PerS;
  if (!m->ozS_ready[sb] || (want_var && !m->ozL_ready[vb])) {
    if (fixed) {
      set_error("tensor-core kernel stage: operands not sliced before a fixed call");
      return FGB_EINVAL;
    }
    if (!m->ozS_ready[sb] && (rc = build_oz_S(m, sb, st))) return rc;
    if (want_var && !m->ozL_ready[vb] && (rc = build_oz_L(m, vb, st)))
      return rc;
  }
  // candidate q usable without preparation; prepare it (not in fixed calls)
  auto usable_k = [m, sb](int q) { return m->ozS_ready[sb + q]; };
  auto usable_v = [m, vb](int q) { return m->ozL_ready[vb + q]; };
  auto prepare_k = [&](int q) -> int {
    if (m->ozS_ready[sb + q]) return FGB_OK;
    if (fixed) {
      set_error("tensor-core kernel stage: tile variant not prepared");
      return FGB_EINVAL;
    }
    return build_oz_S(m, sb + q, st);
  };
  auto prepare_v = [&](int q) -> int {
    if (m->ozL_ready[vb + q]) return FGB_OK;
    if (fixed) {
      set_error("tensor-core kernel stage: tile variant not prepared");
      return FGB_EINVAL;
    }
    return build_oz_L(m, vb + q, st);
  };
  // descriptor rows: the kernel GEMM's slices, or all kS when the fold
  // guard sends the force product through the FP64-level GEMM (the
  // FP32-level force GEMM reads the first kSF32)
  const int SA = m->force_f64 ? oz::kS : SL;
  const B2Params &p = m->b2;
  const int nd = p.n_d;
  const double sig2 = m->sigma * m->sigma;
  // fixed scale of the sliced kernel matrix: |k| <= sig^2 < 2^eK
  const int eK = std::ilogb(sig2) + 1;
  if ((rc = m->ws.ozerr.ensure(sizeof(int)))) return rc;
  int base = 0;
  const int kRows = 32768;
  for (int s = 0; s < p.n_species; s++) {
    const int Ns = counts[s], Ms = m->h_counts[s];
    const int *perm_s = m->ws.perm.as<int>() + base;
    base += Ns;
    if (Ns > 0 && Ms == 0 && want_var) {
      if ((rc = launch_variance_final(Ns, 0, nullptr, perm_s,
                                      m->ws.norms.as<double>(), sig2, m->power,
                                      d_var, st)))
        return rc;
    }
    const bool var_oz = want_var;
    // row partial sums: one slot per 16 columns, for the widest padding
    auto slots = [](int n) {
      int w = 0;
      for (int v = 0; v < oz::kF64Variants; v++)
        w = std::max(w, oz::pad_to(n, oz::kTNF64v[v]) / 16);
      return w;
    };
    const int R = m->h_panel_rows[s];
    const int kslots = Ms > 0 ? slots(Ms) : 0;
    const int vslots = Ms > 0 ? slots(R) : 0;
    for (int r0 = 0; r0 < Ns && Ms > 0; r0 += kRows) {
      const int Mr = std::min(kRows, Ns - r0);
      const int *perm = perm_s + r0;
      if ((rc = m->ws.erows.ensure(sizeof(double) * (size_t)Mr * kslots)) ||
          (var_oz && (rc = oz::prepare(Mr, Ms, oz::kTM, SV, m->ws.ozK))))
        return rc;
      int vk = 0;
      {
        StageTimer _pt(kStRowSlice, st, 2);   // row scales, slices
        if ((rc = oz::slice({Mr, nd, oz::kTM, m->ws.B2.as<double>(), nd, perm,
                             m->ws.norms.as<double>(),
                             m->ws.rowmax.as<double>()},
                            m->ws.ozA, st, SA)))
          return rc;
      }
      {
        StageTimer _pt(kStKernelGemm, st, 1);
        auto launch = [&](int q) -> int {
          int r;
          if ((r = prepare_k(q))) return r;
          const oz::Sliced &B = *m->ozS[sb + q][s];
          return with_slices(SL, [&](auto sc) -> int {
            constexpr int S_ = decltype(sc)::value;
            oz::EpiKernel<S_> epi{
                nullptr, var_oz ? m->ws.ozK.q.as<__nv_bfloat16>() : nullptr,
                var_oz ? m->ws.ozK.scale.as<double>() : nullptr, m->ws.ozK.KP,
                eK, SV, m->ws.erows.as<double>(), B.RP / 16,
                m->alpha.as<double>() + m->h_offsets[s],
                m->svalid.as<unsigned char>() + m->h_offsets[s], perm,
                m->ws.norms.as<double>(), sig2, m->power, Ms};
            return oz::gemm_s<S_>(m->ws.ozA, B, false, epi,
                                  m->ws.ozerr.as<int>(), st);
          });
        };
        if ((rc = tune::run(tune::kOpKernelGemm, Mr, Ms, nd, oz::n_cand_s(SL),
                            launch, usable_k, st, fixed, &vk)))
          return rc;
        vk += sb;
      }
      {
        StageTimer _pt(kStRowEnergy, st);
        oz::k_energy_final<<<
            ceil_div((long long)Mr * kRowLanes, 128), 128, 0, st>>>(
            Mr, m->ozS[vk][s]->RP / 16, m->ws.erows.as<double>(), perm,
            d_e_atom);
        FGB_LAUNCH_CHECK("k_energy_final");
      }
      if (var_oz) {
        if ((rc = m->ws.part.ensure(sizeof(double) * (size_t)Mr * vslots)))
          return rc;
        int vv = 0;
        {
          StageTimer _pt(kStVarianceGemm, st);
          auto launch = [&](int q) -> int {
            int r;
            if ((r = prepare_v(q))) return r;
            const oz::Sliced &B = *m->ozL[vb + q][s];
            oz::EpiZsq epi{m->ws.part.as<double>(), B.RP / 16, R};
            return with_slices(SV, [&](auto sc) -> int {
              return oz::gemm_s<decltype(sc)::value>(
                  m->ws.ozK, B, true, epi, m->ws.ozerr.as<int>(), st);
            });
          };
          if ((rc = tune::run(tune::kOpVarianceGemm, Mr, R, Ms,
                              oz::n_cand_s(SV), launch, usable_v, st, fixed,
                              &vv)))
            return rc;
          vv += vb;
        }
        if ((rc = launch_variance_final(Mr, m->ozL[vv][s]->RP / 16,
                                        m->ws.part.as<double>(), perm,
                                        m->ws.norms.as<double>(), sig2,
                                        m->power, d_var, st)))
          return rc;
      }
      if (after_chunk && (rc = (*after_chunk)(s, Mr, perm))) return rc;
    }
  }
  return FGB_OK;
}

}  // namespace fgb
