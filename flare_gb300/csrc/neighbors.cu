// K1: cell-list neighbour build, bit-exact against the reference's brute-force
// list (src/flare_pp/structure.cpp:52-118).
//
// The reference tests every atom j and every image shift s in
// [-sweep, sweep]^3 for 0 < |w_j - w_i + s.cell| < cutoff.  Here each atom is
// binned by its fractional coordinate; bins are at least `cutoff` wide
// (perpendicular width), so all pairs within the cutoff sit in the 3x3x3 (or
// wider, for small cells) block of bin images around atom i.  Each candidate
// (j, s) is tested with the reference's arithmetic in the same FP64
// operation order (explicit _rn intrinsics, no FMA), filtered to
// |s_a| <= sweep exactly as the reference's loop bounds, and each atom's
// segment is finally ordered by (j, s1, s2, s3) — the reference's loop
// order.  The result is the same set, the same order and the same bits.
//
// FP64 arithmetic is scarce on this GPU (about 2 operations per clock per
// SM), so every candidate is first measured in FP32 from FP32 copies of the
// wrapped positions and the cell.  A margin well above the FP32 rounding
// error (set per structure in make_geom) sorts candidates into certainly
// outside, certainly inside, or near the cutoff (or near zero distance);
// candidates not certainly outside are evaluated in FP64 by the fill, whose
// FP64 test alone decides what is written, and which checks that no
// certainly-inside candidate fails it.  One warp serves one atom, a lane
// per bin image.
//
// The fill normally runs once, into per-atom slots sized from the densest
// structure (no counting pass, no host synchronisation); the counts are
// scanned on the device and the rank sort gathers the slots into the CSR
// list.  An atom with more pairs than its slots flags the build, which is
// then repeated with a counting pass (k_count: only near-cutoff candidates
// take the FP64 test there) that sizes the CSR segments exactly; the fill
// then also checks its counts against that pass.
#include <limits>

#include "fgb_internal.h"

namespace fgb {

namespace {

// Integer-to-float conversions and divisions by run-time divisors go
// through the FP64/conversion pipe, which this GPU runs at a small fraction
// of the integer and FP32 rates; the candidate loops use the forms below.

// n / d for the multiplier m = floor(2^32 / d) + 1 (see StrucGeom).
__device__ __forceinline__ int udiv(int n, unsigned long long m) {
  return (int)(((unsigned long long)(unsigned)n * m) >> 32);
}

// floor(t / nb[k]) for t > -kk[k] - 1
__device__ __forceinline__ int floordiv_k(const StrucGeom &g, int k, int t) {
  return udiv(t + g.wrap_c[k] * g.nb[k], g.m_nb[k]) - g.wrap_c[k];
}

// (float)s for |s| < 2^22, exactly, with one FP32 subtraction: the bits of
// 1.5 * 2^23 + s minus 1.5 * 2^23.
__device__ __forceinline__ float small_int_to_float(int s) {
  return __fsub_rn(__int_as_float(0x4B400000 + s), 12582912.0f);
}

// Search-block image img -> offsets (d0, d1, d2) in [-kk, kk]^3.
__device__ __forceinline__ void image_offsets(const StrucGeom &g, int img,
                                              int &d0, int &d1, int &d2) {
  const int n1 = 2 * g.kk[1] + 1, n2 = 2 * g.kk[2] + 1;
  const int q = udiv(img, g.m_n2);     // img / n2
  const int p = udiv(q, g.m_n1);       // img / (n1 n2)
  d2 = img - q * n2 - g.kk[2];
  d1 = q - p * n1 - g.kk[1];
  d0 = p - g.kk[0];
}

// frac = (p * ct) * cdi ; f = frac - floor(frac); w = (f * cd) * cti
__global__ void k_wrap_bin(int n, const double *__restrict__ pos,
                           const int *__restrict__ atom_struct,
                           const StrucGeom *__restrict__ geom,
                           double *__restrict__ wrapped, float4 *__restrict__ w32,
                           int *__restrict__ raw,
                           int *__restrict__ home, int *__restrict__ slot,
                           int *__restrict__ bin_count, int *__restrict__ flag) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const StrucGeom &g = geom[atom_struct[a]];
  double p0 = pos[3 * a], p1 = pos[3 * a + 1], p2 = pos[3 * a + 2];
  double t[3], f[3], u[3];
#pragma unroll
  for (int k = 0; k < 3; k++)
    t[k] = __dadd_rn(__dadd_rn(__dmul_rn(p0, g.ct[k]), __dmul_rn(p1, g.ct[3 + k])),
                     __dmul_rn(p2, g.ct[6 + k]));
#pragma unroll
  for (int k = 0; k < 3; k++)
    f[k] = __dadd_rn(__dadd_rn(__dmul_rn(t[0], g.cdi[k]), __dmul_rn(t[1], g.cdi[3 + k])),
                     __dmul_rn(t[2], g.cdi[6 + k]));
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if (!isfinite(f[k])) { bad = true; f[k] = 0.0; }
    f[k] = __dsub_rn(f[k], floor(f[k]));
  }
#pragma unroll
  for (int k = 0; k < 3; k++)
    u[k] = __dadd_rn(__dadd_rn(__dmul_rn(f[0], g.cd[k]), __dmul_rn(f[1], g.cd[3 + k])),
                     __dmul_rn(f[2], g.cd[6 + k]));
  double w[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    w[k] = __dadd_rn(__dadd_rn(__dmul_rn(u[0], g.cti[k]), __dmul_rn(u[1], g.cti[3 + k])),
                     __dmul_rn(u[2], g.cti[6 + k]));
    wrapped[3 * a + k] = w[k];
  }
  int hb[3], top = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    // f in [0, 1]; raw bin in [0, nb] (nb only when f rounded up to 1.0)
    int b = (int)floor(f[k] * (double)g.nb[k]);
    b = b < 0 ? 0 : (b > g.nb[k] ? g.nb[k] : b);
    raw[3 * a + k] = b;
    if (b == g.nb[k]) top |= 1 << k;
    hb[k] = b == g.nb[k] ? 0 : b;
  }
  // bad positions were replaced by 0 above; keep the FP32 copy finite too
  w32[a] = make_float4(bad ? 0.f : (float)w[0], bad ? 0.f : (float)w[1],
                       bad ? 0.f : (float)w[2], __int_as_float(top));
  if (bad) atomicExch(flag, 1);
  int hbin = g.bin0 + (hb[0] * g.nb[1] + hb[1]) * g.nb[2] + hb[2];
  home[a] = hbin;
  slot[a] = atomicAdd(&bin_count[hbin], 1);
}

__global__ void k_bin_fill(int n, const int *__restrict__ home,
                           const int *__restrict__ slot,
                           const int *__restrict__ bin_start,
                           int *__restrict__ bin_atoms) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  bin_atoms[bin_start[home[a]] + slot[a]] = a;
}

// Candidate classes of the FP32 prefilter.
enum : int { kOut = 0, kIn = 1, kNear = 2 };

// Visit this lane's share of atom i's candidates (j, s): the bin images
// lane, lane + 32, ... of the search block.  fn(j, s0, s1, s2, cls) gets every
// candidate that passes the reference's sweep filter and is not certainly
// outside the cutoff by the FP32 distance.
template <typename Fn>
__device__ __forceinline__ void visit_lane(int lane, const StrucGeom &g,
                                           float4 wi, int b0, int b1, int b2,
                                           const float4 *__restrict__ w32,
                                           const int *__restrict__ bin_start,
                                           const int *__restrict__ bin_atoms,
                                           Fn fn) {
  const int n0 = 2 * g.kk[0] + 1, n1 = 2 * g.kk[1] + 1, n2 = 2 * g.kk[2] + 1;
  const int nimg = n0 * n1 * n2;
  for (int img = lane; img < nimg; img += 32) {
    int d0, d1, d2;
    image_offsets(g, img, d0, d1, d2);
    const int t0 = b0 + d0, t1 = b1 + d1, t2 = b2 + d2;
    const int q0 = floordiv_k(g, 0, t0), q1 = floordiv_k(g, 1, t1),
              q2 = floordiv_k(g, 2, t2);
    const int h0 = t0 - q0 * g.nb[0], h1 = t1 - q1 * g.nb[1],
              h2 = t2 - q2 * g.nb[2];
    const int bin = g.bin0 + (h0 * g.nb[1] + h1) * g.nb[2] + h2;
    const int qb = bin_start[bin], qe = bin_start[bin + 1];
    for (int q = qb; q < qe; q++) {
      const int j = bin_atoms[q];
      const float4 wj = w32[j];
      const int top = __float_as_int(wj.w);
      // image shift relative to j's wrapped position
      const int s0 = q0 - (top & 1), s1 = q1 - ((top >> 1) & 1),
                s2 = q2 - ((top >> 2) & 1);
      if (s0 < -g.sweep || s0 > g.sweep || s1 < -g.sweep || s1 > g.sweep ||
          s2 < -g.sweep || s2 > g.sweep)
        continue;
      const float f0 = small_int_to_float(s0), f1 = small_int_to_float(s1),
                  f2 = small_int_to_float(s2);
      const float x = (wj.x - wi.x) + f0 * g.cell32[0] + f1 * g.cell32[3] +
                      f2 * g.cell32[6];
      const float y = (wj.y - wi.y) + f0 * g.cell32[1] + f1 * g.cell32[4] +
                      f2 * g.cell32[7];
      const float z = (wj.z - wi.z) + f0 * g.cell32[2] + f1 * g.cell32[5] +
                      f2 * g.cell32[8];
      const float d2 = x * x + y * y + z * z;
      if (d2 > g.d2_out) continue;
      fn(j, s0, s1, s2, (d2 < g.d2_in && d2 > g.d2_zero) ? kIn : kNear);
    }
  }
}

// The reference's FP64 test for one candidate, in its operation order;
// returns true (and x, y, z, d) for a pair inside the cutoff.
__device__ __forceinline__ bool exact_pair(const StrucGeom &g,
                                           const double *__restrict__ wrapped,
                                           double wi0, double wi1, double wi2,
                                           int j, int s0, int s1, int s2,
                                           double cutoff, double &x, double &y,
                                           double &z, double &d) {
  const double e0 = __dsub_rn(wrapped[3 * j], wi0);
  const double e1 = __dsub_rn(wrapped[3 * j + 1], wi1);
  const double e2 = __dsub_rn(wrapped[3 * j + 2], wi2);
  const double f0 = (double)s0, f1 = (double)s1, f2 = (double)s2;
  x = __dadd_rn(__dadd_rn(__dadd_rn(e0, __dmul_rn(f0, g.cell[0])),
                          __dmul_rn(f1, g.cell[3])),
                __dmul_rn(f2, g.cell[6]));
  y = __dadd_rn(__dadd_rn(__dadd_rn(e1, __dmul_rn(f0, g.cell[1])),
                          __dmul_rn(f1, g.cell[4])),
                __dmul_rn(f2, g.cell[7]));
  z = __dadd_rn(__dadd_rn(__dadd_rn(e2, __dmul_rn(f0, g.cell[2])),
                          __dmul_rn(f1, g.cell[5])),
                __dmul_rn(f2, g.cell[8]));
  d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)),
                           __dmul_rn(z, z)));
  return d < cutoff && d != 0.0;
}

// Warp per atom: number of pairs.  FP64 only for candidates near the cutoff
// or near zero distance.
__global__ void k_count(int n, const int *__restrict__ atom_struct,
                        const StrucGeom *__restrict__ geom,
                        const double *__restrict__ wrapped,
                        const float4 *__restrict__ w32,
                        const int *__restrict__ raw,
                        const int *__restrict__ bin_start,
                        const int *__restrict__ bin_atoms, double cutoff,
                        int *__restrict__ counts) {
  const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const StrucGeom &g = geom[atom_struct[i]];
  const double wi0 = wrapped[3 * i], wi1 = wrapped[3 * i + 1],
               wi2 = wrapped[3 * i + 2];
  int c = 0;
  visit_lane(lane, g, w32[i], raw[3 * i], raw[3 * i + 1], raw[3 * i + 2], w32,
             bin_start, bin_atoms, [&](int j, int s0, int s1, int s2, int cls) {
               double x, y, z, d;
               if (cls == kIn ||
                   exact_pair(g, wrapped, wi0, wi1, wi2, j, s0, s1, s2, cutoff,
                              x, y, z, d))
                 c++;
             });
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
  if (lane == 0) counts[i] = c;
}

// One lane's position in its candidate stream: bin images lane, lane + 32,
// ... of the search block and the atoms of the current image's bin.
struct LaneCursor {
  int img, q, qe, q0, q1, q2;
};

__device__ __forceinline__ void cursor_seek(LaneCursor &c, const StrucGeom &g,
                                            int b0, int b1, int b2,
                                            const int *__restrict__ bin_start) {
  const int n1 = 2 * g.kk[1] + 1, n2 = 2 * g.kk[2] + 1;
  const int nimg = (2 * g.kk[0] + 1) * n1 * n2;
  while (c.q >= c.qe && c.img < nimg) {
    int d0, d1, d2;
    image_offsets(g, c.img, d0, d1, d2);
    const int t0 = b0 + d0, t1 = b1 + d1, t2 = b2 + d2;
    c.q0 = floordiv_k(g, 0, t0);
    c.q1 = floordiv_k(g, 1, t1);
    c.q2 = floordiv_k(g, 2, t2);
    const int h0 = t0 - c.q0 * g.nb[0], h1 = t1 - c.q1 * g.nb[1],
              h2 = t2 - c.q2 * g.nb[2];
    const int bin = g.bin0 + (h0 * g.nb[1] + h1) * g.nb[2] + h2;
    c.q = bin_start[bin];
    c.qe = bin_start[bin + 1];
    c.img += 32;
  }
}

constexpr int kFillWarps = 4;   // warps (atoms) per block of k_fill
constexpr int kFillBlocks = 8;  // resident blocks per SM (64 registers)
constexpr int kQueue = 64;      // per-warp candidate queue

// Warp per atom: write the pairs (key = local j, packed shift; FP64
// relative vector and distance) into the atom's segment; the rank sort that
// follows puts them in canonical order.  Segments are either the exact CSR
// segments of a count pass (cap = 0) or fixed slots [i cap, (i + 1) cap)
// of a single pass (cap > 0), whose pair counts go to counts_out; a
// single-pass atom with more than cap pairs sets flag[3] and keeps cap.
// The lanes advance through their candidate streams in lockstep;
// candidates that pass the FP32 filter are compacted into a shared-memory
// queue and evaluated in FP64 32 at a time, so the FP64 work runs on full
// warps.  flag[1] is set when the FP64 decisions disagree with the count
// pass or with a certain-inside class.
__global__ void __launch_bounds__(32 * kFillWarps, kFillBlocks)
k_fill(int n, const int *__restrict__ atom_struct,
       const StrucGeom *__restrict__ geom, const double *__restrict__ wrapped,
       const float4 *__restrict__ w32, const int *__restrict__ raw,
       const int *__restrict__ bin_start, const int *__restrict__ bin_atoms,
       double cutoff, const long long *__restrict__ offsets, long long cap,
       int *__restrict__ counts_out, unsigned long long *__restrict__ key,
       double4_16a *__restrict__ rel, int *__restrict__ flag) {
  __shared__ int2 queue[kFillWarps][kQueue];
  const int wib = threadIdx.x >> 5;
  const int i = blockIdx.x * kFillWarps + wib;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  int2 *qu = queue[wib];
  const StrucGeom &g = geom[atom_struct[i]];
  const double wi0 = wrapped[3 * i], wi1 = wrapped[3 * i + 1],
               wi2 = wrapped[3 * i + 2];
  const float4 wi = w32[i];
  const int b0 = raw[3 * i], b1 = raw[3 * i + 1], b2 = raw[3 * i + 2];
  const long long seg = cap ? (long long)i * cap : offsets[i];
  const long long seg_end = cap ? seg + cap : offsets[i + 1];
  const unsigned lt = (1u << lane) - 1u;
  LaneCursor c{lane, 0, 0, 0, 0, 0};
  cursor_seek(c, g, b0, b1, b2, bin_start);
  int queued = 0;            // warp-uniform
  long long written = 0;     // warp-uniform
  bool bad = false, over = false;
  // evaluate queue entries [0, m) in FP64, one per lane, and write the pairs
  auto drain = [&](int m) {
    bool in = false, certain = false;
    int j = 0, s0 = 0, s1 = 0, s2 = 0;
    double x = 0, y = 0, z = 0, d = 0;
    if (lane < m) {
      const int2 e = qu[lane];
      j = e.x;
      s0 = ((e.y >> 16) & 0xFF) - 128;
      s1 = ((e.y >> 8) & 0xFF) - 128;
      s2 = (e.y & 0xFF) - 128;
      certain = (e.y >> 24) & 1;
      in = exact_pair(g, wrapped, wi0, wi1, wi2, j, s0, s1, s2, cutoff, x, y,
                      z, d);
      if (certain && !in) bad = true;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (in) {
      const long long p = seg + written + __popc(bal & lt);
      if (p < seg_end) {
        const unsigned long long jl = (unsigned long long)(j - g.atom0);
        key[p] = (jl << 24) | ((unsigned long long)(s0 + 128) << 16) |
                 ((unsigned long long)(s1 + 128) << 8) |
                 (unsigned long long)(s2 + 128);
        rel[p] = make_double4_16a(d, x, y, z);
      } else if (cap) {
        over = true;
      } else {
        bad = true;
      }
    }
    written += __popc(bal);
  };
  for (;;) {
    const bool has = c.q < c.qe;
    if (__ballot_sync(0xffffffffu, has) == 0u) break;
    bool pass = false;
    int packed = 0, j = 0;
    if (has) {
      j = bin_atoms[c.q];
      const float4 wj = w32[j];
      const int top = __float_as_int(wj.w);
      const int s0 = c.q0 - (top & 1), s1 = c.q1 - ((top >> 1) & 1),
                s2 = c.q2 - ((top >> 2) & 1);
      if (s0 >= -g.sweep && s0 <= g.sweep && s1 >= -g.sweep &&
          s1 <= g.sweep && s2 >= -g.sweep && s2 <= g.sweep) {
        const float f0 = small_int_to_float(s0),
                    f1 = small_int_to_float(s1), f2 = small_int_to_float(s2);
        const float x = (wj.x - wi.x) + f0 * g.cell32[0] + f1 * g.cell32[3] +
                        f2 * g.cell32[6];
        const float y = (wj.y - wi.y) + f0 * g.cell32[1] + f1 * g.cell32[4] +
                        f2 * g.cell32[7];
        const float z = (wj.z - wi.z) + f0 * g.cell32[2] + f1 * g.cell32[5] +
                        f2 * g.cell32[8];
        const float d2 = x * x + y * y + z * z;
        if (d2 <= g.d2_out) {
          pass = true;
          const int certain = (d2 < g.d2_in && d2 > g.d2_zero) ? 1 : 0;
          packed = (certain << 24) | ((s0 + 128) << 16) | ((s1 + 128) << 8) |
                   (s2 + 128);
        }
      }
      c.q++;
      cursor_seek(c, g, b0, b1, b2, bin_start);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, pass);
    if (pass) qu[queued + __popc(bal & lt)] = make_int2(j, packed);
    queued += __popc(bal);
    __syncwarp();
    if (queued >= 32) {
      drain(32);
      __syncwarp();
      // move the remainder (at most 31 entries) to the front
      int2 rest = make_int2(0, 0);
      if (lane < queued - 32) rest = qu[32 + lane];
      __syncwarp();
      if (lane < queued - 32) qu[lane] = rest;
      queued -= 32;
      __syncwarp();
    }
  }
  if (queued > 0) drain(queued);
  if (cap) {
    if (lane == 0) counts_out[i] = (int)(written < cap ? written : cap);
    if (__any_sync(0xffffffffu, over) && lane == 0) atomicExch(flag + 3, 1);
  } else if (seg + written != seg_end) {
    bad = true;
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicExch(flag + 1, 1);
}

// Warp per atom: rank each key within the atom's segment (keys are unique),
// scatter into canonical (j, s1, s2, s3) order at the atom's CSR segment.
// The source segment is the CSR one (cap = 0) or the single pass's slots
// from i cap (the CSR segment's length).
__global__ void k_rank_scatter(int n, const int *__restrict__ atom_struct,
                               const StrucGeom *__restrict__ geom,
                               const long long *__restrict__ offsets,
                               long long cap,
                               const unsigned long long *__restrict__ key,
                               const double4_16a *__restrict__ rel_in,
                               int *__restrict__ nbr_j,
                               int *__restrict__ nbr_shift,
                               double4_16a *__restrict__ rel_out) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const long long b = offsets[warp], e = offsets[warp + 1];
  const long long sb = cap ? (long long)warp * cap : b, se = sb + (e - b);
  int atom0 = geom[atom_struct[warp]].atom0;
  for (long long p = sb + lane; p < se; p += 32) {
    unsigned long long k = key[p];
    long long r = 0;
    for (long long q = sb; q < se; q++) r += key[q] < k ? 1 : 0;
    long long dst = b + r;
    nbr_j[dst] = atom0 + (int)(k >> 24);
    nbr_shift[dst] = (int)(k & 0xFFFFFFull);
    rel_out[dst] = rel_in[p];
  }
}

// twin of pair p = (i -> j, s) is (j -> i, -s) in j's segment (binary
// search of j's sorted segment); warp per atom, lane per pair.
__global__ void k_twin(int n, const int *__restrict__ atom_struct,
                       const StrucGeom *__restrict__ geom,
                       const long long *__restrict__ offsets,
                       const int *__restrict__ nbr_j,
                       const int *__restrict__ nbr_shift,
                       long long *__restrict__ twin, int *__restrict__ flag) {
  const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const int atom0 = geom[atom_struct[i]].atom0;
  for (long long p = offsets[i] + lane; p < offsets[i + 1]; p += 32) {
    const int j = nbr_j[p];
    const int sh = nbr_shift[p];
    const int s0 = ((sh >> 16) & 0xFF) - 128, s1 = ((sh >> 8) & 0xFF) - 128,
              s2 = (sh & 0xFF) - 128;
    const unsigned long long want = ((unsigned long long)(i - atom0) << 24) |
                                    ((unsigned long long)(-s0 + 128) << 16) |
                                    ((unsigned long long)(-s1 + 128) << 8) |
                                    (unsigned long long)(-s2 + 128);
    long long lo = offsets[j], hi = offsets[j + 1] - 1, found = -1;
    while (lo <= hi) {
      const long long mid = (lo + hi) >> 1;
      const unsigned long long km =
          ((unsigned long long)(nbr_j[mid] - atom0) << 24) |
          (unsigned long long)nbr_shift[mid];
      if (km == want) { found = mid; break; }
      if (km < want) lo = mid + 1; else hi = mid - 1;
    }
    twin[p] = found;
    if (found < 0) atomicExch(flag + 2, 1);
  }
}

__global__ void k_export(int n, const long long *__restrict__ offsets,
                         const int *__restrict__ atom_struct,
                         const StrucGeom *__restrict__ geom,
                         const int *__restrict__ nbr_j,
                         const int *__restrict__ nbr_shift,
                         const double4_16a *__restrict__ rel, int *cnt, int *sidx,
                         int *shifts, double *relp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int atom0 = geom[atom_struct[i]].atom0;
  if (cnt) cnt[i] = (int)(offsets[i + 1] - offsets[i]);
  for (long long p = offsets[i]; p < offsets[i + 1]; p++) {
    if (sidx) sidx[p] = nbr_j[p] - atom0;
    if (shifts) {
      int sh = nbr_shift[p];
      shifts[3 * p] = ((sh >> 16) & 0xFF) - 128;
      shifts[3 * p + 1] = ((sh >> 8) & 0xFF) - 128;
      shifts[3 * p + 2] = (sh & 0xFF) - 128;
    }
    if (relp) {
      double4_16a r = rel[p];
      relp[4 * p] = r.x; relp[4 * p + 1] = r.y;
      relp[4 * p + 2] = r.z; relp[4 * p + 3] = r.w;
    }
  }
}

// Fixed rebuilds: segments past the reserved capacity are cut at it (so
// every later kernel stays inside the buffers) and flag[3] records it.
__global__ void k_clamp_offsets(int n, long long cap,
                                long long *__restrict__ offsets,
                                int *__restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  const long long o = offsets[i];
  if (o > cap) {
    offsets[i] = cap;
    if (i == n) atomicExch(flag + 3, 1);
  }
}

}  // namespace

// Host geometry set-up for one structure: bins and search widths.
static void make_geom(const double *cell, double cutoff, int atom0, int natoms,
                      int bin0, StrucGeom &g, double &single_sweep) {
  for (int k = 0; k < 9; k++) g.cell[k] = cell[k];
  cell_setup(cell, g.ct, g.cti, g.cd, g.cdi, &g.volume, &single_sweep);
  g.sweep = (int)std::ceil(cutoff / single_sweep);
  // Perpendicular widths h_a = V / |b x c| (cyclic).
  const double *a = cell, *b = cell + 3, *c = cell + 6;
  const double *v[3] = {a, b, c};
  double h[3];
  for (int k = 0; k < 3; k++) {
    const double *p = v[(k + 1) % 3], *q = v[(k + 2) % 3];
    double cx = p[1] * q[2] - p[2] * q[1];
    double cy = p[2] * q[0] - p[0] * q[2];
    double cz = p[0] * q[1] - p[1] * q[0];
    h[k] = g.volume / std::sqrt(cx * cx + cy * cy + cz * cz);
  }
  const double rc = cutoff * (1.0 + 1e-9);
  long long cap = std::max<long long>(27, 2LL * natoms);
  for (int k = 0; k < 3; k++) {
    double nbk = std::floor(h[k] / rc);
    g.nb[k] = (int)std::max(1.0, std::min(nbk, 1024.0));
  }
  while ((long long)g.nb[0] * g.nb[1] * g.nb[2] > cap) {
    int k = 0;
    if (g.nb[1] > g.nb[k]) k = 1;
    if (g.nb[2] > g.nb[k]) k = 2;
    g.nb[k] = std::max(1, g.nb[k] / 2);
  }
  for (int k = 0; k < 3; k++)
    g.kk[k] = (int)std::floor(rc * g.nb[k] / h[k]) + 1;
  // multipliers of the device's integer divisions (nb <= 1024, kk <= 127
  // are checked by the callers before any launch)
  auto magic = [](int d) {
    return d > 0 ? (1ULL << 32) / (unsigned long long)d + 1ULL : 0ULL;
  };
  for (int k = 0; k < 3; k++) {
    g.m_nb[k] = magic(g.nb[k]);
    g.wrap_c[k] = g.kk[k] / g.nb[k] + 1;   // wrap_c nb > kk
  }
  g.m_n1 = magic(2 * g.kk[1] + 1);
  g.m_n2 = magic(2 * g.kk[2] + 1);
  // FP32 prefilter bounds.  Every coordinate entering a candidate's FP32
  // difference is at most (2 + sweep) * rowsum in magnitude; the FP32 result
  // is within 5 * 2^-24 of that per component (operand rounding and four
  // rounded operations).  eps takes 16 * 2^-24 of a larger bound, and the
  // distance margin 4 eps + 1e-6 cutoff covers the error of the FP32 length
  // as well: certain-outside and certain-inside classes can never disagree
  // with the FP64 test, and the fill pass checks that they do not.
  double rowsum = 0.0;
  for (int k = 0; k < 3; k++)
    rowsum += std::sqrt(v[k][0] * v[k][0] + v[k][1] * v[k][1] + v[k][2] * v[k][2]);
  const double lam = (2.0 + 3.0 * g.sweep) * rowsum;
  const double eps = 16.0 * 0x1p-24 * lam;
  const double delta = 4.0 * eps + 1e-6 * cutoff;
  for (int k = 0; k < 9; k++) g.cell32[k] = (float)cell[k];
  const float inf = std::numeric_limits<float>::infinity();
  g.d2_out = std::nextafter((float)((cutoff + delta) * (cutoff + delta)), inf);
  g.d2_in = cutoff > delta
                ? std::nextafter((float)((cutoff - delta) * (cutoff - delta)), 0.f)
                : 0.f;
  g.d2_zero = std::nextafter((float)(delta * delta), inf);
  g.atom0 = atom0;
  g.natoms = natoms;
  g.bin0 = bin0;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_nlist_create(fgb_nlist_t *out) {
  if (!out) { set_error("fgb_nlist_create: null output"); return FGB_EINVAL; }
  *out = new fgb_nlist_s();
  return FGB_OK;
}

extern "C" int fgb_nlist_destroy(fgb_nlist_t nl) {
  delete nl;
  return FGB_OK;
}

extern "C" int fgb_nlist_build(fgb_nlist_t nl, int n_struc,
                               const int *h_atom_offsets, const double *h_cells,
                               const double *d_positions, double cutoff,
                               void *stream) {
  return nlist_build(nl, n_struc, h_atom_offsets, h_cells, d_positions,
                     cutoff, (cudaStream_t)stream, true);
}

namespace fgb {

// Slots per atom of a single-pass build: twice the expected neighbour
// count of the densest structure (density x the cutoff sphere) plus 32, in
// multiples of 32, and at least twice the slots of the last build that
// overflowed; 0 (count pass) when that would take more than 2^26 slots.
static long long single_pass_slots(const fgb_nlist_s *nl, double density,
                                   double cutoff, int n_atoms) {
  const double r = cutoff * (1.0 + 1e-9);
  const double expect = density * (4.0 / 3.0) * 3.14159265358979324 * r * r * r;
  const double c = 2.0 * expect + 32.0;
  if (!(c < 65536.0)) return 0;
  long long C = ((long long)std::ceil(c) + 31) / 32 * 32;
  C = std::max(C, nl->min_slots);
  return (long long)n_atoms * C > (1LL << 26) ? 0 : C;
}

int nlist_finish(fgb_nlist_s *nl, const int *hflag) {
  if (hflag[0]) {
    set_error("fgb_nlist_build: non-finite atomic positions");
    return FGB_EINVAL;
  }
  if (nl->total_pending) {
    nl->total_pending = false;
    if (hflag[3]) {   // an atom had more pairs than its slots
      nl->min_slots = 2 * nl->last_slots;
      return kNlistRetry;
    }
    nl->n_pairs = *nl->h_total;
  }
  if (hflag[1] || hflag[2]) {
    set_error("fgb_nlist_build: internal consistency check failed (%d %d)",
              hflag[1], hflag[2]);
    return FGB_ECUDA;
  }
  return FGB_OK;
}

}  // namespace fgb

int fgb::nlist_build(fgb_nlist_s *nl, int n_struc, const int *h_atom_offsets,
                     const double *h_cells, const double *d_positions,
                     double cutoff, cudaStream_t st, bool check) {
  if (!nl || n_struc <= 0 || !h_atom_offsets || !h_cells) {
    set_error("fgb_nlist_build: invalid arguments");
    return FGB_EINVAL;
  }
  if (!(cutoff > 0) || !std::isfinite(cutoff)) {
    set_error("fgb_nlist_build: cutoff must be positive and finite");
    return FGB_EINVAL;
  }
  const int N = h_atom_offsets[n_struc];
  if (h_atom_offsets[0] != 0 || N < 0) {
    set_error("fgb_nlist_build: atom offsets must start at 0");
    return FGB_EINVAL;
  }
  for (int s = 0; s < n_struc; s++)
    if (h_atom_offsets[s + 1] < h_atom_offsets[s]) {
      set_error("fgb_nlist_build: atom offsets must be non-decreasing");
      return FGB_EINVAL;
    }
  if (N > (1 << 24)) {
    set_error("fgb_nlist_build: at most 2^24 atoms per batch");
    return FGB_EINVAL;
  }
  nl->n_struc = n_struc;
  nl->n_atoms = N;
  nl->h_atom_offsets.assign(h_atom_offsets, h_atom_offsets + n_struc + 1);
  nl->h_cells.assign(h_cells, h_cells + 9 * n_struc);
  nl->h_volume.resize(n_struc);
  std::vector<StrucGeom> geom(n_struc);
  std::vector<int> atom_struct(N);
  long long nbins = 0;
  double dmax = 0.0;   // atoms per unit volume, densest structure
  for (int s = 0; s < n_struc; s++) {
    double sweep_cut;
    const double *c = h_cells + 9 * s;
    for (int k = 0; k < 9; k++)
      if (!std::isfinite(c[k])) {
        set_error("fgb_nlist_build: non-finite cell");
        return FGB_EINVAL;
      }
    make_geom(c, cutoff, h_atom_offsets[s],
              h_atom_offsets[s + 1] - h_atom_offsets[s], (int)nbins, geom[s],
              sweep_cut);
    if (!(geom[s].volume > 0) || !std::isfinite(sweep_cut) || sweep_cut <= 0) {
      set_error("fgb_nlist_build: degenerate cell in structure %d", s);
      return FGB_EINVAL;
    }
    if (geom[s].sweep > 127 || geom[s].kk[0] > 127 || geom[s].kk[1] > 127 ||
        geom[s].kk[2] > 127) {
      set_error("fgb_nlist_build: cutoff spans more than 127 cell images");
      return FGB_EINVAL;
    }
    nl->h_volume[s] = geom[s].volume;
    dmax = std::max(dmax, geom[s].natoms / geom[s].volume);
    nbins += (long long)geom[s].nb[0] * geom[s].nb[1] * geom[s].nb[2];
    for (int a = h_atom_offsets[s]; a < h_atom_offsets[s + 1]; a++)
      atom_struct[a] = s;
  }
  if (nbins > (1 << 26)) {
    set_error("fgb_nlist_build: too many bins");
    return FGB_EINVAL;
  }
  int rc;
  if ((rc = nl->geom.ensure(sizeof(StrucGeom) * n_struc)) ||
      (rc = nl->atom_struct.ensure(sizeof(int) * (N + 1))) ||
      (rc = nl->wrapped.ensure(sizeof(double) * 3 * (N + 1))) ||
      (rc = nl->wrapped32.ensure(sizeof(float4) * (N + 1))) ||
      (rc = nl->raw_bin.ensure(sizeof(int) * 3 * (N + 1))) ||
      (rc = nl->home_bin.ensure(sizeof(int) * (N + 1))) ||
      (rc = nl->bin_slot.ensure(sizeof(int) * (N + 1))) ||
      (rc = nl->bin_count.ensure(sizeof(int) * (nbins + 1))) ||
      (rc = nl->bin_start.ensure(sizeof(int) * (nbins + 1))) ||
      (rc = nl->bin_atoms.ensure(sizeof(int) * (N + 1))) ||
      (rc = nl->counts.ensure(sizeof(int) * (N + 1))) ||
      (rc = nl->offsets.ensure(sizeof(long long) * (N + 1))) ||
      (rc = nl->flag.ensure(sizeof(int) * 4)) ||
      (rc = nl->scalars.ensure(sizeof(long long) * 4)))
    return rc;
  FGB_CUDA(cudaMemcpyAsync(nl->geom.p, geom.data(), sizeof(StrucGeom) * n_struc,
                           cudaMemcpyHostToDevice, st));
  if (N > 0)
    FGB_CUDA(cudaMemcpyAsync(nl->atom_struct.p, atom_struct.data(),
                             sizeof(int) * N, cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemsetAsync(nl->bin_count.p, 0, sizeof(int) * (nbins + 1), st));
  FGB_CUDA(cudaMemsetAsync(nl->flag.p, 0, sizeof(int) * 4, st));
  const int T = 128;
  if (N == 0) {
    nl->n_pairs = 0;
    nl->total_pending = false;
    nl->last_launches = 0;
    FGB_CUDA(cudaMemsetAsync(nl->offsets.p, 0, sizeof(long long), st));
    return FGB_OK;
  }
  k_wrap_bin<<<ceil_div(N, T), T, 0, st>>>(
      N, d_positions, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
      nl->wrapped.as<double>(), nl->wrapped32.as<float4>(),
      nl->raw_bin.as<int>(), nl->home_bin.as<int>(),
      nl->bin_slot.as<int>(), nl->bin_count.as<int>(), nl->flag.as<int>());
  FGB_LAUNCH_CHECK("k_wrap_bin");
  if ((rc = scan_int_to_int(nl->bin_count.as<int>(), nl->bin_start.as<int>(),
                            (int)nbins, nl->bin_start.as<int>() + nbins,
                            nl->scan_tmp, st)))
    return rc;
  k_bin_fill<<<ceil_div(N, T), T, 0, st>>>(
      N, nl->home_bin.as<int>(), nl->bin_slot.as<int>(),
      nl->bin_start.as<int>(), nl->bin_atoms.as<int>());
  FGB_LAUNCH_CHECK("k_bin_fill");
  const long long NW = (long long)N * 32;   // warp per atom
  nl->n_bins = nbins;
  // offsets[N] receives the total pair count
  long long *d_total = nl->offsets.as<long long>() + N;
  int hflag[4];
  // Single pass: every atom's pairs go to its own slots [i C, (i + 1) C),
  // C about twice the densest structure's expected neighbour count, so no
  // count pass and no synchronisation are needed; the CSR list is then
  // gathered by the rank sort.  An atom with more than C pairs sets flag[3]
  // and the list is rebuilt with a count pass (below when checking here,
  // by the caller through nlist_finish otherwise), and later builds take
  // at least 2 C slots.
  const long long C = nl->count_pass ? 0 : single_pass_slots(nl, dmax, cutoff, N);
  if (C > 0) {
    const long long slots = (long long)N * C;
    nl->last_slots = C;
    if ((rc = nl->tmp_key.ensure(sizeof(unsigned long long) * (slots + 1))) ||
        (rc = nl->tmp_rel.ensure(sizeof(double4_16a) * (slots + 1))) ||
        (rc = nl->nbr_j.ensure(sizeof(int) * (slots + 1))) ||
        (rc = nl->nbr_shift.ensure(sizeof(int) * (slots + 1))) ||
        (rc = nl->nbr_rel.ensure(sizeof(double4_16a) * (slots + 1))) ||
        (rc = nl->nbr_twin.ensure(sizeof(long long) * (slots + 1))))
      return rc;
    if (!nl->h_total) {
      void *h = nullptr;
      FGB_CUDA(cudaMallocHost(&h, sizeof(long long)));
      nl->h_total = static_cast<long long *>(h);
    }
    k_fill<<<ceil_div(N, kFillWarps), 32 * kFillWarps, 0, st>>>(
        N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
        nl->wrapped.as<double>(), nl->wrapped32.as<float4>(),
        nl->raw_bin.as<int>(), nl->bin_start.as<int>(),
        nl->bin_atoms.as<int>(), cutoff, nl->offsets.as<long long>(), C,
        nl->counts.as<int>(), nl->tmp_key.as<unsigned long long>(),
        nl->tmp_rel.as<double4_16a>(), nl->flag.as<int>());
    FGB_LAUNCH_CHECK("k_fill");
    if ((rc = scan_int_to_ll(nl->counts.as<int>(), nl->offsets.as<long long>(),
                             N, d_total, nl->scan_tmp, st)))
      return rc;
    k_rank_scatter<<<ceil_div(NW, T), T, 0, st>>>(
        N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
        nl->offsets.as<long long>(), C, nl->tmp_key.as<unsigned long long>(),
        nl->tmp_rel.as<double4_16a>(), nl->nbr_j.as<int>(),
        nl->nbr_shift.as<int>(), nl->nbr_rel.as<double4_16a>());
    FGB_LAUNCH_CHECK("k_rank_scatter");
    k_twin<<<ceil_div(NW, T), T, 0, st>>>(
        N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
        nl->offsets.as<long long>(), nl->nbr_j.as<int>(),
        nl->nbr_shift.as<int>(), nl->nbr_twin.as<long long>(),
        nl->flag.as<int>());
    FGB_LAUNCH_CHECK("k_twin");
    FGB_CUDA(cudaMemcpyAsync(nl->h_total, d_total, sizeof(long long),
                             cudaMemcpyDeviceToHost, st));
    nl->n_pairs = slots;   // an upper bound until nlist_finish reads the count
    nl->total_pending = true;
    nl->last_launches = 11;
    if (!check) return FGB_OK;
    FGB_CUDA(cudaMemcpyAsync(hflag, nl->flag.p, sizeof(int) * 4,
                             cudaMemcpyDeviceToHost, st));
    FGB_CUDA(cudaStreamSynchronize(st));
    rc = nlist_finish(nl, hflag);
    if (rc != kNlistRetry) return rc;
    // too many pairs for the slots: the count pass, on the same bins
    FGB_CUDA(cudaMemsetAsync(nl->flag.p, 0, sizeof(int) * 4, st));
  }
  k_count<<<ceil_div(NW, T), T, 0, st>>>(
      N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
      nl->wrapped.as<double>(), nl->wrapped32.as<float4>(),
      nl->raw_bin.as<int>(), nl->bin_start.as<int>(),
      nl->bin_atoms.as<int>(), cutoff, nl->counts.as<int>());
  FGB_LAUNCH_CHECK("k_count");
  if ((rc = scan_int_to_ll(nl->counts.as<int>(), nl->offsets.as<long long>(), N,
                           d_total, nl->scan_tmp, st)))
    return rc;
  long long P = 0;
  FGB_CUDA(cudaMemcpyAsync(&P, d_total, sizeof(long long),
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaMemcpyAsync(hflag, nl->flag.p, sizeof(int) * 4,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (hflag[0]) {
    set_error("fgb_nlist_build: non-finite atomic positions");
    return FGB_EINVAL;
  }
  nl->n_pairs = P;
  nl->total_pending = false;
  // wrap, bin scan (3), bin fill, count, pair scan (3), then fill, rank and
  // twin when there are pairs; after an overflowed single pass its 6 more
  nl->last_launches = 9 + (P > 0 ? 3 : 0) + (C > 0 ? 6 : 0);
  if ((rc = nl->tmp_key.ensure(sizeof(unsigned long long) * (P + 1))) ||
      (rc = nl->tmp_rel.ensure(sizeof(double4_16a) * (P + 1))) ||
      (rc = nl->nbr_j.ensure(sizeof(int) * (P + 1))) ||
      (rc = nl->nbr_shift.ensure(sizeof(int) * (P + 1))) ||
      (rc = nl->nbr_rel.ensure(sizeof(double4_16a) * (P + 1))) ||
      (rc = nl->nbr_twin.ensure(sizeof(long long) * (P + 1))))
    return rc;
  if (P > 0) {
    k_fill<<<ceil_div(N, kFillWarps), 32 * kFillWarps, 0, st>>>(
        N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
        nl->wrapped.as<double>(), nl->wrapped32.as<float4>(),
        nl->raw_bin.as<int>(),
        nl->bin_start.as<int>(), nl->bin_atoms.as<int>(), cutoff,
        nl->offsets.as<long long>(), 0LL, nullptr,
        nl->tmp_key.as<unsigned long long>(), nl->tmp_rel.as<double4_16a>(),
        nl->flag.as<int>());
    FGB_LAUNCH_CHECK("k_fill");
    k_rank_scatter<<<ceil_div((long long)N * 32, T), T, 0, st>>>(
        N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
        nl->offsets.as<long long>(), 0LL, nl->tmp_key.as<unsigned long long>(),
        nl->tmp_rel.as<double4_16a>(), nl->nbr_j.as<int>(), nl->nbr_shift.as<int>(),
        nl->nbr_rel.as<double4_16a>());
    FGB_LAUNCH_CHECK("k_rank_scatter");
    k_twin<<<ceil_div(NW, T), T, 0, st>>>(
        N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
        nl->offsets.as<long long>(), nl->nbr_j.as<int>(),
        nl->nbr_shift.as<int>(), nl->nbr_twin.as<long long>(),
        nl->flag.as<int>());
    FGB_LAUNCH_CHECK("k_twin");
  }
  if (!check) return FGB_OK;   // the caller reads flag[1], flag[2] later
  FGB_CUDA(cudaMemcpyAsync(hflag, nl->flag.p, sizeof(int) * 4,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  return nlist_finish(nl, hflag);
}

namespace fgb {

int nlist_reserve(fgb_nlist_s *nl, long long cap) {
  int rc;
  if ((rc = nl->tmp_key.ensure(sizeof(unsigned long long) * (cap + 1))) ||
      (rc = nl->tmp_rel.ensure(sizeof(double4_16a) * (cap + 1))) ||
      (rc = nl->nbr_j.ensure(sizeof(int) * (cap + 1))) ||
      (rc = nl->nbr_shift.ensure(sizeof(int) * (cap + 1))) ||
      (rc = nl->nbr_rel.ensure(sizeof(double4_16a) * (cap + 1))) ||
      (rc = nl->nbr_twin.ensure(sizeof(long long) * (cap + 1))))
    return rc;
  return FGB_OK;
}

int nlist_rebuild_fixed(fgb_nlist_s *nl, const double *d_positions,
                        double cutoff, long long cap, cudaStream_t st) {
  const int N = nl->n_atoms;
  const long long nbins = nl->n_bins;
  const int T = 128;
  int rc;
  FGB_CUDA(cudaMemsetAsync(nl->bin_count.p, 0, sizeof(int) * (nbins + 1), st));
  FGB_CUDA(cudaMemsetAsync(nl->flag.p, 0, sizeof(int) * 4, st));
  nl->last_launches = 0;
  if (N == 0) return FGB_OK;
  k_wrap_bin<<<ceil_div(N, T), T, 0, st>>>(
      N, d_positions, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
      nl->wrapped.as<double>(), nl->wrapped32.as<float4>(),
      nl->raw_bin.as<int>(), nl->home_bin.as<int>(), nl->bin_slot.as<int>(),
      nl->bin_count.as<int>(), nl->flag.as<int>());
  FGB_LAUNCH_CHECK("k_wrap_bin");
  if ((rc = scan_int_to_int(nl->bin_count.as<int>(), nl->bin_start.as<int>(),
                            (int)nbins, nl->bin_start.as<int>() + nbins,
                            nl->scan_tmp, st)))
    return rc;
  k_bin_fill<<<ceil_div(N, T), T, 0, st>>>(
      N, nl->home_bin.as<int>(), nl->bin_slot.as<int>(),
      nl->bin_start.as<int>(), nl->bin_atoms.as<int>());
  FGB_LAUNCH_CHECK("k_bin_fill");
  const long long NW = (long long)N * 32;
  k_count<<<ceil_div(NW, T), T, 0, st>>>(
      N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
      nl->wrapped.as<double>(), nl->wrapped32.as<float4>(),
      nl->raw_bin.as<int>(), nl->bin_start.as<int>(), nl->bin_atoms.as<int>(),
      cutoff, nl->counts.as<int>());
  FGB_LAUNCH_CHECK("k_count");
  if ((rc = scan_int_to_ll(nl->counts.as<int>(), nl->offsets.as<long long>(),
                           N, nl->offsets.as<long long>() + N, nl->scan_tmp,
                           st)))
    return rc;
  k_clamp_offsets<<<ceil_div(N + 1, T), T, 0, st>>>(
      N, cap, nl->offsets.as<long long>(), nl->flag.as<int>());
  FGB_LAUNCH_CHECK("k_clamp_offsets");
  k_fill<<<ceil_div(N, kFillWarps), 32 * kFillWarps, 0, st>>>(
      N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
      nl->wrapped.as<double>(), nl->wrapped32.as<float4>(),
      nl->raw_bin.as<int>(), nl->bin_start.as<int>(), nl->bin_atoms.as<int>(),
      cutoff, nl->offsets.as<long long>(), 0LL, nullptr,
      nl->tmp_key.as<unsigned long long>(), nl->tmp_rel.as<double4_16a>(),
      nl->flag.as<int>());
  FGB_LAUNCH_CHECK("k_fill");
  k_rank_scatter<<<ceil_div(NW, T), T, 0, st>>>(
      N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
      nl->offsets.as<long long>(), 0LL, nl->tmp_key.as<unsigned long long>(),
      nl->tmp_rel.as<double4_16a>(), nl->nbr_j.as<int>(),
      nl->nbr_shift.as<int>(), nl->nbr_rel.as<double4_16a>());
  FGB_LAUNCH_CHECK("k_rank_scatter");
  k_twin<<<ceil_div(NW, T), T, 0, st>>>(
      N, nl->atom_struct.as<int>(), nl->geom.as<StrucGeom>(),
      nl->offsets.as<long long>(), nl->nbr_j.as<int>(),
      nl->nbr_shift.as<int>(), nl->nbr_twin.as<long long>(),
      nl->flag.as<int>());
  FGB_LAUNCH_CHECK("k_twin");
  nl->n_pairs = cap;   // an upper bound; the device offsets hold the count
  nl->last_launches = 13;
  return FGB_OK;
}

}  // namespace fgb

extern "C" int fgb_nlist_size(fgb_nlist_t nl, long long *n_pairs,
                              int *n_atoms) {
  if (!nl) { set_error("fgb_nlist_size: null handle"); return FGB_EINVAL; }
  if (n_pairs) *n_pairs = nl->n_pairs;
  if (n_atoms) *n_atoms = nl->n_atoms;
  return FGB_OK;
}

extern "C" int fgb_nlist_export(fgb_nlist_t nl, int *d_neighbor_count,
                                int *d_structure_indices, int *d_shifts,
                                double *d_relative_positions,
                                double *d_wrapped, void *stream) {
  if (!nl) { set_error("fgb_nlist_export: null handle"); return FGB_EINVAL; }
  cudaStream_t st = (cudaStream_t)stream;
  int N = nl->n_atoms;
  if (N == 0) return FGB_OK;
  k_export<<<ceil_div(N, 128), 128, 0, st>>>(
      N, nl->offsets.as<long long>(), nl->atom_struct.as<int>(),
      nl->geom.as<StrucGeom>(), nl->nbr_j.as<int>(), nl->nbr_shift.as<int>(),
      nl->nbr_rel.as<double4_16a>(), d_neighbor_count, d_structure_indices,
      d_shifts, d_relative_positions);
  FGB_LAUNCH_CHECK("k_export");
  if (d_wrapped)
    FGB_CUDA(cudaMemcpyAsync(d_wrapped, nl->wrapped.p, sizeof(double) * 3 * N,
                             cudaMemcpyDeviceToDevice, st));
  return FGB_OK;
}

// ------------------------------------------------- no-allocation variant
// fgb_nlist_build_noalloc builds one structure's neighbour list without any
// device allocation: its working memory is the file-scope array below, and
// the list is written straight into buffers the caller owns.  It exists for
// callers that cannot call cudaMalloc themselves or have us call it — for
// instance an MD engine or plugin that manages a fixed device-memory budget
// of its own, or a loop that must not pay allocation latency or fragment
// the heap between steps.
//
// The array's name, used in host code, is only a host-side stand-in for the
// symbol; the kernels need its device address, which every call looks up
// with cudaGetSymbolAddress for the device current at the call (an address
// belongs to one context, so none is cached across calls: a context made
// again after cudaDeviceReset gets a fresh one).  The first lookup on a
// device loads the library's module into that context, so the first call
// on each device should come before any stream capture.  Every call on a device shares the one array and
// leaves its contents behind; each call clears what must start at zero (bin
// counts, error flags, the structure index of each atom), so calls that run
// one after another are independent, but calls that overlap on the GPU (for
// example on two streams at once) race on the same memory.
namespace fgb {
namespace {

constexpr size_t kNoAllocScratchBytes = FGB_NOALLOC_SCRATCH_BYTES;  // 24 MiB
static __device__ __align__(256) unsigned char g_nlist_scratch[kNoAllocScratchBytes];

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Device address of g_nlist_scratch in the current device's context.
int noalloc_scratch(unsigned char **out) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_nlist_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress");
  *out = static_cast<unsigned char *>(p);
  return FGB_OK;
}

}  // namespace
}  // namespace fgb

extern "C" int fgb_nlist_build_noalloc(const double *h_cell,
                                       const double *d_positions, int n_atoms,
                                       double cutoff, long long max_pairs,
                                       int *d_neighbor_count,
                                       int *d_structure_indices, int *d_shifts,
                                       double *d_relative_positions,
                                       long long *h_n_pairs, void *stream) {
  using namespace fgb;
  if (!h_cell || !d_positions || !d_neighbor_count || !d_structure_indices ||
      !d_relative_positions || !h_n_pairs || n_atoms < 0 || max_pairs < 0) {
    set_error("fgb_nlist_build_noalloc: invalid arguments");
    return FGB_EINVAL;
  }
  if (n_atoms > FGB_NOALLOC_MAX_ATOMS) {
    set_error("fgb_nlist_build_noalloc: %d atoms exceed the no-allocation "
              "limit of %d atoms", n_atoms, FGB_NOALLOC_MAX_ATOMS);
    return FGB_EINVAL;
  }
  if (!(cutoff > 0) || !std::isfinite(cutoff)) {
    set_error("fgb_nlist_build_noalloc: cutoff must be positive and finite");
    return FGB_EINVAL;
  }
  if (reinterpret_cast<uintptr_t>(d_relative_positions) % 16 != 0) {
    set_error("fgb_nlist_build_noalloc: relative_positions must be 16-byte "
              "aligned");
    return FGB_EINVAL;
  }
  for (int k = 0; k < 9; k++)
    if (!std::isfinite(h_cell[k])) {
      set_error("fgb_nlist_build_noalloc: non-finite cell");
      return FGB_EINVAL;
    }
  *h_n_pairs = 0;
  cudaStream_t st = (cudaStream_t)stream;
  const int N = n_atoms;
  StrucGeom geom;
  double sweep_cut;
  make_geom(h_cell, cutoff, 0, N, 0, geom, sweep_cut);
  if (!(geom.volume > 0) || !std::isfinite(sweep_cut) || sweep_cut <= 0) {
    set_error("fgb_nlist_build_noalloc: degenerate cell");
    return FGB_EINVAL;
  }
  if (geom.sweep > 127 || geom.kk[0] > 127 || geom.kk[1] > 127 ||
      geom.kk[2] > 127) {
    set_error("fgb_nlist_build_noalloc: cutoff spans more than 127 cell "
              "images");
    return FGB_EINVAL;
  }
  const long long nbins = (long long)geom.nb[0] * geom.nb[1] * geom.nb[2];
  // two int arrays of nbins + 1 entries must fit the scratch; bounding the
  // bin count first also keeps every size below in range
  if (nbins < 1 ||
      nbins > (long long)(kNoAllocScratchBytes / (2 * sizeof(int)))) {
    set_error("fgb_nlist_build_noalloc: %lld cell-list bins exceed the "
              "%zu-byte no-allocation scratch", nbins, kNoAllocScratchBytes);
    return FGB_EINVAL;
  }
  unsigned char *base = nullptr;
  int rc;
  if ((rc = noalloc_scratch(&base))) return rc;
  // carve the scratch (every piece 256-byte aligned)
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char *p = base + off;
    off += align256(bytes);
    return p;
  };
  const int nsum = (int)(std::max<long long>(N, nbins) / 1024 + 2);
  StrucGeom *d_geom = (StrucGeom *)take(sizeof(StrucGeom));
  int *atom_struct = (int *)take(sizeof(int) * (N + 1));
  double *wrapped = (double *)take(sizeof(double) * 3 * (N + 1));
  float4 *w32 = (float4 *)take(sizeof(float4) * (N + 1));
  int *raw = (int *)take(sizeof(int) * 3 * (N + 1));
  int *home = (int *)take(sizeof(int) * (N + 1));
  int *slot = (int *)take(sizeof(int) * (N + 1));
  int *bin_count = (int *)take(sizeof(int) * (nbins + 1));
  int *bin_start = (int *)take(sizeof(int) * (nbins + 1));
  int *bin_atoms = (int *)take(sizeof(int) * (N + 1));
  long long *offsets = (long long *)take(sizeof(long long) * (N + 1));
  long long *sums = (long long *)take(sizeof(long long) * nsum);
  int *flag = (int *)take(sizeof(int) * 4);
  const size_t fixed = off;
  if (fixed > kNoAllocScratchBytes) {
    set_error("fgb_nlist_build_noalloc: structure needs more than the "
              "%zu-byte no-allocation scratch", kNoAllocScratchBytes);
    return FGB_EINVAL;
  }
  FGB_CUDA(cudaMemcpyAsync(d_geom, &geom, sizeof(StrucGeom),
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemsetAsync(atom_struct, 0, sizeof(int) * (N + 1), st));
  FGB_CUDA(cudaMemsetAsync(bin_count, 0, sizeof(int) * (nbins + 1), st));
  FGB_CUDA(cudaMemsetAsync(flag, 0, sizeof(int) * 4, st));
  if (N == 0) {
    FGB_CUDA(cudaStreamSynchronize(st));
    return FGB_OK;
  }
  const int T = 128;
  k_wrap_bin<<<ceil_div(N, T), T, 0, st>>>(N, d_positions, atom_struct, d_geom,
                                           wrapped, w32, raw, home, slot,
                                           bin_count, flag);
  FGB_LAUNCH_CHECK("k_wrap_bin");
  if ((rc = scan_int_to_int_raw(bin_count, bin_start, (int)nbins,
                                bin_start + nbins, (int *)sums, st)))
    return rc;
  k_bin_fill<<<ceil_div(N, T), T, 0, st>>>(N, home, slot, bin_start, bin_atoms);
  FGB_LAUNCH_CHECK("k_bin_fill");
  const long long NW = (long long)N * 32;   // warp per atom
  k_count<<<ceil_div(NW, T), T, 0, st>>>(N, atom_struct, d_geom, wrapped, w32,
                                         raw, bin_start, bin_atoms, cutoff,
                                         d_neighbor_count);
  FGB_LAUNCH_CHECK("k_count");
  if ((rc = scan_int_to_ll_raw(d_neighbor_count, offsets, N, offsets + N, sums,
                               st)))
    return rc;
  long long P = 0;
  int hflag[4] = {0, 0, 0, 0};
  FGB_CUDA(cudaMemcpyAsync(&P, offsets + N, sizeof(long long),
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaMemcpyAsync(hflag, flag, sizeof(int) * 4,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (hflag[0]) {
    set_error("fgb_nlist_build_noalloc: non-finite atomic positions");
    return FGB_EINVAL;
  }
  *h_n_pairs = P;
  const size_t per_pair = align256(sizeof(unsigned long long) * (P + 1)) +
                          align256(sizeof(double4_16a) * (P + 1)) +
                          align256(sizeof(int) * (P + 1)) * 2 +
                          align256(sizeof(double4_16a) * (P + 1));
  if (P > FGB_NOALLOC_MAX_PAIRS || fixed + per_pair > kNoAllocScratchBytes) {
    set_error("fgb_nlist_build_noalloc: %lld pairs exceed the no-allocation "
              "limit of %d pairs", P, FGB_NOALLOC_MAX_PAIRS);
    return FGB_EINVAL;
  }
  if (P > max_pairs) {
    set_error("fgb_nlist_build_noalloc: %lld pairs do not fit the output "
              "capacity of %lld (needed size returned in n_pairs)", P,
              max_pairs);
    return FGB_EINVAL;
  }
  if (P == 0) return FGB_OK;
  unsigned long long *key = (unsigned long long *)take(sizeof(unsigned long long) * (P + 1));
  double4_16a *tmp_rel = (double4_16a *)take(sizeof(double4_16a) * (P + 1));
  int *nbr_j = (int *)take(sizeof(int) * (P + 1));
  int *nbr_shift = (int *)take(sizeof(int) * (P + 1));
  double4_16a *nbr_rel = (double4_16a *)take(sizeof(double4_16a) * (P + 1));
  k_fill<<<ceil_div(N, kFillWarps), 32 * kFillWarps, 0, st>>>(N, atom_struct, d_geom, wrapped, w32,
                                        raw, bin_start, bin_atoms, cutoff,
                                        offsets, 0LL, nullptr, key, tmp_rel,
                                        flag);
  FGB_LAUNCH_CHECK("k_fill");
  k_rank_scatter<<<ceil_div((long long)N * 32, T), T, 0, st>>>(
      N, atom_struct, d_geom, offsets, 0LL, key, tmp_rel, nbr_j, nbr_shift,
      nbr_rel);
  FGB_LAUNCH_CHECK("k_rank_scatter");
  k_export<<<ceil_div(N, T), T, 0, st>>>(N, offsets, atom_struct, d_geom, nbr_j,
                                         nbr_shift, nbr_rel, d_neighbor_count,
                                         d_structure_indices, d_shifts,
                                         d_relative_positions);
  FGB_LAUNCH_CHECK("k_export");
  FGB_CUDA(cudaMemcpyAsync(hflag, flag, sizeof(int) * 4,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (hflag[1]) {
    set_error("fgb_nlist_build_noalloc: internal consistency check failed");
    return FGB_ECUDA;
  }
  return FGB_OK;
}
