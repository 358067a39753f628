// K2 / K5: B2 descriptor forward and its reverse-mode adjoint.
//
// Forward (b2.cpp:244-399 single bond, :181-242 contraction), one CTA per
// atom: the atom's neighbour list is streamed in chunks of kChunk pairs; each
// thread evaluates one pair's radial x cutoff values g_n and real Y_lm into
// shared memory, then the CTA contracts them into A[s_j][n][lm] (thread per
// A entry, fixed pair order: deterministic, no atomics).  B2 is then
// sum_m A[n1][lm] A[n2][lm] for n1 <= n2, in the reference's counter order,
// written with coalesced stores, and the norm is a fixed-order block sum.
//
// Adjoint: dE/dB2 -> u = dE/dA (u[c][lm] = sum_b w((c,b),l) A[b][lm] (1+d_cb))
// -> per pair dE/dr_ij = sum_{n,lm} u[s_j][n][lm] d(g_n Y_lm)/dr_ij, with g
// and Y recomputed instead of stored.  Forces and the virial are assembled by
// owner-computes over each atom's pairs and their twins (no float atomics).
#include <type_traits>

#include "fgb_df.cuh"
#include "fgb_internal.h"
#include "fgb_kernels.h"

namespace fgb {

namespace {

constexpr int kChunk = 64;      // pairs per shared-memory chunk = block size

__device__ __forceinline__ void decode_b2(int q, int L1, int nr, int &n1,
                                          int &n2, int &l) {
  l = q % L1;
  int pidx = q / L1;
  n1 = 0;
  while (pidx >= nr - n1) { pidx -= nr - n1; n1++; }
  n2 = n1 + pidx;
}

__device__ __forceinline__ double shfl_down(double v, int o) {
  return __shfl_down_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ df shfl_down(df v, int o) {
  return df(__shfl_down_sync(0xffffffffu, v.hi, o),
            __shfl_down_sync(0xffffffffu, v.lo, o));
}

// acc += a b.  FP64: one fused multiply-add.  Double-float: the exact
// product's high part enters a TwoSum with acc.hi and every low-order term
// collects in acc.lo, renormalised once by the caller (finish).
__device__ __forceinline__ void mac(double &acc, double a, double b) {
  acc += a * b;
}
__device__ __forceinline__ void mac(df &acc, df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float pe = __fmaf_rn(a.hi, b.hi, -p);
  pe = __fmaf_rn(a.hi, b.lo, pe);
  pe = __fmaf_rn(a.lo, b.hi, pe);
  float s, se;
  two_sum(acc.hi, p, s, se);
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(se, pe));
}
__device__ __forceinline__ double finish(double a) { return a; }
__device__ __forceinline__ df finish(df a) {
  df r;
  fast_two_sum(a.hi, a.lo, r.hi, r.lo);
  return r;
}

// Shared memory: A[nA] | g[kChunk*nmax] | Y[kChunk*nh] | sp[kChunk] | red,
// in the compute type T: double (FP64 path) or df (double-float, the
// mixed-precision path; the pair geometry arrives in FP64 and is split).
template <typename T, int NC, int LC>
__global__ void __launch_bounds__(kChunk, 12)
k_b2_forward(B2Params p, int n_atoms, const long long *__restrict__ offsets,
             const int *__restrict__ nbr_j, const double4_16a *__restrict__ rel,
             const int *__restrict__ species, double *__restrict__ A_out,
             double *__restrict__ B2, double *__restrict__ norms,
             double *__restrict__ rowmax, float *__restrict__ A_out32) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // largest |B2| of the row as written (the bits of |x| order as the
  // values do), for the tensor-core row scales: no second pass over B2
  __shared__ unsigned long long s_max[kChunk / 32];
  unsigned long long lmax = 0;
  const auto track = [&lmax](double x) {
    const unsigned long long a =
        (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFULL;
    lmax = a > lmax ? a : lmax;
  };
  const int i = blockIdx.x;
  if (i >= n_atoms) return;
  // NC / LC > 0: n_max / l_max fixed at compile time
  const int nh = LC > 0 ? (LC + 1) * (LC + 1) : p.n_harm;
  const int nm = NC > 0 ? NC : p.n_max;
  const int nA = p.n_species * nm * nh;
  constexpr bool kFixed = NC > 0 && LC > 0;
  // fixed sizes with at most one (species, lm) per thread: A stays in
  // registers over the pair chunks and is laid over the end of the Y
  // buffer for the contraction (b2_forward_smem leaves A out)
  const bool regA = kFixed && p.n_species * nh <= kChunk &&
                    p.n_species * nm <= kChunk;
  T *A = reinterpret_cast<T *>(smem_raw);
  T *sg = regA ? A : A + nA;
  T *sy = sg + kChunk * nm;
  int *ssp = (int *)(sy + kChunk * nh);
  T *red = (T *)(ssp + kChunk);
  int *sord = (int *)(red + kChunk);      // chunk pairs, sorted by species
  int *scnt = sord + kChunk;              // [warp][species] counts
  int *sbeg = scnt + 2 * kMaxSpecies;     // species starts in sord
  const int t = threadIdx.x;
  // a species outside [0, n_species) contributes nothing here (the caller
  // rejects it before any later stage): no table or shared-memory index is
  // formed from it
  const int ns = p.n_species;
  const int si_raw = species[i];
  const bool si_ok = si_raw >= 0 && si_raw < ns;
  const int si = si_ok ? si_raw : 0;
  T areg[NC > 0 ? NC : 1];
#pragma unroll
  for (int n = 0; n < (NC > 0 ? NC : 1); n++) areg[n] = T(0);
  if (!regA)
    for (int e = t; e < nA; e += blockDim.x) A[e] = T(0);
  const long long b = offsets[i], e_ = offsets[i + 1];
  for (long long c0 = b; c0 < e_; c0 += kChunk) {
    long long pp = c0 + t;
    int sj = -1;
    if (pp < e_) {
      int j = nbr_j[pp];
      double4_16a r = rel[pp];
      sj = species[j];
      const bool ok = si_ok && sj >= 0 && sj < ns;
      double rc = ok ? p.cutoffs[si * kMaxSpecies + sj] : 0.0;
      if (ok && r.x <= rc) {
        radial_eval<T, NC>(p, T(r.x), T(rc), sg + t * nm, (T *)nullptr);
        ylm_eval<T, LC>(p.l_max, T(r.y), T(r.z), T(r.w), sy + t * nh, nullptr);
      } else {
        sj = -1;
      }
    }
    ssp[t] = sj;
    __syncthreads();
    if constexpr (kFixed) {
      // The chunk's pairs grouped by neighbour species (pair order kept in
      // each group): a thread per (species, lm) then sums only its species'
      // pairs, with the n_max accumulators in registers and each Y value
      // loaded once.  The sums run over the same pairs in the same order as
      // entry-by-entry accumulation, so A is the same to the bit.
      constexpr int NH = (LC + 1) * (LC + 1);
      const int S = p.n_species, warp = t >> 5, lane = t & 31;
      int rank = 0;
      for (int s = 0; s < S; s++) {
        const unsigned b = __ballot_sync(0xffffffffu, sj == s);
        if (lane == 0) scnt[warp * kMaxSpecies + s] = __popc(b);
        if (sj == s) rank = __popc(b & ((1u << lane) - 1u));
      }
      __syncthreads();
      if (t == 0) {
        int acc = 0;
        for (int s = 0; s < S; s++) {
          sbeg[s] = acc;
          acc += scnt[s] + scnt[kMaxSpecies + s];
        }
        sbeg[S] = acc;
      }
      __syncthreads();
      if (sj >= 0)
        sord[sbeg[sj] + (warp ? scnt[sj] : 0) + rank] = t;
      __syncthreads();
      for (int it = t; it < S * NH; it += blockDim.x) {
        const int s = it / NH, lm = it % NH;
        T acc[NC];
#pragma unroll
        for (int n = 0; n < NC; n++) acc[n] = T(0);
        for (int q = sbeg[s]; q < sbeg[s + 1]; q++) {
          const int pq = sord[q];
          const T y = sy[pq * NH + lm];
#pragma unroll
          for (int n = 0; n < NC; n++) mac(acc[n], sg[pq * NC + n], y);
        }
        if (regA) {
#pragma unroll
          for (int n = 0; n < NC; n++) areg[n] += finish(acc[n]);
        } else {
#pragma unroll
          for (int n = 0; n < NC; n++) A[(s * NC + n) * NH + lm] += finish(acc[n]);
        }
      }
    } else {
      const int cnt = (int)min((long long)kChunk, e_ - c0);
      for (int e = t; e < nA; e += blockDim.x) {
        int s = e / (nm * nh);
        int n = (e / nh) % nm;
        int lm = e % nh;
        T acc = T(0);
        for (int q = 0; q < cnt; q++)
          if (ssp[q] == s) mac(acc, sg[q * nm + n], sy[q * nh + lm]);
        A[e] += finish(acc);
      }
    }
    __syncthreads();
  }
  if (regA) {
    // the Y buffer is free after the last chunk (synchronised above); A
    // takes its end, clear of the B2 row staged from the start of g
    A = sy + (kChunk * nh - nA);
    if constexpr (kFixed) {
      constexpr int NH = (LC + 1) * (LC + 1);
      if (t < p.n_species * NH) {
        const int s = t / NH, lm = t % NH;
#pragma unroll
        for (int n = 0; n < NC; n++) A[(s * NC + n) * NH + lm] = areg[n];
      }
    }
    __syncthreads();
  }
  if (A_out)
    for (int e = t; e < nA; e += blockDim.x)
      A_out[(long long)i * nA + e] = to_double(A[e]);
  if (A_out32)   // the FP32 adjoint's input: the nearest float, no FP64
    for (int e = t; e < nA; e += blockDim.x)
      A_out32[(long long)i * nA + e] = to_float(A[e]);
  const int L1 = (LC > 0 ? LC : p.l_max) + 1, nr = p.n_species * nm,
            nd = p.n_d;
  T nrm = T(0);
  if constexpr (kFixed) {
    // A thread per radial pair (n1 <= n2) computes its L+1 values (no index
    // decoding per value); the row is staged in the basis-value buffers and
    // written with coalesced stores when it fits there.
    constexpr int L1c = LC + 1, NH = (LC + 1) * (LC + 1);
    const bool stage = nd <= kChunk * (nm + nh) - (regA ? nA : 0);
    T *out_s = sg;
    const int npair = nr * (nr + 1) / 2;
    for (int pi = t; pi < npair; pi += blockDim.x) {
      int n1 = 0, rem = pi;
      while (rem >= nr - n1) { rem -= nr - n1; n1++; }
      const T *a1 = A + n1 * NH, *a2 = A + (n1 + rem) * NH;
#pragma unroll
      for (int l = 0; l < L1c; l++) {
        T v = T(0);
#pragma unroll
        for (int m = 0; m < 2 * l + 1; m++) mac(v, a1[l * l + m], a2[l * l + m]);
        v = finish(v);
        if (stage) out_s[pi * L1c + l] = v;
        else {
          const double x = to_double(v);
          B2[(long long)i * nd + pi * L1c + l] = x;
          track(x);
        }
        mac(nrm, v, v);
      }
    }
    if (stage) {
      __syncthreads();
      for (int q = t; q < nd; q += blockDim.x)
      {
        const double x = to_double(out_s[q]);
        B2[(long long)i * nd + q] = x;
        track(x);
      }
    }
  } else {
    for (int q = t; q < nd; q += blockDim.x) {
      int n1, n2, l;
      decode_b2(q, L1, nr, n1, n2, l);
      const T *a1 = A + n1 * nh + l * l, *a2 = A + n2 * nh + l * l;
      T v = T(0);
      for (int m = 0; m < 2 * l + 1; m++) mac(v, a1[m], a2[m]);
      v = finish(v);
      const double x = to_double(v);
      B2[(long long)i * nd + q] = x;
      track(x);
      mac(nrm, v, v);
    }
  }
  // norm and row maximum: shuffles down each warp (fixed order), then
  // thread 0 adds the warps' partials in warp order -- one barrier
  nrm = finish(nrm);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nrm = nrm + shfl_down(nrm, o);
    const unsigned long long m =
        (unsigned long long)__shfl_down_sync(0xffffffffu, (long long)lmax, o);
    lmax = m > lmax ? m : lmax;
  }
  if ((t & 31) == 0) {
    red[t >> 5] = nrm;
    s_max[t >> 5] = lmax;
  }
  __syncthreads();
  if (t == 0) {
    for (int w = 1; w < kChunk / 32; w++) {
      nrm = nrm + red[w];
      lmax = s_max[w] > lmax ? s_max[w] : lmax;
    }
    norms[i] = to_double(sqrt(nrm));
    if (rowmax) rowmax[i] = __longlong_as_double((long long)lmax);
  }
}

// Shared memory: u[nA] | A[nA] (compute type T: double, or float in the
// mixed-precision path)
// FP64 inputs in the compute type: FP32 takes the mantissa cut on the bit
// pattern (integer instructions; an FP64 -> FP32 conversion runs on the FP64
// pipe, which is scarce on this GPU).
__device__ __forceinline__ double as_compute(double x, double) { return x; }
__device__ __forceinline__ float as_compute(double x, float) {
  return trunc_float(x);
}
// Pair gradients in the adjoint's compute type: the FP32 adjoint writes
// float3 (half the bytes, and the force sums then run in FP32).
template <typename T> struct PairGrad { using type = double3; };
template <> struct PairGrad<float> { using type = float3; };
__device__ __forceinline__ double3 pair_out(double x, double y, double z) {
  return make_double3(x, y, z);
}
__device__ __forceinline__ float3 pair_out(float x, float y, float z) {
  return make_float3(x, y, z);
}

// Atoms per block of the adjoint and its block size: ~42 pairs per atom,
// so three atoms' pairs fill the 128 threads of the pair loop.
// The 2l + 1 entries u[c][l^2 .. l^2 + 2l] (M = 2l + 1 at compile time),
// each summed over b in the order of the thread-per-entry form.
template <typename T, int M>
__device__ __forceinline__ void u_entries(const T *A, const T *wsrc, int nh,
                                          int nr, int L1, int c, int l, T *u,
                                          int nm, int cs, int cn) {
  const T *wl = wsrc + l;
  const T *Al = A + l * l;
  T acc[M];
#pragma unroll
  for (int m = 0; m < M; m++) acc[m] = T(0);
  int pidx = c;   // radial pair (0, c)
  for (int bb = 0; bb < c; bb++) {
    const T w = wl[pidx * L1];
#pragma unroll
    for (int m = 0; m < M; m++) acc[m] += w * Al[bb * nh + m];
    pidx += nr - bb - 1;
  }
  {   // pidx is now the pair (c, c)
    const T w = T(2) * wl[pidx * L1];
#pragma unroll
    for (int m = 0; m < M; m++) acc[m] += w * Al[c * nh + m];
  }
  for (int bb = c + 1; bb < nr; bb++) {
    pidx++;
    const T w = wl[pidx * L1];
#pragma unroll
    for (int m = 0; m < M; m++) acc[m] += w * Al[bb * nh + m];
  }
#pragma unroll
  for (int m = 0; m < M; m++) u[(cs * nh + l * l + m) * nm + cn] = acc[m];
}

// The same for any l (run-time entry count).
template <typename T>
__device__ void u_entries_any(const T *A, const T *wsrc, int nh, int nr,
                              int L1, int c, int l, T *u, int nm, int cs,
                              int cn) {
  const T *wl = wsrc + l;
  for (int m = 0; m < 2 * l + 1; m++) {
    const T *Acol = A + l * l + m;
    T acc = T(0);
    int pidx = c;
    for (int bb = 0; bb < c; bb++) {
      acc += wl[pidx * L1] * Acol[bb * nh];
      pidx += nr - bb - 1;
    }
    acc += T(2) * wl[pidx * L1] * Acol[c * nh];
    for (int bb = c + 1; bb < nr; bb++) {
      pidx++;
      acc += wl[pidx * L1] * Acol[bb * nh];
    }
    u[(cs * nh + l * l + m) * nm + cn] = acc;
  }
}

constexpr int kAdjAtoms = 3;
// Shared-memory values per atom of the adjoint: u and A (n_A each) and
// optionally the dE/dB2 row, rounded up to whole groups of 4.
__host__ __device__ constexpr int adj_atom_values(int nA, int nd_in_smem) {
  return (2 * nA + nd_in_smem + 3) / 4 * 4;
}
constexpr int kAdjThreads = 128;

// Shared memory, per atom of the block: u[nA] | A[nA] | w[nd] (the atom's
// dE/dB2 row, when it fits).  The pair loop is latency-bound (per-pair
// loads, recurrence chains): the FP32 kernel is held to 48 registers for
// 10 blocks (40 warps) per SM.  On the alloy workload that measured 0.212
// ms per 32k atoms, against 0.244 ms at 8 blocks (64 registers) and 0.232
// ms at 12 (40 registers, more spilled values).
template <typename T, int NC, int LC>
__global__ void __launch_bounds__(kAdjThreads, sizeof(T) == 4 ? 10 : 2)
k_b2_adjoint(B2Params p, int n_atoms, const long long *__restrict__ offsets,
             const int *__restrict__ nbr_j, const double4_16a *__restrict__ rel,
             const int *__restrict__ species, const double *__restrict__ A_in,
             const float *__restrict__ A_in32, const T *__restrict__ gB2,
             typename PairGrad<T>::type *__restrict__ pair_grad,
             int w_in_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *smem = reinterpret_cast<T *>(smem_raw);
  const int i0 = blockIdx.x * kAdjAtoms;
  if (i0 >= n_atoms) return;
  const int na = min(kAdjAtoms, n_atoms - i0);
  constexpr int NA = NC > 0 ? NC : kMaxNmax;
  const int nh = LC > 0 ? (LC + 1) * (LC + 1) : p.n_harm;
  const int nm = NC > 0 ? NC : p.n_max;
  const int nA = p.n_species * nm * nh, nr = p.n_species * nm,
            L1 = (LC > 0 ? LC : p.l_max) + 1, nd = p.n_d;
  // T values per atom, in whole 4-value groups (16-byte aligned u rows)
  const int per = adj_atom_values(nA, w_in_smem ? nd : 0);
  const int t = threadIdx.x;
  for (int a = 0; a < na; a++) {
    T *A = smem + (size_t)a * per + nA;
    T *W = w_in_smem ? A + nA : nullptr;
    const long long i = i0 + a;
    for (int e = t; e < nA; e += blockDim.x)
      A[e] = A_in32 ? T(A_in32[i * nA + e]) : as_compute(A_in[i * nA + e], T(0));
    if (W)
      for (int q = t; q < nd; q += blockDim.x)
        W[q] = gB2[i * nd + q];
  }
  __syncthreads();
  // u = dE/dA: u[c][lm] = sum_b (1 + [b == c]) w((c,b), l) A[b][lm], b
  // ascending, stored as u[s][lm][n] (c = s n_max + n) so that a pair reads
  // a harmonic's n_max values together.  The B2 index of the radial pair
  // (min(b,c), max(b,c)) advances by nr - b - 1 while b < c and by 1 after
  // it, so the loop carries it instead of recomputing it.
  if constexpr (LC > 0) {
    // a thread per (l, atom, c) computes the 2l + 1 entries of (c, l),
    // loading each weight w((c,b), l) once for them (l slowest, so that
    // the threads of a warp mostly share l and its entry count)
    const int nac = na * nr;
    for (int it = t; it < L1 * nac; it += blockDim.x) {
      const int l = it / nac, r2 = it - l * nac;
      const int a = r2 / nr, c = r2 - a * nr;
      const T *A = smem + (size_t)a * per + nA;
      T *u = smem + (size_t)a * per;
      const T *wsrc = w_in_smem ? A + nA : gB2 + (long long)(i0 + a) * nd;
      const int cs = c / nm, cn = c - cs * nm;
      switch (l) {
        case 0: u_entries<T, 1>(A, wsrc, nh, nr, L1, c, 0, u, nm, cs, cn); break;
        case 1: u_entries<T, 3>(A, wsrc, nh, nr, L1, c, 1, u, nm, cs, cn); break;
        case 2: if constexpr (LC >= 2) u_entries<T, 5>(A, wsrc, nh, nr, L1, c, 2, u, nm, cs, cn); break;
        case 3: if constexpr (LC >= 3) u_entries<T, 7>(A, wsrc, nh, nr, L1, c, 3, u, nm, cs, cn); break;
        case 4: if constexpr (LC >= 4) u_entries<T, 9>(A, wsrc, nh, nr, L1, c, 4, u, nm, cs, cn); break;
        default: u_entries_any<T>(A, wsrc, nh, nr, L1, c, l, u, nm, cs, cn); break;
      }
    }
  } else {
    for (int it = t; it < na * nA; it += blockDim.x) {
      const int a = it / nA, e = it - a * nA;
      const T *A = smem + (size_t)a * per + nA;
      T *u = smem + (size_t)a * per;
      const T *wsrc = w_in_smem ? A + nA : gB2 + (long long)(i0 + a) * nd;
      const int c = e / nh, lm = e - c * nh;
      int l = 0;
      while ((l + 1) * (l + 1) <= lm) l++;
      const T *Acol = A + lm;
      const T *wl = wsrc + l;
      T acc = T(0);
      int pidx = c;   // radial pair (0, c)
      for (int bb = 0; bb < c; bb++) {
        acc += wl[pidx * L1] * Acol[bb * nh];
        pidx += nr - bb - 1;
      }
      // pidx is now the pair (c, c)
      acc += T(2) * wl[pidx * L1] * Acol[c * nh];
      for (int bb = c + 1; bb < nr; bb++) {
        pidx++;
        acc += wl[pidx * L1] * Acol[bb * nh];
      }
      const int cs = c / nm, cn = c - cs * nm;
      u[(cs * nh + lm) * nm + cn] = acc;
    }
  }
  __syncthreads();
  const long long pbeg = offsets[i0], pend = offsets[i0 + na];
  for (long long pp = pbeg + t; pp < pend; pp += blockDim.x) {
    int a = 0;
    while (a + 1 < na && pp >= offsets[i0 + a + 1]) a++;
    const T *u = smem + (size_t)a * per;
    const int si = species[i0 + a];
    int j = nbr_j[pp];
    double4_16a r = rel[pp];
    int sj = species[j];
    double rc = p.cutoffs[si * kMaxSpecies + sj];
    typename PairGrad<T>::type out = pair_out(T(0), T(0), T(0));
    if (r.x <= rc) {
      // dE/dr = sum_{n,lm} u[n][lm] (dg_n/dr e Y_lm + g_n dY_lm/dr)
      //       = e sum_lm d_lm Y_lm + sum_lm c_lm dY_lm/dr, with
      // c_lm = sum_n u[n][lm] g_n and d_lm = sum_n u[n][lm] dg_n/dr formed
      // as the recurrence produces each harmonic (20 multiply-adds per
      // harmonic instead of 4 n_max)
      T g[NA], dg[NA];
      const T rx = as_compute(r.x, T(0)), ry = as_compute(r.y, T(0)),
              rz = as_compute(r.z, T(0)), rw = as_compute(r.w, T(0));
      radial_eval<T, NC>(p, rx, as_compute(rc, T(0)), g, dg);
      const T *us = u + sj * nm * nh;
      T orad = T(0), ox = T(0), oy = T(0), oz = T(0);
      ylm_visit<T, LC, true>(p.l_max, ry, rz, rw,
                             [&](int idx, T v, T gx, T gy, T gz) {
        T c = T(0), d = T(0);
        const T *ul = us + idx * nm;
        if constexpr (std::is_same<T, float>::value && NC > 0 && NC % 4 == 0) {
          // n_max values of the harmonic in 16-byte loads (u rows start on
          // 16-byte boundaries: per and n_max n_harm are whole 4-groups)
#pragma unroll
          for (int q = 0; q < NC / 4; q++) {
            const float4 uv = reinterpret_cast<const float4 *>(ul)[q];
            c += uv.x * g[4 * q];     d += uv.x * dg[4 * q];
            c += uv.y * g[4 * q + 1]; d += uv.y * dg[4 * q + 1];
            c += uv.z * g[4 * q + 2]; d += uv.z * dg[4 * q + 2];
            c += uv.w * g[4 * q + 3]; d += uv.w * dg[4 * q + 3];
          }
        } else {
#pragma unroll
          for (int n = 0; n < nm; n++) {
            const T uv = ul[n];
            c += uv * g[n];
            d += uv * dg[n];
          }
        }
        orad += d * v;
        ox += c * gx;
        oy += c * gy;
        oz += c * gz;
      });
      const T ir = T(1) / rx;
      out = pair_out(orad * (ry * ir) + ox, orad * (rz * ir) + oy,
                     orad * (rw * ir) + oz);
    }
    pair_grad[pp] = out;
  }
}

// F_i = sum_{p in out(i)} (g_p - g_twin(p)); per-atom virial partials
// v_i[ab] = sum_{p in out(i)} g_p,a r_p,b (flare order xx xy xz yy yz zz).
// kForceLanes lanes per atom take its pairs lane, lane + kForceLanes, ...
// (enough threads to hide the dependent twin loads), then a fixed-order
// butterfly over those lanes sums them (each level is 9 FP64 additions per
// lane, so the group stays small: FP64 is scarce on this GPU).
// Sums in the pair gradients' type (FP32 after the FP32 adjoint).
constexpr int kForceLanes = 4;
template <typename T>
__global__ void k_forces(int n_atoms, const long long *__restrict__ offsets,
                         const long long *__restrict__ twin,
                         const double4_16a *__restrict__ rel,
                         const typename PairGrad<T>::type *__restrict__ pg,
                         double *__restrict__ forces,
                         double *__restrict__ virial) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = (int)(gt % kForceLanes);
  // whole groups of kForceLanes lanes leave together (n_atoms is uniform)
  const int i = (int)(gt / kForceLanes);
  if (i >= n_atoms) return;
  T a[9] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
  const long long e = offsets[i + 1];   // a: F (3), virial (6)
  for (long long q = offsets[i] + lane; q < e; q += kForceLanes) {
    const auto g = pg[q];
    const long long tw = twin[q];
    const auto h = tw >= 0 ? pg[tw] : pair_out(T(0), T(0), T(0));
    a[0] += g.x - h.x;
    a[1] += g.y - h.y;
    a[2] += g.z - h.z;
    const double4_16a r = rel[q];
    const T ry = as_compute(r.y, T(0)), rz = as_compute(r.z, T(0)),
            rw = as_compute(r.w, T(0));
    a[3] += g.x * ry; a[4] += g.x * rz; a[5] += g.x * rw;
    a[6] += g.y * rz; a[7] += g.y * rw; a[8] += g.z * rw;
  }
  // the group's lanes are consecutive lanes of one warp; groups past
  // n_atoms returned as a whole, so the mask names the live lanes
  const unsigned gmask = ((1u << kForceLanes) - 1u)
                         << ((threadIdx.x & 31) & ~(kForceLanes - 1));
#pragma unroll
  for (int off = kForceLanes / 2; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < 9; k++) a[k] += __shfl_xor_sync(gmask, a[k], off);
  if (lane == 0) {
    if (forces)
      for (int k = 0; k < 3; k++) forces[3 * i + k] = (double)a[k];
    if (virial)
      for (int k = 0; k < 6; k++) virial[6 * i + k] = (double)a[3 + k];
  }
}

// Per-structure energy and stress: fixed-order tree sums over the
// structure's atoms.  One block per structure.
__global__ void k_struct_reduce(int n_struc, const int *__restrict__ atom_off,
                                const double *__restrict__ volume,
                                const double *__restrict__ e_atom,
                                const double *__restrict__ virial,
                                double *__restrict__ energy,
                                double *__restrict__ stress) {
  __shared__ double red[7][256];
  int s = blockIdx.x;
  if (s >= n_struc) return;
  int t = threadIdx.x;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int a = atom_off[s] + t; a < atom_off[s + 1]; a += blockDim.x) {
    if (e_atom) acc[0] += e_atom[a];
    if (virial)
      for (int k = 0; k < 6; k++) acc[1 + k] += virial[6 * a + k];
  }
  for (int k = 0; k < 7; k++) red[k][t] = acc[k];
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (t < h)
      for (int k = 0; k < 7; k++) red[k][t] += red[k][t + h];
    __syncthreads();
  }
  if (t == 0) {
    if (energy) energy[s] = red[0][0];
    if (stress)
      for (int k = 0; k < 6; k++) stress[6 * s + k] = -red[1 + k][0] / volume[s];
  }
}

}  // namespace

size_t b2_forward_smem(const B2Params &p, bool regA) {
  // A (unless it stays in registers and is laid over Y) | g | Y | pair
  // species | reduction | species-sorted pair order and per-warp species
  // counts (2 x kMaxSpecies) and starts (kMaxSpecies + 1)
  return sizeof(double) * ((regA ? 0 : p.n_A) +
                           (size_t)kChunk * (p.n_max + p.n_harm)) +
         sizeof(int) * kChunk + sizeof(double) * kChunk +
         sizeof(int) * (kChunk + 3 * kMaxSpecies + 1);
}


// The descriptor sizes with compile-time specialisations (registers instead
// of local memory for the per-pair basis values; Chebyshev basis); others
// take the runtime-sized kernels.
template <template <typename, int, int> class K, typename T, typename F>
static void dispatch_nl(const B2Params &p, F &&f) {
  const bool cheb = p.radial_basis == FGB_RADIAL_CHEBYSHEV;
  if (cheb && p.n_max == 8 && p.l_max == 4) f(K<T, 8, 4>{});
  else if (cheb && p.n_max == 8 && p.l_max == 3) f(K<T, 8, 3>{});
  else if (cheb && p.n_max == 10 && p.l_max == 6) f(K<T, 10, 6>{});
  else f(K<T, 0, 0>{});
}

template <typename T, int NC, int LC>
struct FwdK {
  static constexpr auto fn = k_b2_forward<T, NC, LC>;
  static constexpr bool kFixed = NC > 0 && LC > 0;
};
template <typename T, int NC, int LC>
struct AdjK {
  static constexpr auto fn = k_b2_adjoint<T, NC, LC>;
  using type = T;
};

int launch_b2_forward(const B2Params &p, const fgb_nlist_s *nl,
                      const int *d_species, double *d_A, double *d_B2,
                      double *d_norms, cudaStream_t st, bool dfloat,
                      double *d_rowmax, float *d_A32) {
  const int N = nl->n_atoms;
  if (N == 0) return FGB_OK;
  const size_t sm_full = b2_forward_smem(p, false);   // sizeof(df) == 8
  if (sm_full > 200 * 1024) {
    set_error("B2 settings need %zu bytes of shared memory", sm_full);
    return FGB_EINVAL;
  }
  cudaError_t e = cudaSuccess;
  auto go = [&](auto k) {
    auto fn = decltype(k)::fn;
    // the specialised kernels keep A in registers when one (species, lm)
    // per thread covers it (the same test as in the kernel)
    const bool regA = decltype(k)::kFixed && p.n_species * p.n_harm <= kChunk &&
                      p.n_species * p.n_max <= kChunk;
    const size_t sm = b2_forward_smem(p, regA);
    // all of the SM's unified memory as shared memory: twelve blocks of
    // ~19 KB each
    e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sm);
    if (e != cudaSuccess) return;
    fn<<<N, kChunk, sm, st>>>(p, N, nl->offsets.as<long long>(),
                              nl->nbr_j.as<int>(), nl->nbr_rel.as<double4_16a>(),
                              d_species, d_A, d_B2, d_norms, d_rowmax, d_A32);
  };
  if (dfloat) dispatch_nl<FwdK, df>(p, go);
  else dispatch_nl<FwdK, double>(p, go);
  FGB_CUDA(e);
  FGB_LAUNCH_CHECK("k_b2_forward");
  return FGB_OK;
}

int launch_b2_adjoint(const B2Params &p, const fgb_nlist_s *nl,
                      const int *d_species, const double *d_A,
                      const void *d_gB2, void *d_pair_grad,
                      cudaStream_t st, bool fp32, const float *d_A32) {
  const int N = nl->n_atoms;
  if (N == 0) return FGB_OK;
  // per atom of a block: u and A, and the atom's dE/dB2 row when it fits
  const size_t es = fp32 ? sizeof(float) : sizeof(double);
  size_t sm = es * (size_t)adj_atom_values(p.n_A, 0) * kAdjAtoms;
  if (sm > 200 * 1024) {
    set_error("B2 adjoint needs %zu bytes of shared memory", sm);
    return FGB_EINVAL;
  }
  const size_t smw = es * (size_t)adj_atom_values(p.n_A, p.n_d) * kAdjAtoms;
  const int w_in_smem = smw <= 96 * 1024 ? 1 : 0;
  if (w_in_smem) sm = smw;
  cudaError_t e = cudaSuccess;
  auto go = [&](auto k) {
    auto fn = decltype(k)::fn;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sm);
    if (e != cudaSuccess) return;
    using G = typename decltype(k)::type;   // dE/dB2 in the compute type
    fn<<<ceil_div(N, kAdjAtoms), kAdjThreads, sm, st>>>(
        p, N, nl->offsets.as<long long>(), nl->nbr_j.as<int>(),
        nl->nbr_rel.as<double4_16a>(), d_species, d_A,
        fp32 ? d_A32 : nullptr, static_cast<const G *>(d_gB2),
        static_cast<typename PairGrad<G>::type *>(d_pair_grad), w_in_smem);
  };
  if (fp32) dispatch_nl<AdjK, float>(p, go);
  else dispatch_nl<AdjK, double>(p, go);
  FGB_CUDA(e);
  FGB_LAUNCH_CHECK("k_b2_adjoint");
  return FGB_OK;
}

int launch_forces(const fgb_nlist_s *nl, const void *d_pair_grad, bool fp32,
                  double *d_forces, double *d_virial, cudaStream_t st) {
  const int N = nl->n_atoms;
  if (N == 0) return FGB_OK;
  const unsigned nb = (unsigned)ceil_div((long long)N * kForceLanes, 256);
  if (fp32)
    k_forces<float><<<nb, 256, 0, st>>>(
        N, nl->offsets.as<long long>(), nl->nbr_twin.as<long long>(),
        nl->nbr_rel.as<double4_16a>(), static_cast<const float3 *>(d_pair_grad),
        d_forces, d_virial);
  else
    k_forces<double><<<nb, 256, 0, st>>>(
        N, nl->offsets.as<long long>(), nl->nbr_twin.as<long long>(),
        nl->nbr_rel.as<double4_16a>(),
        static_cast<const double3 *>(d_pair_grad), d_forces, d_virial);
  FGB_LAUNCH_CHECK("k_forces");
  return FGB_OK;
}

int launch_struct_reduce(int n_struc, const int *d_atom_off,
                         const double *d_volume, const double *d_e_atom,
                         const double *d_virial, double *d_energy,
                         double *d_stress, cudaStream_t st) {
  k_struct_reduce<<<n_struc, 256, 0, st>>>(n_struc, d_atom_off, d_volume,
                                           d_e_atom, d_virial, d_energy,
                                           d_stress);
  FGB_LAUNCH_CHECK("k_struct_reduce");
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_b2_forward(fgb_b2_t b2, fgb_nlist_t nl, const int *d_species,
                              double *d_B2, double *d_norms, void *stream) {
  if (!b2 || !nl || !d_B2 || !d_norms) {
    set_error("fgb_b2_forward: invalid arguments");
    return FGB_EINVAL;
  }
  if (nl->n_atoms > 0 && !d_species) {
    set_error("fgb_b2_forward: species required");
    return FGB_EINVAL;
  }
  return launch_b2_forward(b2->p, nl, d_species, nullptr, d_B2, d_norms,
                           (cudaStream_t)stream);
}
