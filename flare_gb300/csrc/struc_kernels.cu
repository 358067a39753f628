// Structure kernels of the NormalizedDotProduct kernel on the GPU in FP64:
// self_kernel_struc (kernels/normalized_dot_product.cpp:450-586; the K_self
// term of SparseGP::predict_DTC, bffs/sparse_gp.cpp:694-729) and
// struc_struc (normalized_dot_product.cpp:216-448).
//
// The reference forms, per species, force_force = dD1 dD2^T over every pair
// of neighbour entries (3P1 x 3P2) and loops over atom pairs x entry pairs.
// Each force-force term is the bilinear form
//     g_p^T H_ij g_q,   H_ij = d2 k(d_i, d_j) / dd_i dd_j
//     = sig2 [ xi (xi-1) c^(xi-2) (P_i u_j)(P_j u_i)^T + xi c^(xi-1) P_i P_j ]
// with u = d/|d|, c = u_i.u_j, P = (I - u u^T)/|d|, and the four index
// tests of the reference's scatter make the entry of atoms (a, b)
//     sum_ij G_ia^T H_ij G_jb,   G_ia = dd_i/dr_a = sum_p (delta(a, n_p) -
//                                                   delta(a, i)) g_p,
// non-zero only for i = a and the neighbours of a.  Stress entries use the
// rows W_i,mn = sum_p g_p,m x_p,n over V, energy-force entries
// -sig2 xi c^(xi-1) u_i.(P_j G_jb).  So every entry is a sum over atom or
// neighbourhood pairs of a few dot products of projected rows; nothing of
// size P x P is formed.
#include <algorithm>
#include <vector>

#include "fgb_internal.h"
#include "fgb_kernels.h"
#include "fgb_model.h"

namespace fgb {
namespace {

constexpr int kDT = 256;   // threads of the row kernels
constexpr int kTile = 16;  // atoms per side of a pair tile
constexpr int kKC = 16;    // columns per shared-memory chunk

// Sum over the block in a fixed order (deterministic); all threads get it.
__device__ double block_sum(double v, double *red) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int k = 0; k < nw; k++) t += red[k];
  return t;
}

__device__ __forceinline__ double pw(double c, double xi) {
  if (xi == 2.0) return c * c;
  if (xi == 1.0) return c;
  if (xi == 0.0) return 1.0;
  return pow(c, xi);
}

// Unit rows u (zero for empty descriptors) and projected stress rows
// W^_mn = P_i W_mn, both in species-sorted row order r (atom perm[r]).
__global__ void __launch_bounds__(kDT)
k_dtc_rows(int N, int nd, const int *__restrict__ perm,
           const double *__restrict__ B2, const double *__restrict__ norms,
           const long long *__restrict__ offsets,
           const double4_16a *__restrict__ rel, const double *__restrict__ dB2,
           double *__restrict__ U, double *__restrict__ W) {
  __shared__ double red[32];
  const int r = blockIdx.x;
  if (r >= N) return;
  const int a = perm[r];
  const double n = norms[a];
  const bool ok = n >= kEmptyThresh;
  const double inv = ok ? 1.0 / n : 0.0;
  const long long p0 = offsets[a], p1 = offsets[a + 1];
  double *Ur = U + (long long)r * nd;
  double *Wr = W + (long long)r * 6 * nd;
  double dot[6] = {0, 0, 0, 0, 0, 0};
  for (int k = threadIdx.x; k < nd; k += kDT) {
    const double u = ok ? B2[(long long)a * nd + k] * inv : 0.0;
    Ur[k] = u;
    double w[6] = {0, 0, 0, 0, 0, 0};
    if (ok)
      for (long long p = p0; p < p1; p++) {
        const double4_16a x = rel[p];
        const double g0 = dB2[(3 * p + 0) * nd + k];
        const double g1 = dB2[(3 * p + 1) * nd + k];
        const double g2 = dB2[(3 * p + 2) * nd + k];
        w[0] += g0 * x.y; w[1] += g0 * x.z; w[2] += g0 * x.w;
        w[3] += g1 * x.z; w[4] += g1 * x.w; w[5] += g2 * x.w;
      }
#pragma unroll
    for (int c = 0; c < 6; c++) {
      Wr[(long long)c * nd + k] = w[c];
      dot[c] += u * w[c];
    }
  }
#pragma unroll
  for (int c = 0; c < 6; c++) dot[c] = block_sum(dot[c], red);
  // each thread rewrites the columns it wrote above
  for (int k = threadIdx.x; k < nd; k += kDT) {
    const double u = Ur[k];
#pragma unroll
    for (int c = 0; c < 6; c++) {
      double *x = Wr + (long long)c * nd + k;
      *x = (*x - u * dot[c]) * inv;
    }
  }
}

// Neighbourhood slots of atom a: a itself, then each distinct neighbour
// j != a (a's list is ordered by j, so repeats through images are runs).
__global__ void k_dtc_slot_count(int N, const long long *__restrict__ offsets,
                                 const int *__restrict__ nbr_j,
                                 int *__restrict__ cnt) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  int c = 1, prev = -1;
  for (long long p = offsets[a]; p < offsets[a + 1]; p++) {
    const int j = nbr_j[p];
    if (j != prev && j != a) c++;
    prev = j;
  }
  cnt[a] = c;
}

// Projected neighbourhood gradients G^_ia,m = P_i dd_i/dr_a,m for every
// slot (a, i): G = sum over a's pairs q with j_q = i of g_twin(q) (the pairs
// of i whose neighbour is a), minus sum_p g_p of a's own pairs when i = a.
// slot_row[t] = sorted row of i, or -1 for an empty descriptor.
// Atoms a0 .. a0 + n - 1 (one block each); slot_base is local to them.
__global__ void __launch_bounds__(kDT)
k_dtc_slots(int a0, int n, int nd, const int *__restrict__ inv_perm,
            const double *__restrict__ norms, const long long *__restrict__ offsets,
            const int *__restrict__ nbr_j, const long long *__restrict__ twin,
            const double *__restrict__ dB2, const double *__restrict__ U,
            const long long *__restrict__ slot_base, int *__restrict__ slot_row,
            double *__restrict__ G) {
  __shared__ double red[32];
  if ((int)blockIdx.x >= n) return;
  const int a = a0 + blockIdx.x;
  const long long p0 = offsets[a], p1 = offsets[a + 1];
  long long t = slot_base[blockIdx.x];
  long long q = p0;
  // slot 0 is a; then one slot per run of equal j (j != a)
  for (int slot = 0;; slot++) {
    int i;
    long long q0, q1;
    if (slot == 0) {
      i = a;
      q0 = p0; q1 = p1;
    } else {
      while (q < p1 && nbr_j[q] == a) q++;
      if (q >= p1) break;
      i = nbr_j[q];
      q0 = q;
      while (q < p1 && nbr_j[q] == i) q++;
      q1 = q;
    }
    const bool ok = norms[i] >= kEmptyThresh;
    const double inv = ok ? 1.0 / norms[i] : 0.0;
    const int ri = inv_perm[i];
    const double *Ui = U + (long long)ri * nd;
    double *Gt = G + t * 3 * nd;
    double dot[3] = {0, 0, 0};
    for (int k = threadIdx.x; k < nd; k += kDT) {
      double g[3] = {0, 0, 0};
      if (ok) {
        for (long long p = q0; p < q1; p++) {
          if (nbr_j[p] != i) continue;
          const long long tw = twin[p];
#pragma unroll
          for (int m = 0; m < 3; m++) g[m] += dB2[(3 * tw + m) * nd + k];
        }
        if (slot == 0)
          for (long long p = p0; p < p1; p++)
#pragma unroll
            for (int m = 0; m < 3; m++) g[m] -= dB2[(3 * p + m) * nd + k];
      }
      const double u = Ui[k];
#pragma unroll
      for (int m = 0; m < 3; m++) {
        Gt[(long long)m * nd + k] = g[m];
        dot[m] += u * g[m];
      }
    }
#pragma unroll
    for (int m = 0; m < 3; m++) dot[m] = block_sum(dot[m], red);
    for (int k = threadIdx.x; k < nd; k += kDT) {
      const double u = Ui[k];
#pragma unroll
      for (int m = 0; m < 3; m++) {
        double *x = Gt + (long long)m * nd + k;
        *x = (*x - u * dot[m]) * inv;
      }
    }
    if (threadIdx.x == 0) slot_row[t] = ok ? ri : -1;
    t++;
  }
}

// Force entries: one block per atom a, one warp per unordered slot pair
// (x <= y) of the same species; 10 dot products per pair.
__global__ void __launch_bounds__(kDT)
k_dtc_force_var(int a0, int n_atoms, int nd, const int *__restrict__ species_row,
                const long long *__restrict__ slot_base,
                const int *__restrict__ slot_row, const double *__restrict__ U,
                const double *__restrict__ G, double sig2, double xi,
                double *__restrict__ out) {
  __shared__ double red[3][kDT / 32];
  if ((int)blockIdx.x >= n_atoms) return;
  const int a = a0 + blockIdx.x;
  const long long t0 = slot_base[blockIdx.x];
  const int n = (int)(slot_base[blockIdx.x + 1] - t0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double acc[3] = {0, 0, 0};
  const int npairs = n * (n + 1) / 2;
  for (int idx = warp; idx < npairs; idx += kDT / 32) {
    // idx -> (x, y), x <= y, row-major over the upper triangle
    int x = 0, rem = idx;
    while (rem >= n - x) { rem -= n - x; x++; }
    const int y = x + rem;
    const int ri = slot_row[t0 + x], rj = slot_row[t0 + y];
    if (ri < 0 || rj < 0 || species_row[ri] != species_row[rj]) continue;
    const double *ui = U + (long long)ri * nd, *uj = U + (long long)rj * nd;
    const double *gx = G + (t0 + x) * 3 * nd, *gy = G + (t0 + y) * 3 * nd;
    double c = 0, A[3] = {0, 0, 0}, B[3] = {0, 0, 0}, Y[3] = {0, 0, 0};
    for (int k = lane; k < nd; k += 32) {
      const double vi = ui[k], vj = uj[k];
      c += vi * vj;
#pragma unroll
      for (int m = 0; m < 3; m++) {
        const double a1 = gx[(long long)m * nd + k], b1 = gy[(long long)m * nd + k];
        A[m] += a1 * vj;
        B[m] += b1 * vi;
        Y[m] += a1 * b1;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      c += __shfl_xor_sync(0xffffffffu, c, off);
#pragma unroll
      for (int m = 0; m < 3; m++) {
        A[m] += __shfl_xor_sync(0xffffffffu, A[m], off);
        B[m] += __shfl_xor_sync(0xffffffffu, B[m], off);
        Y[m] += __shfl_xor_sync(0xffffffffu, Y[m], off);
      }
    }
    const double mult = x == y ? 1.0 : 2.0;
    const double f2 = (xi - 1) * xi * pw(c, xi - 2), f1 = xi * pw(c, xi - 1);
#pragma unroll
    for (int m = 0; m < 3; m++) acc[m] += mult * (f2 * A[m] * B[m] + f1 * Y[m]);
  }
  if (lane == 0)
    for (int m = 0; m < 3; m++) red[m][warp] = acc[m];
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int w = 0; w < kDT / 32; w++) s += red[threadIdx.x][w];
    out[1 + 3LL * a + threadIdx.x] = sig2 * s;
  }
}

// Energy and stress entries: tiles of 16 x 16 atom pairs (j >= i) inside
// each species' sorted rows; per pair c, W^_i.u_j, W^_j.u_i, W^_i.W^_j for
// the six stress components.  part[tile] = {energy, stress[6]} partial
// sums; bad[0] set where |c| < 1e-8 with power < 2 (the reference throws).
__global__ void __launch_bounds__(kTile *kTile)
k_dtc_struct_tiles(int nd, const int4 *__restrict__ tiles,
                   const unsigned char *__restrict__ valid,
                   const double *__restrict__ U, const double *__restrict__ W,
                   double xi, double *__restrict__ part, int *__restrict__ bad) {
  __shared__ double sI[7][kKC][kTile + 1], sJ[7][kKC][kTile + 1];
  __shared__ double red[8][7];
  const int4 tl = tiles[blockIdx.x];   // i0, j0, end (exclusive), unused
  const int ti = threadIdx.x / kTile, tj = threadIdx.x % kTile;
  const int i = tl.x + ti, j = tl.y + tj;
  const bool act = i < tl.z && j < tl.z && j >= i && valid[i] && valid[j];
  double c = 0, A[6] = {0}, B[6] = {0}, Y[6] = {0};
  for (int k0 = 0; k0 < nd; k0 += kKC) {
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * 7 * kTile * kKC; e += kTile * kTile) {
      const int side = e / (7 * kTile * kKC);
      int rem = e % (7 * kTile * kKC);
      const int v = rem / (kTile * kKC);
      rem %= kTile * kKC;
      const int row = rem / kKC, kk = rem % kKC;
      const int r = (side ? tl.y : tl.x) + row, k = k0 + kk;
      double val = 0.0;
      if (r < tl.z && k < nd)
        val = v == 0 ? U[(long long)r * nd + k]
                     : W[((long long)r * 6 + (v - 1)) * nd + k];
      (side ? sJ : sI)[v][kk][row] = val;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kKC; kk++) {
      const double ui = sI[0][kk][ti], uj = sJ[0][kk][tj];
      c += ui * uj;
#pragma unroll
      for (int q = 0; q < 6; q++) {
        const double wi = sI[q + 1][kk][ti], wj = sJ[q + 1][kk][tj];
        A[q] += wi * uj;
        B[q] += wj * ui;
        Y[q] += wi * wj;
      }
    }
  }
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  if (act) {
    if (xi < 2.0 && fabs(c) < kEmptyThresh) atomicOr(bad, 1);
    const double mult = i == j ? 1.0 : 2.0;
    const double f2 = (xi - 1) * xi * pw(c, xi - 2), f1 = xi * pw(c, xi - 1);
    v[0] = mult * pw(c, xi);
#pragma unroll
    for (int q = 0; q < 6; q++) v[q + 1] = mult * (f2 * A[q] * B[q] + f1 * Y[q]);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < 7; q++) {
    double s = v[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) red[w][q] = s;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    double s = 0.0;
    for (int k = 0; k < kTile * kTile / 32; k++) s += red[k][threadIdx.x];
    part[(long long)blockIdx.x * 7 + threadIdx.x] = s;
  }
}

__global__ void k_dtc_struct_final(int n_tiles, int N, const double *__restrict__ part,
                                   double sig2, double vol_inv,
                                   double *__restrict__ out) {
  const int q = threadIdx.x;
  if (q >= 7) return;
  double s = 0.0;
  for (int t = 0; t < n_tiles; t++) s += part[(long long)t * 7 + q];
  if (q == 0) out[0] = sig2 * s;
  else out[1 + 3LL * N + (q - 1)] = sig2 * vol_inv * vol_inv * s;
}

// ---------------------------------------------------------- struc_struc
// Output groups of one structure: the energy (C = 1, items = atoms), each
// atom's three force components (items = its neighbourhood slots) and the
// stress in two halves of three components (items = atoms).
struct SsGroup {
  int beg, end;          // item range
  int idx_shift;         // item -> row index of `base`
  int C;                 // components (1 or 3)
  const double *base;    // component rows (C > 1)
  long long stride;      // doubles per row index
  int comp0;             // first component within a row index
  long long out0;        // output index of component 0
  double scale;          // 1, or 1/V for stress
};
struct SsWork {
  int g1, g2;
  long long p0, p1;      // item pairs [p0, p1) of the group pair
};
struct SsPair {
  int g1, g2, w0, w1;    // work items [w0, w1) of the group pair
};

// One block per work item, one warp per item pair: c, A_p = R1_p.u_j,
// B_q = R2_q.u_i, Y_pq = R1_p.R2_q; lane L < C1 C2 keeps entry (L / C2,
// L % C2) of the partial sum.
template <int C1, int C2>
__global__ void __launch_bounds__(kDT)
k_ss(const SsWork *__restrict__ work, const SsGroup *__restrict__ G1,
     const SsGroup *__restrict__ G2, const int *__restrict__ row1,
     const int *__restrict__ row2, const int *__restrict__ sp1,
     const int *__restrict__ sp2, const double *__restrict__ U1,
     const double *__restrict__ U2, int nd, double xi,
     double *__restrict__ part, int *__restrict__ bad) {
  __shared__ double red[kDT / 32][C1 * C2];
  const SsWork wk = work[blockIdx.x];
  const SsGroup g1 = G1[wk.g1], g2 = G2[wk.g2];
  const int n2 = g2.end - g2.beg;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double acc = 0.0;
  for (long long pr = wk.p0 + warp; pr < wk.p1; pr += kDT / 32) {
    const int xi1 = g1.beg + (int)(pr / n2), xi2 = g2.beg + (int)(pr % n2);
    const int ri = row1[xi1], rj = row2[xi2];
    if (ri < 0 || rj < 0 || sp1[ri] != sp2[rj]) continue;
    const double *ui = U1 + (long long)ri * nd, *uj = U2 + (long long)rj * nd;
    const double *r1 = g1.base + (long long)(xi1 - g1.idx_shift) * g1.stride +
                       (long long)g1.comp0 * nd;
    const double *r2 = g2.base + (long long)(xi2 - g2.idx_shift) * g2.stride +
                       (long long)g2.comp0 * nd;
    double c = 0, A[3] = {0, 0, 0}, B[3] = {0, 0, 0}, Y[3][3] = {};
    for (int k = lane; k < nd; k += 32) {
      const double vi = ui[k], vj = uj[k];
      c += vi * vj;
      double a1[3], b1[3];
#pragma unroll
      for (int q = 0; q < 3; q++) {
        a1[q] = C1 > 1 ? r1[(long long)q * nd + k] : 0.0;
        b1[q] = C2 > 1 ? r2[(long long)q * nd + k] : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 3; q++) {
        if (C1 > 1) A[q] += a1[q] * vj;
        if (C2 > 1) B[q] += b1[q] * vi;
      }
      if (C1 > 1 && C2 > 1) {
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
          for (int q = 0; q < 3; q++) Y[p][q] += a1[p] * b1[q];
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      c += __shfl_xor_sync(0xffffffffu, c, off);
#pragma unroll
      for (int q = 0; q < 3; q++) {
        if (C1 > 1) A[q] += __shfl_xor_sync(0xffffffffu, A[q], off);
        if (C2 > 1) B[q] += __shfl_xor_sync(0xffffffffu, B[q], off);
      }
      if (C1 > 1 && C2 > 1) {
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
          for (int q = 0; q < 3; q++)
            Y[p][q] += __shfl_xor_sync(0xffffffffu, Y[p][q], off);
      }
    }
    if (C1 == 1 && C2 == 1) {
      if (xi < 2.0 && fabs(c) < kEmptyThresh && lane == 0) atomicOr(bad, 1);
      acc += pw(c, xi);
    } else if (lane < C1 * C2) {
      const double f1 = xi * pw(c, xi - 1);
      const int p = lane / C2, q = lane % C2;
      double v;
      if (C1 == 1) {
        v = -f1 * B[q];
      } else if (C2 == 1) {
        v = -f1 * A[p];
      } else {
        const double f2 = (xi - 1) * xi * pw(c, xi - 2);
        double a = 0, b = 0, y = 0;
#pragma unroll
        for (int pp = 0; pp < 3; pp++) {
          if (pp == p) a = A[pp];
#pragma unroll
          for (int qq = 0; qq < 3; qq++)
            if (pp == p && qq == q) y = Y[pp][qq];
        }
#pragma unroll
        for (int qq = 0; qq < 3; qq++)
          if (qq == q) b = B[qq];
        v = f2 * a * b + f1 * y;
      }
      acc += v;
    }
  }
  if (lane < C1 * C2) red[warp][lane] = acc;
  __syncthreads();
  if (threadIdx.x < C1 * C2) {
    double t = 0.0;
    for (int w = 0; w < kDT / 32; w++) t += red[w][threadIdx.x];
    part[(long long)blockIdx.x * C1 * C2 + threadIdx.x] = t;
  }
}

// Sum each group pair's work items in order and write its entries.
template <int C1, int C2>
__global__ void k_ss_final(int n_pairs, const SsPair *__restrict__ pairs,
                           const SsGroup *__restrict__ G1,
                           const SsGroup *__restrict__ G2,
                           const double *__restrict__ part, double sig2,
                           long long ncol, double *__restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n_pairs * C1 * C2) return;
  const int gp = (int)(t / (C1 * C2)), L = (int)(t % (C1 * C2));
  const SsPair pr = pairs[gp];
  double s = 0.0;
  for (int w = pr.w0; w < pr.w1; w++) s += part[(long long)w * C1 * C2 + L];
  const SsGroup g1 = G1[pr.g1], g2 = G2[pr.g2];
  out[(g1.out0 + L / C2) * ncol + g2.out0 + L % C2] =
      sig2 * g1.scale * g2.scale * s;
}

}  // namespace

int self_kernel_impl(const B2Params &p, double sigma, double power,
                     fgb_nlist_s *nl, const int *d_species, double *d_out,
                     fgb_workspace &ws, cudaStream_t st, bool have_dervs) {
  if (nl->n_struc != 1) {
    set_error("self_kernel_struc needs a single-structure neighbour list");
    return FGB_EINVAL;
  }
  const int N = nl->n_atoms, S = p.n_species, nd = p.n_d;
  const long long P = nl->n_pairs;
  const long long ncol = 1 + 3LL * N + 6;
  int rc;
  FGB_CUDA(cudaMemsetAsync(d_out, 0, sizeof(double) * ncol, st));
  if (N == 0) return FGB_OK;
  if (!have_dervs) {
    if ((rc = check_species(d_species, N, S, ws.flag, st))) return rc;
    if ((rc = ws.A.ensure(sizeof(double) * ((size_t)N * p.n_A + 1))) ||
        (rc = ws.B2.ensure(sizeof(double) * ((size_t)N * nd + 1))) ||
        (rc = ws.norms.ensure(sizeof(double) * (N + 1))) ||
        (rc = ws.dB2.ensure(sizeof(double) * ((size_t)3 * P * nd + 1))) ||
        (rc = ws.fdots.ensure(sizeof(double) * (3 * P + 1))))
      return rc;
    if ((rc = launch_b2_forward(p, nl, d_species, ws.A.as<double>(),
                                ws.B2.as<double>(), ws.norms.as<double>(), st)) ||
        (rc = launch_b2_dervs(p, nl, d_species, ws.A.as<double>(),
                              ws.B2.as<double>(), ws.dB2.as<double>(),
                              ws.fdots.as<double>(), st)))
      return rc;
  }
  // species-sorted rows (host: this is a synchronous FP64 path)
  std::vector<int> hs(N);
  std::vector<double> hn(N);
  FGB_CUDA(cudaMemcpyAsync(hs.data(), d_species, sizeof(int) * N,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaMemcpyAsync(hn.data(), ws.norms.p, sizeof(double) * N,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int> perm, inv(N), srow;
  std::vector<unsigned char> valid;
  std::vector<int> sbase(S + 1, 0);
  for (int s = 0; s < S; s++) {
    sbase[s] = (int)perm.size();
    for (int a = 0; a < N; a++)
      if (hs[a] == s) {
        inv[a] = (int)perm.size();
        perm.push_back(a);
        srow.push_back(s);
        valid.push_back(hn[a] >= kEmptyThresh ? 1 : 0);
      }
  }
  sbase[S] = N;
  std::vector<int4> tiles;
  for (int s = 0; s < S; s++)
    for (int i0 = sbase[s]; i0 < sbase[s + 1]; i0 += kTile)
      for (int j0 = i0; j0 < sbase[s + 1]; j0 += kTile)
        tiles.push_back(make_int4(i0, j0, sbase[s + 1], 0));
  DevBuf dperm, dinv, dsrow, dvalid, U, W, cnt, base, srows, G, dtiles, part,
      bad;
  if ((rc = dperm.ensure(sizeof(int) * N)) || (rc = dinv.ensure(sizeof(int) * N)) ||
      (rc = dsrow.ensure(sizeof(int) * N)) || (rc = dvalid.ensure(N)) ||
      (rc = U.ensure(sizeof(double) * (size_t)N * nd)) ||
      (rc = W.ensure(sizeof(double) * (size_t)N * 6 * nd)) ||
      (rc = cnt.ensure(sizeof(int) * N)) ||
      (rc = base.ensure(sizeof(long long) * (N + 1))) ||
      (rc = dtiles.ensure(sizeof(int4) * (tiles.size() + 1))) ||
      (rc = part.ensure(sizeof(double) * 7 * (tiles.size() + 1))) ||
      (rc = bad.ensure(sizeof(int))))
    return rc;
  FGB_CUDA(cudaMemcpyAsync(dperm.p, perm.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(dinv.p, inv.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(dsrow.p, srow.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(dvalid.p, valid.data(), N, cudaMemcpyHostToDevice, st));
  if (!tiles.empty())
    FGB_CUDA(cudaMemcpyAsync(dtiles.p, tiles.data(), sizeof(int4) * tiles.size(),
                             cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  const double sig2 = sigma * sigma;
  k_dtc_rows<<<N, kDT, 0, st>>>(N, nd, dperm.as<int>(), ws.B2.as<double>(),
                                ws.norms.as<double>(),
                                nl->offsets.as<long long>(),
                                nl->nbr_rel.as<double4_16a>(), ws.dB2.as<double>(),
                                U.as<double>(), W.as<double>());
  FGB_LAUNCH_CHECK("k_dtc_rows");
  if (!tiles.empty()) {
    k_dtc_struct_tiles<<<(unsigned)tiles.size(), kTile * kTile, 0, st>>>(
        nd, dtiles.as<int4>(), dvalid.as<unsigned char>(), U.as<double>(),
        W.as<double>(), power, part.as<double>(), bad.as<int>());
    FGB_LAUNCH_CHECK("k_dtc_struct_tiles");
    k_dtc_struct_final<<<1, 32, 0, st>>>((int)tiles.size(), N, part.as<double>(),
                                         sig2, 1.0 / nl->h_volume[0], d_out);
    FGB_LAUNCH_CHECK("k_dtc_struct_final");
  }
  // neighbourhood slots
  k_dtc_slot_count<<<ceil_div(N, 128), 128, 0, st>>>(
      N, nl->offsets.as<long long>(), nl->nbr_j.as<int>(), cnt.as<int>());
  FGB_LAUNCH_CHECK("k_dtc_slot_count");
  std::vector<int> hc(N);
  int hbad = 0;
  FGB_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, sizeof(int) * N,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  if (hbad) {
    set_error("Dot product of descriptors is 0, and the negative power "
              "function in force-force kernel diverges.");
    return FGB_EINVAL;
  }
  // atoms in chunks whose slot rows fit a bounded workspace
  const long long kMaxSlotRows = std::max<long long>(1LL << 16, 4LL * N);
  std::vector<long long> hb(N + 1, 0);
  for (int a = 0; a < N; a++) hb[a + 1] = hb[a] + hc[a];
  for (int a0 = 0; a0 < N;) {
    int a1 = a0 + 1;
    while (a1 < N && hb[a1 + 1] - hb[a0] <= kMaxSlotRows) a1++;
    const long long T = hb[a1] - hb[a0];
    std::vector<long long> lb(a1 - a0 + 1);
    for (int a = a0; a <= a1; a++) lb[a - a0] = hb[a] - hb[a0];
    if ((rc = srows.ensure(sizeof(int) * T)) ||
        (rc = G.ensure(sizeof(double) * (size_t)T * 3 * nd)))
      return rc;
    FGB_CUDA(cudaMemcpyAsync(base.p, lb.data(), sizeof(long long) * lb.size(),
                             cudaMemcpyHostToDevice, st));
    const int n = a1 - a0;
    k_dtc_slots<<<n, kDT, 0, st>>>(
        a0, n, nd, dinv.as<int>(), ws.norms.as<double>(),
        nl->offsets.as<long long>(), nl->nbr_j.as<int>(),
        nl->nbr_twin.as<long long>(), ws.dB2.as<double>(), U.as<double>(),
        base.as<long long>(), srows.as<int>(), G.as<double>());
    FGB_LAUNCH_CHECK("k_dtc_slots");
    k_dtc_force_var<<<n, kDT, 0, st>>>(a0, n, nd, dsrow.as<int>(),
                                        base.as<long long>(), srows.as<int>(),
                                        U.as<double>(), G.as<double>(), sig2,
                                        power, d_out);
    FGB_LAUNCH_CHECK("k_dtc_force_var");
    FGB_CUDA(cudaStreamSynchronize(st));   // chunk buffers are reused
    a0 = a1;
  }
  return FGB_OK;
}


namespace {

// One structure's rows for struc_struc: B2 and stored gradients, unit rows
// U and projected stress rows W (sorted row order), every neighbourhood
// slot's projected gradient rows G, and the item rows (atoms, then slots).
struct SsSide {
  int N = 0;
  double vol = 1.0;
  long long T = 0;
  std::vector<long long> base;        // slot base per atom (N + 1)
  fgb_workspace ws;
  DevBuf dperm, dinv, dsrow, U, W, dbase, srows, G, item_row;
};

int ss_prepare(const B2Params &p, fgb_nlist_s *nl, const int *d_species,
               SsSide &sd, cudaStream_t st) {
  if (nl->n_struc != 1) {
    set_error("struc_struc needs single-structure neighbour lists");
    return FGB_EINVAL;
  }
  const int N = nl->n_atoms, S = p.n_species, nd = p.n_d;
  const long long P = nl->n_pairs;
  sd.N = N;
  sd.vol = nl->h_volume[0];
  int rc;
  fgb_workspace &ws = sd.ws;
  if ((rc = check_species(d_species, N, S, ws.flag, st))) return rc;
  if ((rc = ws.A.ensure(sizeof(double) * ((size_t)N * p.n_A + 1))) ||
      (rc = ws.B2.ensure(sizeof(double) * ((size_t)N * nd + 1))) ||
      (rc = ws.norms.ensure(sizeof(double) * (N + 1))) ||
      (rc = ws.dB2.ensure(sizeof(double) * ((size_t)3 * P * nd + 1))) ||
      (rc = ws.fdots.ensure(sizeof(double) * (3 * P + 1))))
    return rc;
  if (N > 0 &&
      ((rc = launch_b2_forward(p, nl, d_species, ws.A.as<double>(),
                               ws.B2.as<double>(), ws.norms.as<double>(), st)) ||
       (rc = launch_b2_dervs(p, nl, d_species, ws.A.as<double>(),
                             ws.B2.as<double>(), ws.dB2.as<double>(),
                             ws.fdots.as<double>(), st))))
    return rc;
  std::vector<int> hs(N), perm, inv(N), srow, item_row;
  std::vector<double> hn(N);
  if (N > 0) {
    FGB_CUDA(cudaMemcpyAsync(hs.data(), d_species, sizeof(int) * N,
                             cudaMemcpyDeviceToHost, st));
    FGB_CUDA(cudaMemcpyAsync(hn.data(), ws.norms.p, sizeof(double) * N,
                             cudaMemcpyDeviceToHost, st));
    FGB_CUDA(cudaStreamSynchronize(st));
  }
  for (int s = 0; s < S; s++)
    for (int a = 0; a < N; a++)
      if (hs[a] == s) {
        inv[a] = (int)perm.size();
        item_row.push_back(hn[a] >= kEmptyThresh ? (int)perm.size() : -1);
        perm.push_back(a);
        srow.push_back(s);
      }
  if ((rc = sd.dperm.ensure(sizeof(int) * (N + 1))) ||
      (rc = sd.dinv.ensure(sizeof(int) * (N + 1))) ||
      (rc = sd.dsrow.ensure(sizeof(int) * (N + 1))) ||
      (rc = sd.U.ensure(sizeof(double) * ((size_t)N * nd + 1))) ||
      (rc = sd.W.ensure(sizeof(double) * ((size_t)N * 6 * nd + 1))) ||
      (rc = sd.dbase.ensure(sizeof(long long) * (N + 1))))
    return rc;
  sd.base.assign(N + 1, 0);
  if (N == 0) {
    sd.T = 0;
    return sd.item_row.ensure(sizeof(int));
  }
  FGB_CUDA(cudaMemcpyAsync(sd.dperm.p, perm.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(sd.dinv.p, inv.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(sd.dsrow.p, srow.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  k_dtc_rows<<<N, kDT, 0, st>>>(N, nd, sd.dperm.as<int>(), ws.B2.as<double>(),
                                ws.norms.as<double>(),
                                nl->offsets.as<long long>(),
                                nl->nbr_rel.as<double4_16a>(), ws.dB2.as<double>(),
                                sd.U.as<double>(), sd.W.as<double>());
  FGB_LAUNCH_CHECK("k_dtc_rows");
  DevBuf cnt;
  if ((rc = cnt.ensure(sizeof(int) * N))) return rc;
  k_dtc_slot_count<<<ceil_div(N, 128), 128, 0, st>>>(
      N, nl->offsets.as<long long>(), nl->nbr_j.as<int>(), cnt.as<int>());
  FGB_LAUNCH_CHECK("k_dtc_slot_count");
  std::vector<int> hc(N);
  FGB_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, sizeof(int) * N,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  for (int a = 0; a < N; a++) sd.base[a + 1] = sd.base[a] + hc[a];
  sd.T = sd.base[N];
  if ((rc = sd.srows.ensure(sizeof(int) * sd.T)) ||
      (rc = sd.G.ensure(sizeof(double) * (size_t)sd.T * 3 * nd)) ||
      (rc = sd.item_row.ensure(sizeof(int) * (N + sd.T))))
    return rc;
  FGB_CUDA(cudaMemcpyAsync(sd.dbase.p, sd.base.data(), sizeof(long long) * (N + 1),
                           cudaMemcpyHostToDevice, st));
  k_dtc_slots<<<N, kDT, 0, st>>>(
      0, N, nd, sd.dinv.as<int>(), ws.norms.as<double>(),
      nl->offsets.as<long long>(), nl->nbr_j.as<int>(),
      nl->nbr_twin.as<long long>(), ws.dB2.as<double>(), sd.U.as<double>(),
      sd.dbase.as<long long>(), sd.srows.as<int>(), sd.G.as<double>());
  FGB_LAUNCH_CHECK("k_dtc_slots");
  // items: atoms (sorted rows, -1 where empty), then slots
  FGB_CUDA(cudaMemcpyAsync(sd.item_row.p, item_row.data(), sizeof(int) * N,
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(sd.item_row.as<int>() + N, sd.srows.p,
                           sizeof(int) * sd.T, cudaMemcpyDeviceToDevice, st));
  return FGB_OK;
}

// Groups of one side: energy, atoms 0..N-1, stress halves.
std::vector<SsGroup> ss_groups(const SsSide &sd, int nd) {
  std::vector<SsGroup> g;
  const int N = sd.N;
  g.push_back({0, N, 0, 1, nullptr, 0, 0, 0, 1.0});
  for (int a = 0; a < N; a++)
    g.push_back({N + (int)sd.base[a], N + (int)sd.base[a + 1], N, 3,
                 sd.G.as<double>(), 3LL * nd, 0, 1 + 3LL * a, 1.0});
  for (int h = 0; h < 2; h++)
    g.push_back({0, N, 0, 3, sd.W.as<double>(), 6LL * nd, 3 * h,
                 1 + 3LL * N + 3 * h, 1.0 / sd.vol});
  return g;
}

template <int C1, int C2>
int ss_launch(const std::vector<std::pair<int, int>> &gps,
              const std::vector<SsGroup> &h1, const std::vector<SsGroup> &h2,
              const DevBuf &d1, const DevBuf &d2, const SsSide &s1,
              const SsSide &s2, int nd, double xi, double sig2, long long ncol,
              double *d_out, DevBuf &bad, cudaStream_t st) {
  constexpr long long kChunk = 2048;   // item pairs per work item
  std::vector<SsWork> work;
  std::vector<SsPair> pairs;
  for (const auto &gp : gps) {
    const long long n = (long long)(h1[gp.first].end - h1[gp.first].beg) *
                        (h2[gp.second].end - h2[gp.second].beg);
    SsPair pr{gp.first, gp.second, (int)work.size(), 0};
    for (long long p0 = 0; p0 < n; p0 += kChunk)
      work.push_back({gp.first, gp.second, p0, std::min(n, p0 + kChunk)});
    pr.w1 = (int)work.size();
    pairs.push_back(pr);
  }
  if (pairs.empty()) return FGB_OK;
  DevBuf dw, dp, part;
  int rc;
  if ((rc = dw.ensure(sizeof(SsWork) * (work.size() + 1))) ||
      (rc = dp.ensure(sizeof(SsPair) * pairs.size())) ||
      (rc = part.ensure(sizeof(double) * C1 * C2 * (work.size() + 1))))
    return rc;
  if (!work.empty())
    FGB_CUDA(cudaMemcpyAsync(dw.p, work.data(), sizeof(SsWork) * work.size(),
                             cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(dp.p, pairs.data(), sizeof(SsPair) * pairs.size(),
                           cudaMemcpyHostToDevice, st));
  if (!work.empty()) {
    k_ss<C1, C2><<<(unsigned)work.size(), kDT, 0, st>>>(
        dw.as<SsWork>(), d1.as<SsGroup>(), d2.as<SsGroup>(),
        s1.item_row.as<int>(), s2.item_row.as<int>(), s1.dsrow.as<int>(),
        s2.dsrow.as<int>(), s1.U.as<double>(), s2.U.as<double>(), nd, xi,
        part.as<double>(), bad.as<int>());
    FGB_LAUNCH_CHECK("k_ss");
  }
  const long long nt = (long long)pairs.size() * C1 * C2;
  k_ss_final<C1, C2><<<ceil_div(nt, 256), 256, 0, st>>>(
      (int)pairs.size(), dp.as<SsPair>(), d1.as<SsGroup>(), d2.as<SsGroup>(),
      part.as<double>(), sig2, ncol, d_out);
  FGB_LAUNCH_CHECK("k_ss_final");
  // the work lists are freed on return
  FGB_CUDA(cudaStreamSynchronize(st));
  return FGB_OK;
}

}  // namespace

int struc_struc_impl(const B2Params &p, double sigma, double power,
                     fgb_nlist_s *nl1, const int *d_species1,
                     fgb_nlist_s *nl2, const int *d_species2, double *d_out,
                     cudaStream_t st) {
  SsSide s1, s2;
  int rc;
  if ((rc = ss_prepare(p, nl1, d_species1, s1, st)) ||
      (rc = ss_prepare(p, nl2, d_species2, s2, st)))
    return rc;
  const int nd = p.n_d;
  const long long nrow = 1 + 3LL * s1.N + 6, ncol = 1 + 3LL * s2.N + 6;
  FGB_CUDA(cudaMemsetAsync(d_out, 0, sizeof(double) * nrow * ncol, st));
  const std::vector<SsGroup> h1 = ss_groups(s1, nd), h2 = ss_groups(s2, nd);
  DevBuf d1, d2, bad;
  if ((rc = d1.ensure(sizeof(SsGroup) * h1.size())) ||
      (rc = d2.ensure(sizeof(SsGroup) * h2.size())) ||
      (rc = bad.ensure(sizeof(int))))
    return rc;
  FGB_CUDA(cudaMemcpyAsync(d1.p, h1.data(), sizeof(SsGroup) * h1.size(),
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemcpyAsync(d2.p, h2.data(), sizeof(SsGroup) * h2.size(),
                           cudaMemcpyHostToDevice, st));
  FGB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  // group pairs by component counts (energy groups have one component)
  std::vector<std::pair<int, int>> gp11, gp13, gp31, gp33;
  for (int a = 0; a < (int)h1.size(); a++)
    for (int b = 0; b < (int)h2.size(); b++) {
      const int c1 = h1[a].C, c2 = h2[b].C;
      (c1 == 1 ? (c2 == 1 ? gp11 : gp13) : (c2 == 1 ? gp31 : gp33))
          .push_back({a, b});
    }
  const double sig2 = sigma * sigma;
  if ((rc = ss_launch<1, 1>(gp11, h1, h2, d1, d2, s1, s2, nd, power, sig2, ncol,
                            d_out, bad, st)))
    return rc;
  int hbad = 0;
  FGB_CUDA(cudaMemcpy(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (hbad) {
    set_error("Dot product of descriptors is 0, and the negative power "
              "function in force-force kernel diverges.");
    return FGB_EINVAL;
  }
  if ((rc = ss_launch<1, 3>(gp13, h1, h2, d1, d2, s1, s2, nd, power, sig2, ncol,
                            d_out, bad, st)) ||
      (rc = ss_launch<3, 1>(gp31, h1, h2, d1, d2, s1, s2, nd, power, sig2, ncol,
                            d_out, bad, st)) ||
      (rc = ss_launch<3, 3>(gp33, h1, h2, d1, d2, s1, s2, nd, power, sig2, ncol,
                            d_out, bad, st)))
    return rc;
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_self_kernel_struc(fgb_b2_t b2, double sigma, double power,
                                     fgb_nlist_t nl, const int *d_species,
                                     double *d_out, void *stream) {
  if (!b2 || !nl || !d_species || !d_out) {
    set_error("fgb_self_kernel_struc: invalid arguments");
    return FGB_EINVAL;
  }
  fgb_workspace ws;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = self_kernel_impl(b2->p, sigma, power, nl, d_species, d_out, ws,
                                 st, false);
  if (!rc) FGB_CUDA(cudaStreamSynchronize(st));
  return rc;
}

extern "C" int fgb_struc_struc(fgb_b2_t b2, double sigma, double power,
                               fgb_nlist_t nl1, const int *d_species1,
                               fgb_nlist_t nl2, const int *d_species2,
                               double *d_out, void *stream) {
  if (!b2 || !nl1 || !nl2 || !d_out) {
    set_error("fgb_struc_struc: invalid arguments");
    return FGB_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc = struc_struc_impl(b2->p, sigma, power, nl1, d_species1, nl2,
                            d_species2, d_out, st);
  if (!rc) FGB_CUDA(cudaStreamSynchronize(st));
  return rc;
}
