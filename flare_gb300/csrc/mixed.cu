// Mixed-precision kernel stage.
//
// Energy and local variance need FP64-level accuracy: the sparse-set sum and
// sigma^2 - |L_inv k|^2 cancel too many digits for any 24-bit arithmetic.
// They come from the kernel GEMM and the variance GEMM run on the BF16 tensor
// cores with exact integer slicing (ozaki.cu, FP64-accurate).  The forces,
// which only need 1e-4 eV/A, use the alpha-weighted sum folded into the
// sparse set before the GEMM:
//   power 2:  E_i = sigma^2 d^_i^T B_s d^_i,  B_s = S^_s^T diag(alpha_s) S^_s
//             dE/dd^ = 2 sigma^2 B_s d^   (one GEMM, n_d x n_d per species)
//   power 1:  E_i = sigma^2 beta_s . d^_i,  beta_s = S^_s^T alpha_s
// B_s / beta_s are built once per model in FP64 on the GPU; B_s is kept in
// FP32-level exact slices for the tensor-core GEMM Y = D^ B_s (ozaki.cu, 4
// slices, 10 pair products, exact accumulation) and beta_s in FP32.
// dE/dB2 = (dE/dd^ - (d^ . dE/dd^) d^) / |d| in FP32; the per-pair adjoint
// then runs in FP32.  Other powers use the FP64 kernel, adjoint and variance
// GEMMs.
#include <cstring>
#include <type_traits>

#include "fgb_df.cuh"
#include "fgb_internal.h"
#include "fgb_kernels.h"
#include "fgb_model.h"
#include "fgb_ozaki.h"
#include "fgb_gemm64.cuh"
#include "fgb_profile.h"
#include "fgb_tune.h"

namespace fgb {
namespace {
using namespace gemm64;


// S^T (M x nd) -> ST (nd x M) scaled by alpha*valid (for B = S^T diag(a) S)
__global__ void k_scaled_transpose(int M, int nd, const double *__restrict__ S,
                                   const double *__restrict__ alpha,
                                   const unsigned char *__restrict__ valid,
                                   double *__restrict__ ST,
                                   double *__restrict__ STa) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)M * nd) return;
  int t = (int)(idx / nd), q = (int)(idx % nd);
  double v = S[idx];
  ST[(long long)q * M + t] = v;
  STa[(long long)q * M + t] = valid[t] ? v * alpha[t] : 0.0;
}

// B = ST STa^T (nd x nd), written as FP32 and as FP64.
__global__ void __launch_bounds__(GT)
k_fold_gemm(int nd, int M, const double *__restrict__ ST,
            const double *__restrict__ STa, float *__restrict__ B,
            double *__restrict__ Bd) {
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  double acc[4][4];
  gemm_mainloop<true>(acc, m0, n0, nd, nd, M, ST, M, nullptr, STa, M);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int m = m0 + ty + 16 * i;
    if (m >= nd) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int n = n0 + tx + 16 * j;
      if (n < nd) {
        B[(long long)m * nd + n] = (float)acc[i][j];
        Bd[(long long)m * nd + n] = acc[i][j];
      }
    }
  }
}

// beta = S^T (alpha * valid), FP64 output
__global__ void k_fold_vec64(int M, int nd, const double *__restrict__ S,
                             const double *__restrict__ alpha,
                             const unsigned char *__restrict__ valid,
                             double *__restrict__ beta) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nd) return;
  double acc = 0.0;
  for (int t = 0; t < M; t++)
    if (valid[t]) acc += alpha[t] * S[(long long)t * nd + q];
  beta[q] = acc;
}

// beta = S^T (alpha * valid), FP32 output
__global__ void k_fold_vec(int M, int nd, const double *__restrict__ S,
                           const double *__restrict__ alpha,
                           const unsigned char *__restrict__ valid,
                           float *__restrict__ beta) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nd) return;
  double acc = 0.0;
  for (int t = 0; t < M; t++)
    if (valid[t]) acc += alpha[t] * S[(long long)t * nd + q];
  beta[q] = (float)acc;
}

// dE/dB2 rows from g = dE/dd^ (power 2: g = 2 sig2 Y; power 1: g = sig2 beta)
// warp per row: d^ = B2 / |d| in FP32 (mantissa cut, no FP64 arithmetic),
// q = d^ . g, dE/dB2 = (g - q d^) / |d|, written in FP32 for the FP32
// adjoint.
__global__ void k_mapped_grad(int Mr, int nd, const int *__restrict__ perm,
                              const double *__restrict__ norms,
                              const double *__restrict__ B2,
                              const float *__restrict__ Y,
                              const float *__restrict__ beta, float scale,
                              float *__restrict__ gB2) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= Mr) return;
  const int atom = perm[warp];
  const double n = norms[atom];
  const bool ok = n >= kEmptyThresh;
  const float inv = ok ? __frcp_rn(trunc_float(n)) : 0.f;
  const double *b = B2 + (long long)atom * nd;
  const float *y = Y ? Y + (long long)warp * nd : nullptr;
  float q = 0.f;
  for (int k = lane; k < nd; k += 32)
    q = __fmaf_rn(trunc_float(b[k]) * inv, y ? y[k] : beta[k], q);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) q += __shfl_xor_sync(0xffffffffu, q, off);
  for (int k = lane; k < nd; k += 32) {
    const float d = trunc_float(b[k]) * inv;
    const float g = scale * (y ? y[k] : beta[k]);
    gB2[(long long)atom * nd + k] = (g - scale * q * d) * inv;
  }
}

// The same for power 2 with rows of n_d = 4 t <= 1024 values: a lane takes
// four consecutive columns at a time (two double2 loads of B2, one float4
// of Y, one float4 store), keeps d^ and g in registers between the dot
// product and the update, and the row's bytes are read once.
// IT: 4-column groups per lane, ceil(n_d / 128) (the row's registers)
constexpr int kGradV4It = 8;   // 8 x 32 lanes x 4 columns = 1024
template <int IT>
__global__ void __launch_bounds__(256)
k_mapped_grad_v4(int Mr, int nd, const int *__restrict__ perm,
                 const double *__restrict__ norms,
                 const double *__restrict__ B2, const float *__restrict__ Y,
                 float scale, float *__restrict__ gB2) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= Mr) return;
  const int atom = perm[warp];
  const double n = norms[atom];
  const bool ok = n >= kEmptyThresh;
  const float inv = ok ? __frcp_rn(trunc_float(n)) : 0.f;
  const int n4 = nd >> 2;
  const double2 *b = reinterpret_cast<const double2 *>(B2 + (long long)atom * nd);
  const float4 *y = reinterpret_cast<const float4 *>(Y + (long long)warp * nd);
  float4 dv[IT], yv[IT];
  float q = 0.f;
#pragma unroll
  for (int it = 0; it < IT; it++) {
    const int k4 = lane + 32 * it;
    if (k4 < n4) {
      const double2 b0 = b[2 * k4], b1 = b[2 * k4 + 1];
      dv[it] = make_float4(trunc_float(b0.x) * inv, trunc_float(b0.y) * inv,
                           trunc_float(b1.x) * inv, trunc_float(b1.y) * inv);
      yv[it] = y[k4];
      q = __fmaf_rn(dv[it].x, yv[it].x, q);
      q = __fmaf_rn(dv[it].y, yv[it].y, q);
      q = __fmaf_rn(dv[it].z, yv[it].z, q);
      q = __fmaf_rn(dv[it].w, yv[it].w, q);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) q += __shfl_xor_sync(0xffffffffu, q, off);
  const float sq = scale * q;
  float4 *out = reinterpret_cast<float4 *>(gB2 + (long long)atom * nd);
#pragma unroll
  for (int it = 0; it < IT; it++) {
    const int k4 = lane + 32 * it;
    if (k4 < n4)
      out[k4] = make_float4((scale * yv[it].x - sq * dv[it].x) * inv,
                            (scale * yv[it].y - sq * dv[it].y) * inv,
                            (scale * yv[it].z - sq * dv[it].z) * inv,
                            (scale * yv[it].w - sq * dv[it].w) * inv);
  }
}

// The same in FP64, for the guarded path (large folded coefficients):
// Y = D^ B_s from the FP64-level product, or the FP64 fold vector.
__global__ void k_mapped_grad64(int Mr, int nd, const int *__restrict__ perm,
                                const double *__restrict__ norms,
                                const double *__restrict__ B2,
                                const double *__restrict__ Y,
                                const double *__restrict__ beta, double scale,
                                double *__restrict__ gB2) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= Mr) return;
  const int atom = perm[warp];
  const double n = norms[atom];
  const bool ok = n >= kEmptyThresh;
  const double inv = ok ? 1.0 / n : 0.0;
  const double *b = B2 + (long long)atom * nd;
  const double *y = Y ? Y + (long long)warp * nd : nullptr;
  double q = 0.0;
  for (int k = lane; k < nd; k += 32) q += (b[k] * inv) * (y ? y[k] : beta[k]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) q += __shfl_xor_sync(0xffffffffu, q, off);
  for (int k = lane; k < nd; k += 32) {
    const double g = scale * (y ? y[k] : beta[k]);
    gB2[(long long)atom * nd + k] = (g - scale * q * (b[k] * inv)) * inv;
  }
}

// Largest |x| over n doubles into *out (bits of non-negative doubles order
// as integers; *out zeroed by the caller).
__global__ void k_max_abs(long long n, const double *__restrict__ x,
                          unsigned long long *__restrict__ out) {
  unsigned long long mb = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    mb = max(mb, (unsigned long long)__double_as_longlong(x[i]) &
                     0x7FFFFFFFFFFFFFFFULL);
  for (int off = 16; off > 0; off >>= 1)
    mb = max(mb, (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)mb, off));
  if ((threadIdx.x & 31) == 0) atomicMax(out, mb);
}

}  // namespace

// FP32-level slices of the folded matrices for B tiles of set `set`.
static int build_fold_slices(fgb_model_s *m, int set, cudaStream_t st) {
  const int nd = m->b2.n_d, S = m->b2.n_species;
  m->ozB[set].clear();
  int rc;
  for (int s = 0; s < S; s++) {
    m->ozB[set].emplace_back(new oz::Sliced());
    if (m->h_counts[s] == 0) continue;
    // B_s is symmetric: its rows are the B operand of Y = D^ B_s
    if ((rc = oz::slice({nd, nd, oz::kTNF32set[set],
                         m->Bfold.as<double>() + (size_t)s * nd * nd, nd,
                         nullptr, nullptr},
                        *m->ozB[set][s], st, oz::kSF32)))
      return rc;
  }
  m->ozB_ready[set] = true;
  return FGB_OK;
}

static int build_fold(fgb_model_s *m, cudaStream_t st) {
  const B2Params &p = m->b2;
  const int nd = p.n_d, S = p.n_species;
  const bool quad = m->power == 2.0;
  size_t per = quad ? (size_t)nd * nd : (size_t)nd;
  int rc;
  if ((rc = m->Bmap.ensure(sizeof(float) * (per * S + 1)))) return rc;
  FGB_CUDA(cudaMemsetAsync(m->Bmap.p, 0, sizeof(float) * per * S, st));
  if ((rc = m->Bfold.ensure(sizeof(double) * (per * S + 1)))) return rc;
  FGB_CUDA(cudaMemsetAsync(m->Bfold.p, 0, sizeof(double) * per * S, st));
  DevBuf ST, STa;
  for (bool &r : m->ozB_ready) r = false;
  for (int s = 0; s < S; s++) {
    const int Ms = m->h_counts[s], c = m->h_offsets[s];
    if (Ms == 0) continue;
    const double *Ss = m->S.as<double>() + (size_t)c * nd;
    float *Bs = m->Bmap.as<float>() + per * s;
    if (quad) {
      if ((rc = ST.ensure(sizeof(double) * (size_t)Ms * nd)) ||
          (rc = STa.ensure(sizeof(double) * (size_t)Ms * nd)))
        return rc;
      k_scaled_transpose<<<ceil_div((long long)Ms * nd, 256), 256, 0, st>>>(
          Ms, nd, Ss, m->alpha.as<double>() + c,
          m->svalid.as<unsigned char>() + c, ST.as<double>(), STa.as<double>());
      FGB_LAUNCH_CHECK("k_scaled_transpose");
      dim3 g(ceil_div(nd, BN), ceil_div(nd, BM));
      k_fold_gemm<<<g, GT, 0, st>>>(nd, Ms, ST.as<double>(), STa.as<double>(),
                                    Bs, m->Bfold.as<double>() + per * s);
      FGB_LAUNCH_CHECK("k_fold_gemm");
      FGB_CUDA(cudaStreamSynchronize(st));   // ST/STa reused next species
    } else {
      k_fold_vec<<<ceil_div(nd, 128), 128, 0, st>>>(
          Ms, nd, Ss, m->alpha.as<double>() + c,
          m->svalid.as<unsigned char>() + c, Bs);
      FGB_LAUNCH_CHECK("k_fold_vec");
      k_fold_vec64<<<ceil_div(nd, 128), 128, 0, st>>>(
          Ms, nd, Ss, m->alpha.as<double>() + c,
          m->svalid.as<unsigned char>() + c,
          m->Bfold.as<double>() + per * s);
      FGB_LAUNCH_CHECK("k_fold_vec64");
    }
  }
  // Guard: the FP32-level force stage errs by about 2.5e-7 eV/A per unit
  // of the largest folded coefficient sigma^2 |sum alpha s^ s^T| (measured
  // over models with coefficients from 7.5 to 9e6); above kFoldMaxF32 the
  // force product, the gradient and the adjoint run at FP64 level instead.
  DevBuf mx;
  if ((rc = mx.ensure(sizeof(unsigned long long)))) return rc;
  FGB_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), st));
  k_max_abs<<<256, 256, 0, st>>>((long long)per * S, m->Bfold.as<double>(),
                                 mx.as<unsigned long long>());
  FGB_LAUNCH_CHECK("k_max_abs");
  unsigned long long hb = 0;
  FGB_CUDA(cudaMemcpyAsync(&hb, mx.p, sizeof(hb), cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  double bmax;
  std::memcpy(&bmax, &hb, sizeof(bmax));
  m->fold_max = bmax * m->sigma * m->sigma;
  m->force_f64 = m->fold_max > kFoldMaxF32;
  if (quad) {
    if (m->force_f64) {
      // B_s rows in FP64-level slices (B tiles of kTN rows)
      m->ozB64.clear();
      for (int s = 0; s < S; s++) {
        m->ozB64.emplace_back(new oz::Sliced());
        if (m->h_counts[s] == 0) continue;
        if ((rc = oz::slice({nd, nd, oz::kTN, m->Bfold.as<double>() + per * s,
                             nd, nullptr, nullptr},
                            *m->ozB64[s], st)))
          return rc;
      }
    } else if ((rc = build_fold_slices(m, 0, st))) {
      return rc;
    }
  }
  FGB_CUDA(cudaStreamSynchronize(st));
  m->bmap_ready = true;
  return FGB_OK;
}

int prepare_mixed(fgb_model_s *m, cudaStream_t st) {
  if (m->power != 2.0 && m->power != 1.0) return FGB_OK;   // FP64 stages
  int rc;
  if (!m->bmap_ready && (rc = build_fold(m, st))) return rc;
  if (!m->slices_chosen && (rc = choose_kernel_slices(m, st))) return rc;
  return FGB_OK;
}

int kernel_stage_mixed(fgb_model_s *m, int N, const std::vector<int> &counts,
                       bool want_grad, bool want_var, double *d_e_atom,
                       double *d_gB2, double *d_var, cudaStream_t st,
                       bool fixed) {
  const bool foldable = m->power == 2.0 || m->power == 1.0;
  int rc;
  if (!foldable)   // powers other than 1 and 2: FP64 kernel, adjoint, variance
    return kernel_stage_fp64(m, N, counts, want_grad, want_var, d_e_atom,
                             d_gB2, d_var, st);
  if (want_grad && !m->bmap_ready) {
    if (fixed) {
      set_error("mixed force stage: folded matrices not built before a fixed call");
      return FGB_EINVAL;
    }
    if ((rc = build_fold(m, st))) return rc;
  }
  const B2Params &p = m->b2;
  const int nd = p.n_d;
  const bool quad = m->power == 2.0;
  const float sig2 = (float)(m->sigma * m->sigma);
  const size_t per = quad ? (size_t)nd * nd : (size_t)nd;
  if (quad && (rc = m->ws.ozerr.ensure(sizeof(int)))) return rc;
  // Forces of one row chunk, right after its kernel and variance GEMMs: the
  // FP32-level operand is the first four of the rows' nine slices (their
  // most significant digits, within half a unit of the 24-bit rounding),
  // read in place from ws.ozA.
  const ChunkHook forces = [&](int s, int Mr, const int *perm) -> int {
    int r;
    if (m->force_f64) {
      // large folded coefficients: FP64-level product and FP64 gradient
      if (quad && (r = m->ws.kmat.ensure(sizeof(double) * (size_t)Mr * nd)))
        return r;
      StageTimer _pt(kStMappedGemm, st, quad ? 2 : 1);
      if (quad && (r = oz::gemm_store(m->ws.ozA, *m->ozB64[s],
                                      m->ws.kmat.as<double>(), nd,
                                      m->ws.ozerr.as<int>(), st)))
        return r;
      k_mapped_grad64<<<ceil_div((long long)Mr * 32, 256), 256, 0, st>>>(
          Mr, nd, perm, m->ws.norms.as<double>(), m->ws.B2.as<double>(),
          quad ? m->ws.kmat.as<double>() : nullptr,
          quad ? nullptr : m->Bfold.as<double>() + per * s,
          quad ? 2.0 * m->sigma * m->sigma : m->sigma * m->sigma, d_gB2);
      FGB_LAUNCH_CHECK("k_mapped_grad64");
      return FGB_OK;
    }
    if (quad && (r = m->ws.yf.ensure(sizeof(float) * (size_t)Mr * nd)))
      return r;
    StageTimer _pt(kStMappedGemm, st, quad ? 2 : 1);
    if (quad) {
      // Y = D^ B_s on the tensor cores (FP32-level exact slices)
      auto usable = [m](int v) { return m->ozB_ready[oz::f32_set(v)]; };
      auto launch = [&](int v) -> int {
        const int set = oz::f32_set(v);
        int q;
        if (!m->ozB_ready[set]) {
          if (fixed) {
            set_error("mixed force stage: tile variant not prepared");
            return FGB_EINVAL;
          }
          if ((q = build_fold_slices(m, set, st))) return q;
        }
        return oz::gemm_f32(m->ws.ozA, *m->ozB[set][s], m->ws.yf.as<float>(),
                            nd, m->ws.ozerr.as<int>(), st, oz::kEWF32v[v]);
      };
      int v = 0;
      if ((r = tune::run(tune::kOpForceGemm, Mr, nd, nd, oz::kF32Variants,
                         launch, usable, st, fixed, &v)))
        return r;
    }
    if (quad && nd % 4 == 0 && nd <= 4 * 32 * kGradV4It) {
      const unsigned nb = (unsigned)ceil_div((long long)Mr * 32, 256);
      const auto go = [&](auto it) {
        k_mapped_grad_v4<decltype(it)::value><<<nb, 256, 0, st>>>(
            Mr, nd, perm, m->ws.norms.as<double>(), m->ws.B2.as<double>(),
            m->ws.yf.as<float>(), 2.f * sig2,
            reinterpret_cast<float *>(d_gB2));
      };
      switch ((nd + 127) / 128) {   // 4-column groups per lane
        case 1: go(std::integral_constant<int, 1>()); break;
        case 2: go(std::integral_constant<int, 2>()); break;
        case 3: go(std::integral_constant<int, 3>()); break;
        case 4: go(std::integral_constant<int, 4>()); break;
        case 5: go(std::integral_constant<int, 5>()); break;
        case 6: go(std::integral_constant<int, 6>()); break;
        case 7: go(std::integral_constant<int, 7>()); break;
        default: go(std::integral_constant<int, kGradV4It>()); break;
      }
      FGB_LAUNCH_CHECK("k_mapped_grad_v4");
    } else {
      k_mapped_grad<<<ceil_div((long long)Mr * 32, 256), 256, 0, st>>>(
          Mr, nd, perm, m->ws.norms.as<double>(), m->ws.B2.as<double>(),
          quad ? m->ws.yf.as<float>() : nullptr,
          quad ? nullptr : m->Bmap.as<float>() + per * s,
          quad ? 2.f * sig2 : sig2, reinterpret_cast<float *>(d_gB2));
      FGB_LAUNCH_CHECK("k_mapped_grad");
    }
    return FGB_OK;
  };
  // Kernel and variance GEMMs on the tensor cores, FP64-accurate by exact
  // integer slicing (ozaki.cu); species with no sparse environments keep
  // zero energy gradients.
  return kernel_stage_oz(m, N, counts, false, want_var, d_e_atom, d_var, st,
                         fixed, want_grad ? &forces : nullptr);
}

}  // namespace fgb

using namespace fgb;

// Mapping coefficients of a solved power-1 or power-2 model
// (normalized_dot_product.cpp:653-767): per species s,
//   power 2: sigma^2 sum_t alpha_t s^_t s^_t^T   (n_d x n_d, row-major)
//   power 1: sigma^2 sum_t alpha_t s^_t          (n_d)
// over the valid sparse environments of the species (s^ = s / |s|), in
// FP64 on the device.
extern "C" int fgb_model_fold_guard(fgb_model_t m, double *h_fold_max,
                                    int *h_fp64_forces, void *stream) {
  if (!m || (m->power != 1.0 && m->power != 2.0)) {
    set_error("fgb_model_fold_guard: invalid arguments (power 1 or 2 models)");
    return FGB_EINVAL;
  }
  if (!m->solved) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  int rc;
  if (!m->bmap_ready && (rc = build_fold(m, (cudaStream_t)stream))) return rc;
  if (h_fold_max) *h_fold_max = m->fold_max;
  if (h_fp64_forces) *h_fp64_forces = m->force_f64 ? 1 : 0;
  return FGB_OK;
}

extern "C" int fgb_model_mixed_plan(fgb_model_t m, int *h_kernel_slices,
                                    double *h_slice_err_est, double *h_fold_max,
                                    int *h_fp64_forces, void *stream) {
  if (!m) {
    set_error("fgb_model_mixed_plan: invalid arguments");
    return FGB_EINVAL;
  }
  if (!m->solved) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  int rc;
  if ((rc = prepare_mixed(m, (cudaStream_t)stream))) return rc;
  if (h_kernel_slices) *h_kernel_slices = m->oz_S;
  if (h_slice_err_est) *h_slice_err_est = m->oz_err_est;
  if (h_fold_max) *h_fold_max = m->fold_max;
  if (h_fp64_forces) *h_fp64_forces = m->force_f64 ? 1 : 0;
  return FGB_OK;
}

extern "C" int fgb_model_slice_plan(fgb_model_t m, int *h_kernel_slices,
                                    int *h_variance_slices,
                                    double *h_energy_err_est,
                                    double *h_var_err_est, void *stream) {
  if (!m) {
    set_error("fgb_model_slice_plan: invalid arguments");
    return FGB_EINVAL;
  }
  if (!m->solved) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  int rc;
  if ((rc = prepare_mixed(m, (cudaStream_t)stream))) return rc;
  if (h_kernel_slices) *h_kernel_slices = m->oz_S;
  if (h_variance_slices) *h_variance_slices = m->oz_Sv;
  if (h_energy_err_est) *h_energy_err_est = m->oz_err_est;
  if (h_var_err_est) *h_var_err_est = m->oz_var_err_est;
  return FGB_OK;
}

extern "C" int fgb_model_set_slices(fgb_model_t m, int kernel_slices,
                                    int variance_slices) {
  if (!m || !(kernel_slices == 0 || (kernel_slices >= oz::kMinKernelSlices &&
                                     kernel_slices <= oz::kS)) ||
      !(variance_slices == 0 ||
        (variance_slices >= oz::kMinVarianceSlices &&
         variance_slices <= oz::kS))) {
    set_error("fgb_model_set_slices: kernel slices must be 0 (chosen) or "
              "%d..%d, variance slices 0 or %d..%d", oz::kMinKernelSlices,
              oz::kS, oz::kMinVarianceSlices, oz::kS);
    return FGB_EINVAL;
  }
  m->oz_S_forced = kernel_slices;
  m->oz_Sv_forced = variance_slices;
  m->slices_chosen = false;   // chosen again before the next mixed call
  return FGB_OK;
}

extern "C" int fgb_model_mapping(fgb_model_t m, double *h_beta, void *stream) {
  if (!m || !h_beta || (m->power != 1.0 && m->power != 2.0)) {
    set_error("fgb_model_mapping: invalid arguments (power 1 or 2 models)");
    return FGB_EINVAL;
  }
  if (!m->solved) {
    set_error("L_inv must be up to date to make predictions. Please call "
              "update_matrices_QR and try again.");
    return FGB_ESTALE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int S = m->b2.n_species, nd = m->b2.n_d;
  const bool quad = m->power == 2.0;
  const size_t per = quad ? (size_t)nd * nd : (size_t)nd;
  const double sig2 = m->sigma * m->sigma;
  DevBuf out, ST, STa, Bf;
  int rc;
  if ((rc = out.ensure(sizeof(double) * per * S)) ||
      (quad && (rc = Bf.ensure(sizeof(float) * per))))
    return rc;
  FGB_CUDA(cudaMemsetAsync(out.p, 0, sizeof(double) * per * S, st));
  for (int s = 0; s < S; s++) {
    const int Ms = m->h_counts[s], c = m->h_offsets[s];
    if (Ms == 0) continue;
    const double *Ss = m->S.as<double>() + (size_t)c * nd;
    double *dst = out.as<double>() + per * s;
    if (quad) {
      if ((rc = ST.ensure(sizeof(double) * (size_t)Ms * nd)) ||
          (rc = STa.ensure(sizeof(double) * (size_t)Ms * nd)))
        return rc;
      k_scaled_transpose<<<ceil_div((long long)Ms * nd, 256), 256, 0, st>>>(
          Ms, nd, Ss, m->alpha.as<double>() + c,
          m->svalid.as<unsigned char>() + c, ST.as<double>(), STa.as<double>());
      FGB_LAUNCH_CHECK("k_scaled_transpose");
      dim3 g(ceil_div(nd, BN), ceil_div(nd, BM));
      k_fold_gemm<<<g, GT, 0, st>>>(nd, Ms, ST.as<double>(), STa.as<double>(),
                                    Bf.as<float>(), dst);
      FGB_LAUNCH_CHECK("k_fold_gemm");
      FGB_CUDA(cudaStreamSynchronize(st));   // ST/STa reused next species
    } else {
      k_fold_vec64<<<ceil_div(nd, 128), 128, 0, st>>>(
          Ms, nd, Ss, m->alpha.as<double>() + c,
          m->svalid.as<unsigned char>() + c, dst);
      FGB_LAUNCH_CHECK("k_fold_vec64");
    }
  }
  FGB_CUDA(cudaMemcpyAsync(h_beta, out.p, sizeof(double) * per * S,
                           cudaMemcpyDeviceToHost, st));
  FGB_CUDA(cudaStreamSynchronize(st));
  for (size_t i = 0; i < per * S; i++) h_beta[i] *= sig2;
  return FGB_OK;
}
