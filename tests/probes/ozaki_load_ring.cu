// Measurement probe (not part of the library): the exact-slicing GEMM's
// shared-memory ring without its epilogue, on zero operands sized like the
// alloy kernel GEMM (128 A tiles x 21 B tiles, 43 chunks of 16).
// mode bit 0: issue the 13-span MMAs; bit 1: chunk-major operand layout
// (2 bulk copies per chunk) instead of slice-major (18 copies).
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../flare_gb300/csrc/fgb_tc.cuh"
using namespace fgb::tc;
constexpr int S = 9, TM = 128, TN = 48, KC = 16;
constexpr uint32_t TA = TM * KC * 2, TB = TN * KC * 2, ST = S * (TA + TB);

template <int A, int B0, int NB>
__device__ __forceinline__ void span(uint32_t tmem, uint64_t ad0, uint64_t bd0, bool first) {
  mma_bf16(tmem + (A + B0) * 48, ad0 + ((A * TA) >> 4), bd0 + ((B0 * TB) >> 4),
           idesc_bf16_f32(128, NB * 48), (A == 0 && first) ? 0u : 1u);
}
__device__ __forceinline__ void kstep(uint32_t tmem, uint64_t ad, uint64_t bd, bool f) {
  span<0,0,5>(tmem, ad, bd, f); span<0,5,4>(tmem, ad, bd, f);
  span<1,0,4>(tmem, ad, bd, f); span<1,4,4>(tmem, ad, bd, f);
  span<2,0,4>(tmem, ad, bd, f); span<2,4,3>(tmem, ad, bd, f);
  span<3,0,3>(tmem, ad, bd, f); span<3,3,3>(tmem, ad, bd, f);
  span<4,0,5>(tmem, ad, bd, f); span<5,0,4>(tmem, ad, bd, f);
  span<6,0,3>(tmem, ad, bd, f); span<7,0,2>(tmem, ad, bd, f);
  span<8,0,1>(tmem, ad, bd, f);
}

template <int NST>
__global__ void __launch_bounds__(128, 1)
k_ring(int KCH, int MT, int NT, const unsigned char *Ag, const unsigned char *Bg, int mode, int *err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *bl = (uint64_t *)(smem + NST * ST);
  uint64_t *bm = bl + NST;
  uint32_t *slot = (uint32_t *)(bm + NST);
  const int nt = blockIdx.x, mt = blockIdx.y, warp = threadIdx.x >> 5;
  if (warp == 0) { tmem_alloc(slot, 512); tmem_relinquish(); }
  if (threadIdx.x == 0) {
    for (int b = 0; b < NST; b++) { mbar_init(&bl[b], 1); mbar_init(&bm[b], 1); }
    mbar_fence_init();
  }
  fence_before_sync(); __syncthreads(); fence_after_sync();
  const uint32_t tmem = *slot;
  const bool mma = mode & 1, cm = mode & 2;
  if (threadIdx.x == 0) {
    bool ok = true;
    auto load = [&](int c) {
      const int b = c % NST;
      unsigned char *st = smem + b * ST;
      mbar_expect_tx(&bl[b], ST);
      if (cm) {
        bulk_g2s(st, Ag + ((size_t)mt * KCH + c) * (S * TA), S * TA, &bl[b]);
        bulk_g2s(st + S * TA, Bg + ((size_t)nt * KCH + c) * (S * TB), S * TB, &bl[b]);
      } else {
        for (int a = 0; a < S; a++) {
          bulk_g2s(st + a * TA, Ag + ((size_t)(a * MT + mt) * KCH + c) * TA, TA, &bl[b]);
          bulk_g2s(st + S * TA + a * TB, Bg + ((size_t)(a * NT + nt) * KCH + c) * TB, TB, &bl[b]);
        }
      }
    };
    int issued = 0, done = 0;
    for (; issued < KCH && issued < NST - 1; issued++) load(issued);
    for (int c = 0; c < KCH; c++) {
      const int b = c % NST;
      if (!mbar_wait(&bl[b], (c / NST) & 1, 1LL << 22)) { ok = false; break; }
      fence_after_sync();
      if (mma) {
        uint32_t base = smem_u32(smem + b * ST);
        kstep(tmem, smem_desc(base, 128, 256), smem_desc(base + S * TA, 128, 256), c == 0);
      }
      mma_commit(&bm[b]);
      if (issued < KCH) {
        const int prev = issued - NST;
        if (prev >= 0) {
          if (!mbar_wait(&bm[prev % NST], (prev / NST) & 1, 1LL << 22)) { ok = false; break; }
          done = prev + 1;
        }
        load(issued); issued++;
      }
    }
    const int last = ok ? KCH : 0;
    for (int c = done; c < last; c++)
      if (!mbar_wait(&bm[c % NST], (c / NST) & 1, 1LL << 22)) { ok = false; break; }
    if (!ok) atomicExch(err, 1);
  }
  fence_before_sync(); __syncthreads(); fence_after_sync();
  if (warp == 0) tmem_dealloc(tmem, 512);
}

template <int NST>
void run(int KCH, int MT, int NT, const unsigned char *A, const unsigned char *B, int mode, int *err) {
  size_t sm = NST * ST + 256;
  cudaFuncSetAttribute(k_ring<NST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  dim3 g(NT, MT);
  for (int w = 0; w < 2; w++) k_ring<NST><<<g, 128, sm>>>(KCH, MT, NT, A, B, mode, err);
  cudaEventRecord(e0);
  const int reps = 5;
  for (int r = 0; r < reps; r++) k_ring<NST><<<g, 128, sm>>>(KCH, MT, NT, A, B, mode, err);
  cudaEventRecord(e1);
  cudaError_t ce = cudaEventSynchronize(e1);
  float ms; cudaEventElapsedTime(&ms, e0, e1); ms /= reps;
  int he = 0; cudaMemcpy(&he, err, 4, cudaMemcpyDeviceToHost);
  double ctas = (double)MT * NT, waves = ctas / 152.0;
  double cyc_per_chunk = ms * 1e-3 * 1.97e9 / waves / KCH;
  printf("stages=%d mma=%d chunk_major=%d: %.3f ms, %.0f cycles/chunk/CTA, L2->SM %.2f TB/s (err=%d cuda=%d)\n",
         NST, mode & 1, (mode >> 1) & 1, ms, cyc_per_chunk, ctas * KCH * ST / (ms * 1e-3) / 1e12, he, (int)ce);
}

int main() {
  const int KCH = 43, MT = 128, NT = 21;
  unsigned char *A, *B; int *err;
  size_t nA = (size_t)S * MT * KCH * TA, nB = (size_t)S * NT * KCH * TB;
  cudaMalloc(&A, nA); cudaMalloc(&B, nB); cudaMalloc(&err, 4);
  cudaMemset(A, 0, nA); cudaMemset(B, 0, nB); cudaMemset(err, 0, 4);
  for (int mode = 0; mode < 4; mode++) run<4>(KCH, MT, NT, A, B, mode, err);
  for (int mode = 0; mode < 4; mode++) run<3>(KCH, MT, NT, A, B, mode, err);
  for (int mode = 0; mode < 4; mode++) run<2>(KCH, MT, NT, A, B, mode, err);
  return 0;
}
