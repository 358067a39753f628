// Measurement probe (not part of the library): cycles per tcgen05.mma
// (M = 128, K = 16, BF16 -> FP32) against N, one CTA per SM, one thread
// issuing back-to-back MMAs on zero tiles in shared memory, bounded mbarrier
// wait; then the exact-slicing GEMM's k-step as 45 separate N = 48 MMAs and
// as the 13 stacked-N spans.  Prints one line per case.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../flare_gb300/csrc/fgb_tc.cuh"
using namespace fgb::tc;

template <int N>
__global__ void __launch_bounds__(128, 1) k_probe(int reps, int rotate, long long *out, int *err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  // A: 128x16 bf16 = 4096 B, B: Nx16 bf16 = N*32 B (zeros)
  unsigned char *A = smem, *B = smem + 4096;
  uint64_t *bar = (uint64_t *)(smem + 4096 + 256 * 32);
  uint32_t *slot = (uint32_t *)(bar + 1);
  for (int i = threadIdx.x; i < (4096 + 256 * 32) / 4; i += blockDim.x) ((uint32_t *)smem)[i] = 0;
  int warp = threadIdx.x >> 5;
  if (warp == 0) { tmem_alloc(slot, 512); tmem_relinquish(); }
  if (threadIdx.x == 0) { mbar_init(bar, 1); mbar_fence_init(); }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  fence_before_sync(); __syncthreads(); fence_after_sync();
  uint32_t tmem = *slot;
  if (threadIdx.x == 0) {
    const uint32_t idesc = idesc_bf16_f32(128, N);
    uint64_t ad = smem_desc(smem_u32(A), 128, 256);
    uint64_t bd = smem_desc(smem_u32(B), 128, 256);
    int ngroups = 512 / N; if (ngroups > 9) ngroups = 9;
    long long t0 = clock64();
    for (int r = 0; r < reps; r++) {
      int g = rotate ? (r % ngroups) : 0;
      mma_bf16(tmem + g * N, ad, bd, idesc, r >= ngroups ? 1u : 0u);
    }
    mma_commit(bar);
    long long t1 = clock64();
    bool ok = mbar_wait(bar, 0, 1LL << 22);
    long long t2 = clock64();
    if (!ok) atomicExch(err, 1);
    out[2 * blockIdx.x] = t1 - t0;
    out[2 * blockIdx.x + 1] = t2 - t0;
  }
  fence_before_sync(); __syncthreads(); fence_after_sync();
  if (warp == 0) tmem_dealloc(tmem, 512);
}

template <int N>
void run(int reps, int rotate) {
  long long *d; int *e; cudaMalloc(&d, 2 * 152 * 8); cudaMalloc(&e, 4); cudaMemset(e, 0, 4);
  size_t sm = 4096 + 256 * 32 + 64;
  cudaFuncSetAttribute(k_probe<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_probe<N><<<152, 128, sm>>>(reps, rotate, d, e);
  cudaError_t err = cudaDeviceSynchronize();
  long long h[2 * 152]; int he = 0;
  cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost); cudaMemcpy(&he, e, 4, cudaMemcpyDeviceToHost);
  double issue = 0, total = 0;
  for (int i = 0; i < 152; i++) { issue += h[2 * i]; total += h[2 * i + 1]; }
  issue /= 152; total /= 152;
  double flop = 2.0 * 128 * N * 16 * reps;
  printf("N=%3d rotate=%d reps=%d: issue %.1f cyc/mma, complete %.1f cyc/mma, %.0f flop/cyc/SM (err=%d cuda=%d)\n",
         N, rotate, reps, issue / reps, total / reps, flop / total, he, (int)err);
  cudaFree(d); cudaFree(e);
}

// The 13-span plan of the exact-slicing GEMM on zero tiles: 9 A slices of
// 128x16, 9 B slices of 48x16 stacked, accumulators at (a+b0)*48.
template <int A, int B0, int NB>
__device__ __forceinline__ void span(uint32_t tmem, uint64_t ad0, uint64_t bd0, bool first) {
  mma_bf16(tmem + (A + B0) * 48, ad0 + ((A * 4096) >> 4), bd0 + ((B0 * 1536) >> 4),
           idesc_bf16_f32(128, NB * 48), (A == 0 && first) ? 0u : 1u);
}
__global__ void __launch_bounds__(128, 1) k_plan(int reps, int single, long long *out, int *err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int bytes = 9 * 4096 + 9 * 1536;
  uint64_t *bar = (uint64_t *)(smem + bytes);
  uint32_t *slot = (uint32_t *)(bar + 1);
  for (int i = threadIdx.x; i < bytes / 4; i += blockDim.x) ((uint32_t *)smem)[i] = 0;
  int warp = threadIdx.x >> 5;
  if (warp == 0) { tmem_alloc(slot, 512); tmem_relinquish(); }
  if (threadIdx.x == 0) { mbar_init(bar, 1); mbar_fence_init(); }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  fence_before_sync(); __syncthreads(); fence_after_sync();
  uint32_t tmem = *slot;
  if (threadIdx.x == 0) {
    uint64_t ad = smem_desc(smem_u32(smem), 128, 256);
    uint64_t bd = smem_desc(smem_u32(smem + 9 * 4096), 128, 256);
    long long t0 = clock64();
    for (int r = 0; r < reps; r++) {
      bool f = r == 0;
      if (single) {
        // old form: 45 N=48 MMAs
        for (int a = 0; a < 9; a++)
          for (int b = 0; a + b < 9; b++)
            mma_bf16(tmem + (a + b) * 48, ad + ((a * 4096) >> 4), bd + ((b * 1536) >> 4),
                     idesc_bf16_f32(128, 48), (a == 0 && f) ? 0u : 1u);
      } else {
        span<0,0,5>(tmem, ad, bd, f); span<0,5,4>(tmem, ad, bd, f);
        span<1,0,4>(tmem, ad, bd, f); span<1,4,4>(tmem, ad, bd, f);
        span<2,0,4>(tmem, ad, bd, f); span<2,4,3>(tmem, ad, bd, f);
        span<3,0,3>(tmem, ad, bd, f); span<3,3,3>(tmem, ad, bd, f);
        span<4,0,5>(tmem, ad, bd, f); span<5,0,4>(tmem, ad, bd, f);
        span<6,0,3>(tmem, ad, bd, f); span<7,0,2>(tmem, ad, bd, f);
        span<8,0,1>(tmem, ad, bd, f);
      }
    }
    mma_commit(bar);
    long long t1 = clock64();
    bool ok = mbar_wait(bar, 0, 1LL << 24);
    long long t2 = clock64();
    if (!ok) atomicExch(err, 1);
    out[2 * blockIdx.x] = t1 - t0;
    out[2 * blockIdx.x + 1] = t2 - t0;
  }
  fence_before_sync(); __syncthreads(); fence_after_sync();
  if (warp == 0) tmem_dealloc(tmem, 512);
}
void run_plan(int reps, int single) {
  long long *d; int *e; cudaMalloc(&d, 2 * 152 * 8); cudaMalloc(&e, 4); cudaMemset(e, 0, 4);
  size_t sm = 9 * 4096 + 9 * 1536 + 64;
  cudaFuncSetAttribute(k_plan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_plan<<<152, 128, sm>>>(reps, single, d, e);
  cudaError_t err = cudaDeviceSynchronize();
  long long h[2 * 152]; int he = 0;
  cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost); cudaMemcpy(&he, e, 4, cudaMemcpyDeviceToHost);
  double total = 0;
  for (int i = 0; i < 152; i++) total += h[2 * i + 1];
  total /= 152;
  double flop = 2.0 * 128 * 48 * 16 * 45 * reps;
  printf("plan %s: %.1f cyc per k-step, %.0f flop/cyc/SM (err=%d cuda=%d)\n",
         single ? "45 x N=48" : "13 spans", total / reps, flop / total, he, (int)err);
  cudaFree(d); cudaFree(e);
}

int main() {
  for (int rot = 0; rot < 2; rot++) {
    run<16>(2000, rot); run<32>(2000, rot); run<48>(2000, rot); run<64>(2000, rot);
    run<96>(2000, rot); run<128>(2000, rot); run<144>(2000, rot); run<192>(2000, rot);
    run<240>(2000, rot); run<256>(2000, rot);
  }
  run_plan(400, 1); run_plan(400, 0);
  return 0;
}
