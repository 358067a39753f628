// Measurement probe (not part of the library): cycles to drain 9 x 48 TMEM
// columns per lane with the exact-slicing epilogue's integer recombination
// (one wait per load, three loads per wait, loads alone).  TMEM content is
// whatever the allocation holds; the values only feed integer sums.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../flare_gb300/csrc/fgb_tc.cuh"
using namespace fgb::tc;

template <int MODE>
__global__ void __launch_bounds__(128, 1) k_drain(int reps, long long *out, long long *sink) {
  __shared__ uint32_t slot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) { tmem_alloc(&slot, 512); tmem_relinquish(); }
  fence_before_sync(); __syncthreads(); fence_after_sync();
  const uint32_t tmem = slot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  long long t0 = clock64();
  long long tot = 0;
  for (int r = 0; r < reps; r++) {
    for (int c0 = 0; c0 < 48; c0 += 16) {
      long long hi[16], lo[16];
#pragma unroll
      for (int j = 0; j < 16; j++) { hi[j] = 0; lo[j] = 0; }
      if (MODE == 0) {          // wait after every load (current epilogue)
#pragma unroll
        for (int g = 0; g < 9; g++) {
          uint32_t rr[16];
          tmem_ld16(trow + g * 48 + c0, rr);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; j++) {
            long long q = (long long)__float2int_rn(__uint_as_float(rr[j]) * 0.f + (float)(j + g));
            if (g < 5) hi[j] += q << (6 * (4 - g)); else lo[j] += q << (6 * (8 - g));
          }
        }
      } else if (MODE == 1) {   // three loads per wait
#pragma unroll
        for (int g0 = 0; g0 < 9; g0 += 3) {
          uint32_t a[16], b[16], c[16];
          tmem_ld16(trow + (g0 + 0) * 48 + c0, a);
          tmem_ld16(trow + (g0 + 1) * 48 + c0, b);
          tmem_ld16(trow + (g0 + 2) * 48 + c0, c);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; j++) {
            long long qa = (long long)__float2int_rn(__uint_as_float(a[j]) * 0.f + (float)j);
            long long qb = (long long)__float2int_rn(__uint_as_float(b[j]) * 0.f + (float)j);
            long long qc = (long long)__float2int_rn(__uint_as_float(c[j]) * 0.f + (float)j);
            const int g = g0;
            if (g < 5) hi[j] += qa << (6 * (4 - g)); else lo[j] += qa << (6 * (8 - g));
            if (g + 1 < 5) hi[j] += qb << (6 * (3 - g)); else lo[j] += qb << (6 * (7 - g));
            if (g + 2 < 5) hi[j] += qc << (6 * (2 - g)); else lo[j] += qc << (6 * (6 - g));
          }
        }
      } else {                  // loads only (no arithmetic), wait per load
#pragma unroll
        for (int g = 0; g < 9; g++) {
          uint32_t rr[16];
          tmem_ld16(trow + g * 48 + c0, rr);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; j++) hi[j] += rr[j];
        }
      }
#pragma unroll
      for (int j = 0; j < 16; j++) tot += hi[j] ^ lo[j];
    }
  }
  long long t1 = clock64();
  if (lane == 0) out[blockIdx.x * 4 + warp] = t1 - t0;
  sink[blockIdx.x * 128 + threadIdx.x] = tot;
  fence_before_sync(); __syncthreads(); fence_after_sync();
  if (warp == 0) tmem_dealloc(tmem, 512);
}

template <int MODE>
void run(int reps) {
  long long *d, *s; cudaMalloc(&d, 152 * 4 * 8); cudaMalloc(&s, 152 * 128 * 8);
  k_drain<MODE><<<152, 128>>>(reps, d, s);
  cudaError_t e = cudaDeviceSynchronize();
  long long h[152 * 4]; cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  double avg = 0; for (int i = 0; i < 152 * 4; i++) avg += h[i]; avg /= 152 * 4;
  printf("mode %d: %.0f cycles per 48-column drain (cuda=%d)\n", MODE, avg / reps, (int)e);
  cudaFree(d); cudaFree(s);
}

int main() { run<0>(200); run<1>(200); run<2>(200); return 0; }
