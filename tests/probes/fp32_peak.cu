// Measurement probe (not part of the library): FP32 FMA throughput of the
// SMs (the bound of the double-float descriptor stage) and the throughput
// of the double-float multiply-accumulate that stage uses (exact FP32
// product by FMA, TwoSum into the high word, low-order terms collected in
// the low word).  Independent chains per thread, a grid of 8 blocks per SM,
// timed with CUDA events.
#include <cstdio>
#include <cuda_runtime.h>

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_fma(int iters, float a, float b,
                                             float *out) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = threadIdx.x * 1e-3f + c;
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = __fmaf_rn(x[c], a, b);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

struct dfl {
  float hi, lo;
};

__device__ __forceinline__ void dfmac(dfl &acc, dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float pe = __fmaf_rn(a.hi, b.hi, -p);
  pe = __fmaf_rn(a.hi, b.lo, pe);
  pe = __fmaf_rn(a.lo, b.hi, pe);
  const float s = __fadd_rn(acc.hi, p);
  const float bb = __fsub_rn(s, acc.hi);
  const float e = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)),
                            __fsub_rn(p, bb));
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, pe));
}

__global__ void __launch_bounds__(256) k_dfmac(int iters, float a, float b,
                                               float *out) {
  dfl x[kChains];
  const dfl u{a, a * 1e-8f}, v{b, b * 1e-8f};
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = dfl{threadIdx.x * 1e-3f + c, 0.f};
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int c = 0; c < kChains; c++) dfmac(x[c], u, v);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c].hi + x[c].lo;
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int main() {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  float *out = nullptr;
  cudaMalloc(&out, sizeof(float) * blocks * threads);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_fma = 1e30f, best_df = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    float ms = 0.f;
    cudaEventRecord(e0);
    k_fma<<<blocks, threads>>>(iters, 0.999f, 1e-3f, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best_fma) best_fma = ms;
    cudaEventRecord(e0);
    k_dfmac<<<blocks, threads>>>(iters, 0.999f, 1e-3f, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best_df) best_df = ms;
  }
  const double n = (double)blocks * threads * iters * kChains;
  printf("sms=%d fp32_tflops=%.2f dfmac_gops=%.1f\n", sms,
         2.0 * n / (best_fma * 1e-3) / 1e12, n / (best_df * 1e-3) / 1e9);
  printf("cuda=%d\n", (int)cudaGetLastError());
  cudaFree(out);
  return 0;
}
