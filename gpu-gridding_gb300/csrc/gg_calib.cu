// FP32 fused-multiply-add throughput probe: the denominator of the
// gridding kernel's roofline.  The gridder's arithmetic is FP32 FMA on the
// CUDA cores (4 FMA per complex multiply-add), a peak that an HBM copy or
// a bf16 tensor GEMM does not measure, so it is measured here:
// every SM runs independent FMA chains long enough to reach steady clocks.
#include "gg_internal.h"

namespace gg {

namespace {

constexpr int kChains = 16;

__global__ void __launch_bounds__(256) k_ffma(float* out, int iters,
                                              float b, float c) {
  float acc[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) acc[k] = threadIdx.x * 1e-7f + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) acc[k] = fmaf(acc[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += acc[k];
  // Never true for the values used; keeps the chains live.
  if (s == 1234.5f) out[blockIdx.x] = s;
}

// The same chains as packed FP32x2 FMAs (two FMAs per instruction), the
// form the gridding kernel issues: the FP32 FMA rate is the larger of the
// two probes.
__global__ void __launch_bounds__(256) k_ffma2(float* out, int iters,
                                               float b, float c) {
  float2 acc[kChains / 2];
#pragma unroll
  for (int k = 0; k < kChains / 2; ++k)
    acc[k] = make_float2(threadIdx.x * 1e-7f + 2 * k,
                         threadIdx.x * 1e-7f + 2 * k + 1);
  const float2 bb = make_float2(b, b), cc = make_float2(c, c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains / 2; ++k) acc[k] = __ffma2_rn(acc[k], bb, cc);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains / 2; ++k) s += acc[k].x + acc[k].y;
  if (s == 1234.5f) out[blockIdx.x] = s;
}

}  // namespace

cudaError_t measure_fp32_fma(int num_sms, double* tflops_best,
                             float* ms_out) {
  float* dummy = nullptr;
  cudaError_t e = cudaMalloc(&dummy, 4096 * sizeof(float));
  if (e != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = num_sms * 8, threads = 256, iters = 1 << 15;
  double best = 0.0;
  float best_ms = 0.f;
  for (int rep = 0; rep < 12; ++rep) {
    cudaEventRecord(a);
    if (rep % 2 == 0)
      k_ffma<<<blocks, threads>>>(dummy, iters, 0.9999f, 1e-4f);
    else
      k_ffma2<<<blocks, threads>>>(dummy, iters, 0.9999f, 1e-4f);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    if (e != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    const double flops = 2.0 * kChains * (double)iters * blocks * threads;
    const double tf = flops / (ms * 1e-3) / 1e12;
    if (rep > 1 && tf > best) { best = tf; best_ms = ms; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(dummy);
  *tflops_best = best;
  if (ms_out) *ms_out = best_ms;
  return e == cudaSuccess ? cudaGetLastError() : e;
}

}  // namespace gg
