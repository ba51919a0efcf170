// calib.cu -- FP32 CUDA-core throughput calibration (the roofline denominator of the
// direct-sum kernels, which run on the FMA pipe, not on tensor cores or HBM).
#include "lpm_common.cuh"

namespace lpm {
namespace {

constexpr int kChains = 8;

// Each thread runs kChains independent FMA recurrences a = a*m + c (|m| < 1, bounded).
__global__ void __launch_bounds__(256) ffma_loop_kernel(int iters, float m, float c, float* sink) {
  float a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = threadIdx.x * 1e-3f + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
#pragma unroll
      for (int k = 0; k < kChains; ++k) a[k] = __fmaf_rn(a[k], m, c);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == 1234.5f) sink[threadIdx.x] = s;  // keeps the chains alive
}

}  // namespace
}  // namespace lpm

extern "C" int lpm_measure_fp32_peak(double ms_target, double* tflops) {
  using namespace lpm;
  if (!tflops) return set_error(LPM_ERR_ARG, "null output");
  Context* ctx = nullptr;
  LPM_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lock(ctx->mu);
  void* sink = nullptr;
  LPM_TRY(workspace(ctx, kWsOutput, 256 * sizeof(float), &sink));
  const int blocks = ctx->sm_count * 8;
  const int threads = 256;
  cudaEvent_t e0, e1;
  LPM_CUDA_TRY(cudaEventCreate(&e0));
  LPM_CUDA_TRY(cudaEventCreate(&e1));
  int iters = 256;
  float ms = 0.f;
  int measured_iters = iters;
  for (int rep = 0; rep < 12; ++rep) {
    LPM_CUDA_TRY(cudaEventRecord(e0, ctx->stream));
    ffma_loop_kernel<<<blocks, threads, 0, ctx->stream>>>(iters, 0.999f, 0.001f, static_cast<float*>(sink));
    LPM_CUDA_TRY(cudaEventRecord(e1, ctx->stream));
    LPM_CUDA_TRY(cudaEventSynchronize(e1));
    LPM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    measured_iters = iters;  // the iteration count the timing belongs to
    if (ms >= ms_target || iters >= (1 << 24)) break;
    iters *= 2;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * kChains * 16.0 * static_cast<double>(measured_iters) * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return LPM_OK;
}
