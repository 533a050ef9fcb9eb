// Measured FP64 peak of the GPU the library runs on: the denominator of the
// element kernel's FP64 roofline (the element R+J assembly is bound by the FP64
// pipe). Every thread runs eight independent fused multiply-add chains, so
// the pipe, not latency, limits the rate.
#include "common.cuh"

namespace goal {
namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_dfma_peak(int iters, double a, double b, double* out) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-9 + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace
}  // namespace goal

extern "C" int goal_measure_fp64_peak(double* tflops) {
  using namespace goal;
  try {
    if (!tflops) throw Error(GOAL_ERR_ARG, "goal_measure_fp64_peak: null argument");
    const int blocks = kSMs * 8, threads = 256, iters = 4096;
    DevBuf<double> out;
    out.alloc(1);
    cudaEvent_t e0, e1;
    GOAL_CUDA(cudaEventCreate(&e0));
    GOAL_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 6; ++rep) {
      GOAL_CUDA(cudaEventRecord(e0));
      k_dfma_peak<<<blocks, threads>>>(iters, 0.999999, 1e-7, out.ptr);
      GOAL_CHECK_LAUNCH();
      GOAL_CUDA(cudaEventRecord(e1));
      GOAL_CUDA(cudaEventSynchronize(e1));
      float ms = 0.0f;
      GOAL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0 && ms < best) best = ms;  // the first launch warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flop = 2.0 * kChains * (double)iters * blocks * threads;
    *tflops = flop / (best * 1e-3) / 1e12;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  }
  return GOAL_OK;
}
