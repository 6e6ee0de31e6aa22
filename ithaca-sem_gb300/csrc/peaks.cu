// Arithmetic-pipe peaks of the device, measured: FP64 FMA, FP64 tensor-core MMA (DMMA,
// mma.sync m8n8k4 f64) and FP32 FMA throughput. They are the compute roofs the FP64
// element operators and the FP32 inner applies are judged against (the copy-bandwidth
// and bf16 peaks come from outside the library). Each kernel runs a fixed number of
// independent dependency chains per thread; one launch per pipe is timed with CUDA events
// after a warm-up launch.
#include <cuda_runtime.h>

#include "ithaca_internal.h"

namespace ithaca {
namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) fp64_fma_loop(double* sink, int iters, double a, double b) {
  double v[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) v[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < kChains; ++i) v[i] = fma(v[i], a, b);
  double s = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += v[i];
  if (s == 1234.5678) sink[0] = s;  // keeps the chains live; never true for these inputs
}

__global__ void __launch_bounds__(256) fp32_fma_loop(float* sink, int iters, float a, float b) {
  float v[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) v[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < kChains; ++i) v[i] = fmaf(v[i], a, b);
  float s = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += v[i];
  if (s == 1234.5678f) sink[0] = s;
}

// one m8n8k4 FP64 MMA per warp per chain and iteration: 8 x 8 x 4 x 2 flops
__global__ void __launch_bounds__(256) dmma_loop(double* sink, int iters) {
  const double a = threadIdx.x * 1e-3, b = 0.5;
  double c[kChains / 2][2];
#pragma unroll
  for (int i = 0; i < kChains / 2; ++i) c[i][0] = c[i][1] = 0.0;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < kChains / 2; ++i)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[i][0]), "+d"(c[i][1])
                   : "d"(a), "d"(b));
  double s = 0;
#pragma unroll
  for (int i = 0; i < kChains / 2; ++i) s += c[i][0] + c[i][1];
  if (s == 1234.5678) sink[0] = s;
}

template <typename F>
double time_ms(F launch, cudaStream_t s) {
  cudaEvent_t e0, e1;
  ITHACA_CUDA(cudaEventCreate(&e0));
  ITHACA_CUDA(cudaEventCreate(&e1));
  launch();  // warm-up
  ITHACA_CUDA(cudaEventRecord(e0, s));
  launch();
  ITHACA_CUDA(cudaEventRecord(e1, s));
  ITHACA_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  ITHACA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ITHACA_CUDA(cudaGetLastError());
  return ms;
}

}  // namespace
}  // namespace ithaca

using namespace ithaca;

struct ithaca_gpu_ctx : public Ctx {};

extern "C" int ithaca_gpu_measure_pipe_peaks(ithaca_gpu_ctx* ctx, double* fp64_fma_tflops, double* fp64_mma_tflops,
                                             double* fp32_fma_tflops) {
  try {
    if (!ctx || !fp64_fma_tflops || !fp64_mma_tflops || !fp32_fma_tflops) fail(ITHACA_GPU_ERR_ARG, "null argument");
    Ctx* c = ctx;
    cudaStream_t s = c->stream;
    const int sms = device_sm_count(), blocks = sms * 8, threads = 256, iters = 4096;
    double* sink = static_cast<double*>(c->stage_ptr(3, 64));
    const double nthr = (double)blocks * threads;
    double ms = time_ms([&] { fp64_fma_loop<<<blocks, threads, 0, s>>>(sink, iters, 1.000001, 1e-7); }, s);
    *fp64_fma_tflops = 2.0 * nthr * iters * kChains / (ms * 1e-3) / 1e12;
    ms = time_ms([&] { fp32_fma_loop<<<blocks, threads, 0, s>>>((float*)sink, iters * 8, 1.000001f, 1e-7f); }, s);
    *fp32_fma_tflops = 2.0 * nthr * iters * 8 * kChains / (ms * 1e-3) / 1e12;
    ms = time_ms([&] { dmma_loop<<<blocks, threads, 0, s>>>(sink, iters / 4); }, s);
    *fp64_mma_tflops = (double)blocks * (threads / 32) * (iters / 4) * (kChains / 2) * 8 * 8 * 4 * 2 / (ms * 1e-3) / 1e12;
    c->launches += 6;
    return ITHACA_GPU_OK;
  } catch (const Error& e) {
    set_last_error(e.msg);
    return e.code;
  }
}
