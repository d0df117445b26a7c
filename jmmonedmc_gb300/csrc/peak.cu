// peak.cu -- live roofline denominators for the pair kernels: the FP32 FMA
// rate and the MUFU reciprocal rate of this device, each from a kernel that
// keeps every SM busy with independent dependency chains, timed with CUDA
// events (best of several launches).
#include "common.cuh"

namespace {

constexpr int kChains = 8;      // independent accumulators per thread
constexpr int kIters = 4096;

__global__ void fma_kernel(float *out, float a, float b) {
  float acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = threadIdx.x * 1e-3f + c;
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc[c] = __fmaf_rn(acc[c], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += acc[c];
  if (s == 1234.5f) out[0] = s;  // keeps the loop alive
}

__global__ void rcp_kernel(float *out) {
  float acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = 1.0f + threadIdx.x * 1e-6f + c * 1e-3f;
  for (int it = 0; it < kIters / 4; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
      float y;  // x <- 1 / (x + 1): one reciprocal and one add per link
      asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(acc[c] + 1.0f));
      acc[c] = y;
    }
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += acc[c];
  if (s == 1234.5f) out[0] = s;
}

}  // namespace

extern "C" int jmm_measure_peaks(double *fp32_tflops, double *rcp_tops) {
  jmm::clear_error();
  JMM_CHECK_ARG(fp32_tflops && rcp_tops, "null output");
  int dev = 0, sms = 0;
  JMM_CUDA(cudaGetDevice(&dev));
  JMM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  float *out = nullptr;
  JMM_CUDA(cudaMalloc((void **)&out, sizeof(float)));
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  const int blocks = sms * 8, threads = 256;
  float best_fma = 1e30f, best_rcp = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    float ms;
    cudaEventRecord(t0);
    fma_kernel<<<blocks, threads>>>(out, 0.999f, 1e-3f);
    cudaEventRecord(t1);
    cudaEventSynchronize(t1);
    cudaEventElapsedTime(&ms, t0, t1);
    if (rep > 0 && ms < best_fma) best_fma = ms;
    cudaEventRecord(t0);
    rcp_kernel<<<blocks, threads>>>(out);
    cudaEventRecord(t1);
    cudaEventSynchronize(t1);
    cudaEventElapsedTime(&ms, t0, t1);
    if (rep > 0 && ms < best_rcp) best_rcp = ms;
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  if (e != cudaSuccess) return jmm::cuda_status(e, "jmm_measure_peaks", __FILE__, __LINE__);
  const double threads_total = (double)blocks * threads;
  *fp32_tflops = threads_total * kIters * kChains * 2.0 / (best_fma * 1e-3) / 1e12;
  *rcp_tops = threads_total * (kIters / 4) * kChains / (best_rcp * 1e-3) / 1e12;
  return JMM_OK;
}
