// Diagnostics: live measurement of the FP64 FMA rate, the roofline denominator of the LLG kernels.
#include "mgx_internal.cuh"

namespace mgx {

// Eight independent DFMA chains per thread keep the FP64 pipe busy without memory traffic.
__global__ void __launch_bounds__(256) k_dfma_rate(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
  double x4 = x0 + 4.0, x5 = x0 + 5.0, x6 = x0 + 6.0, x7 = x0 + 7.0;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace mgx

using namespace mgx;

extern "C" mgx_status mgx_measure_fp64_peak(double* flops_per_s) {
  if (!flops_per_s) return set_error(MGX_ERR_INVALID, "mgx_measure_fp64_peak: null argument");
  int dev = 0, sms = 0;
  MGX_CUDA_TRY(cudaGetDevice(&dev));
  MGX_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256, iters = 1000;
  double* buf = nullptr;
  MGX_CUDA_TRY(cudaMalloc(&buf, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_rate<<<blocks, threads>>>(buf, 16, 1.0000001, 1e-9);      // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_dfma_rate<<<blocks, threads>>>(buf, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (err != cudaSuccess) return cuda_error(err, "mgx_measure_fp64_peak");
  const double fmas = (double)blocks * threads * iters * 64.0;
  *flops_per_s = 2.0 * fmas / (best * 1e-3);
  return MGX_OK;
}
