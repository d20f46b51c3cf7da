// Diagnostic: FP64 FMA throughput of the current device (roofline denominator of the FP64
// kernels). Eight independent dependent-FMA chains per thread, 8 CTAs of 256 threads per SM.
#include <cuda_runtime.h>

#include "oakg_internal.cuh"

namespace oakg {
void count_launches(int k);
cudaStream_t current_stream();
int record_failure(int code, const char* msg);
}

namespace {
__global__ void k_dfma_peak(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4,
         x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

extern "C" int oakg_fp64_peak(double* tflops) {
  if (!tflops) return OAKG_ERR_ARGS;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return OAKG_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return OAKG_ERR_NOMEM;
  cudaStream_t st = oakg::current_stream();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_peak<<<blocks, threads, 0, st>>>(out, 200, 1.0000001, 1e-9);
  const int iters = 20000;
  cudaEventRecord(e0, st);
  k_dfma_peak<<<blocks, threads, 0, st>>>(out, iters, 1.0000001, 1e-9);
  cudaEventRecord(e1, st);
  oakg::count_launches(2);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) return OAKG_ERR_CUDA;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return OAKG_OK;
}
