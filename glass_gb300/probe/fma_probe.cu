// Measured FMA throughput of the GPU's FP32 and FP64 pipes, so that rooflines
// of the CUDA-core-bound kernels are reported against this machine's own peak
// rather than a datasheet figure.  A measuring aid for the benchmark, built
// into its own library (lib/libglass_probe.so), not into the engine.
#include <cuda_runtime.h>

#define GLASS_OK 0
#define GLASS_ERR_ARG -1
#define GLASS_ERR_CUDA -3

namespace {

template <typename R>
__global__ void fma_probe_kernel(R *out, int iters, R a, R b) {
  // 8 independent chains per thread keep the pipe busy.
  R x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  R s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (R)-12345.678) out[0] = s;  // keeps the chains live
}

template <typename R>
int run_probe(int device, double *tflops) {
  if (cudaSetDevice(device) != cudaSuccess) return GLASS_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  R *out = nullptr;
  if (cudaMalloc(&out, sizeof(R)) != cudaSuccess) return GLASS_ERR_CUDA;
  const int threads = 512, blocks = sms * 4;
  const int iters = sizeof(R) == 4 ? 4096 : 64;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_probe_kernel<R><<<blocks, threads>>>(out, iters, (R)0.999999, (R)1e-7);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; rep++) {
    cudaEventRecord(e0);
    fma_probe_kernel<R><<<blocks, threads>>>(out, iters, (R)0.999999, (R)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return GLASS_ERR_CUDA;
  double flops = 2.0 * 8 * 16 * (double)iters * threads * (double)blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  return GLASS_OK;
}

}  // namespace

extern "C" int glass_gpu_probe_fma_tflops(int device, int fp64, double *tflops) {
  if (!tflops) return GLASS_ERR_ARG;
  return fp64 ? run_probe<double>(device, tflops) : run_probe<float>(device, tflops);
}
