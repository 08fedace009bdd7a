// probe.cu -- libmsfem_probe.so: measures this GPU's FP64 / FP32 FMA issue
// rate, the roofline denominator of the basis kernels (they are bound by the
// CUDA-core FMA pipes, not by HBM or the tensor cores).  Not part of the
// msfem C-ABI.
#include <cuda_runtime.h>

namespace {

template <typename T>
__global__ void fma_chain(T *out, T b, T c, int iters) {
  // 8 independent accumulators per thread hide the FMA latency
  T a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  T a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == T(-1.2345)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chain live
}

}  // namespace

extern "C" int msfem_probe_fma_flops(int fp64, double *flops_per_s) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  const int threads = 256, blocks = sms * 8;
  const int iters = fp64 ? 4096 : 65536;
  void *buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * threads * blocks) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    if (fp64) fma_chain<double><<<blocks, threads>>>((double *)buf, 0.999999, 1e-7, iters);
    else fma_chain<float><<<blocks, threads>>>((float *)buf, 0.999999f, 1e-7f, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (cudaGetLastError() != cudaSuccess) return -1;
  *flops_per_s = 2.0 * 8.0 * iters * (double)threads * blocks / (best * 1e-3);
  return 0;
}
