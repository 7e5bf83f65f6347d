// lbm_probe.cu - FMA throughput of the current GPU, the compute roofline of
// the FP64 fused kernel (which is bound by the FP64 pipe on GB300).
#include "lbm_internal.cuh"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chains(T* out, int iters, T a, T b) {
  T x0 = T(threadIdx.x), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int run(double* tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LBM_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return LBM_ERR_CUDA;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return LBM_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chains<T><<<blocks, threads>>>(out, 64, T(0.999), T(0.001));
  lbm::count_launch();
  cudaEventRecord(e0);
  k_fma_chains<T><<<blocks, threads>>>(out, iters, T(0.999), T(0.001));
  lbm::count_launch();
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return LBM_ERR_CUDA;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return LBM_OK;
}

}  // namespace

extern "C" int lbm_fma_throughput(int precision, double* tflops) {
  if (!tflops) return LBM_ERR_ARG;
  return precision == LBM_PREC_F32 ? run<float>(tflops) : run<double>(tflops);
}
