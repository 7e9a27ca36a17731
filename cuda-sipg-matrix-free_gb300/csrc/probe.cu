// probe.cu -- diagnostic: the FP64 and FP32 FMA throughput of the current
// device, measured with independent FMA chains (used to state what fraction of
// the FP64 pipe the FP64 apply reaches; GB300's FP64 rate is about 1/50 of FP32).
#include "sipg_internal.cuh"

namespace sipg {

template <typename T, int CHAINS, int ITERS>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, T a, T b) {
  T acc[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) acc[c] = (T)(threadIdx.x + c);
#pragma unroll 1
  for (int it = 0; it < ITERS; ++it) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = fma(acc[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += acc[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T, int ITERS>
static sipg_status probe(double* tflops) {
  int dev = 0, sms = 0;
  SIPG_CUDA_TRY(cudaGetDevice(&dev));
  SIPG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256;
  T* out = nullptr;
  SIPG_CUDA_TRY(cudaMalloc(&out, sizeof(T) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int w = 0; w < 2; ++w) k_fma_probe<T, 8, ITERS><<<blocks, threads>>>(out, (T)0.999, (T)0.001);
  cudaEventRecord(e0);
  const int reps = 3;
  for (int r = 0; r < reps; ++r) k_fma_probe<T, 8, ITERS><<<blocks, threads>>>(out, (T)0.999, (T)0.001);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  count_launch(2 + reps);
  SIPG_CUDA_TRY(err);
  SIPG_CUDA_TRY(cudaGetLastError());
  *tflops = 2.0 * blocks * threads * 8.0 * ITERS * reps / (ms * 1e-3) / 1e12;
  return SIPG_OK;
}

}  // namespace sipg

extern "C" sipg_status sipg_probe_fma_peak(double* fp64_tflops, double* fp32_tflops) {
  if (!fp64_tflops || !fp32_tflops) return SIPG_ERR_INVALID;
  sipg_status s = sipg::probe<double, 2048>(fp64_tflops);
  if (s != SIPG_OK) return s;
  return sipg::probe<float, 16384>(fp32_tflops);
}
