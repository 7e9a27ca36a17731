// vec.cu -- the vector operations of the reference's generic CG, for callers
// that drive the iteration themselves around their own operator (the
// abs_mvm interface, abs_mvm.hpp:10-19):
//   sipg_dot_*      r = x.y                 (cublas_dot, cublas_wrapper.hpp:62-84)
//   sipg_cg_step_*  x += a p; r -= a Ap     (alpha_kernel, conjugate_gradient_kernels.hpp:5-23)
//   sipg_xpby_*     y = x + b y             (beta_kernel, conjugate_gradient_kernels.hpp:26-38)
// The dot is a deterministic two-level reduction (fixed block partials summed
// in index order by the last block).
#include "sipg_cg.cuh"

namespace sipg {

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_dot(const T* __restrict__ x, const T* __restrict__ y, size_t n,
                                                     ReduceScratch red, T* __restrict__ result) {
  __shared__ T sh[32];
  T acc = T(0);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) acc = fma(x[i], y[i], acc);
  const T bt = block_sum<T, kVecThreads>(acc, sh);
  T total;
  if (grid_sum_last<T, kVecThreads>(bt, red, gridDim.x, sh, &total) && threadIdx.x == 0) *result = total;
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_cg_step(size_t n, T alpha, T* __restrict__ x, const T* __restrict__ p,
                                                         T* __restrict__ r, const T* __restrict__ Ap) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] = fma(alpha, p[i], x[i]);
    r[i] = fma(-alpha, Ap[i], r[i]);
  }
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_xpby(size_t n, const T* __restrict__ x, T beta, T* __restrict__ y) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) y[i] = fma(beta, y[i], x[i]);
}

static int vblocks(size_t n) {
  const size_t want = (n + kVecThreads - 1) / kVecThreads;
  return (int)std::max<size_t>(1, std::min<size_t>(want, 152 * 8));
}

template <typename T>
static sipg_status dot(size_t n, const T* x, const T* y, T* result, cudaStream_t s) {
  if (!x || !y || !result) {
    set_error("sipg_dot: null argument");
    return SIPG_ERR_INVALID;
  }
  const int nb = vblocks(n);
  // scratch: nb partials, the counter, the result (stream-ordered pool allocation)
  char* buf = nullptr;
  const size_t bytes = sizeof(double) * (nb + 2) + 64;
  SIPG_CUDA_TRY(cudaMallocAsync((void**)&buf, bytes, s));
  ReduceScratch red;
  red.partials = (double*)buf;
  red.counter = (unsigned int*)(buf + sizeof(double) * nb);
  red.capacity = nb;
  T* d_res = (T*)(buf + sizeof(double) * (nb + 1));
  cudaError_t e = cudaMemsetAsync(red.counter, 0, sizeof(unsigned int), s);
  if (e == cudaSuccess) {
    k_dot<T><<<nb, kVecThreads, 0, s>>>(x, y, n, red, d_res);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(result, d_res, sizeof(T), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(buf, s);
  SIPG_CUDA_TRY(e);
  return SIPG_OK;
}

template <typename T>
static sipg_status cg_step(size_t n, T alpha, T* x, const T* p, T* r, const T* Ap, cudaStream_t s) {
  if (!x || !p || !r || !Ap) {
    set_error("sipg_cg_step: null argument");
    return SIPG_ERR_INVALID;
  }
  k_cg_step<T><<<vblocks(n), kVecThreads, 0, s>>>(n, alpha, x, p, r, Ap);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  return SIPG_OK;
}

template <typename T>
static sipg_status xpby(size_t n, const T* x, T beta, T* y, cudaStream_t s) {
  if (!x || !y) {
    set_error("sipg_xpby: null argument");
    return SIPG_ERR_INVALID;
  }
  k_xpby<T><<<vblocks(n), kVecThreads, 0, s>>>(n, x, beta, y);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  return SIPG_OK;
}

}  // namespace sipg

extern "C" {
sipg_status sipg_dot_f64(size_t n, const double* d_x, const double* d_y, double* result, void* stream) {
  return sipg::dot<double>(n, d_x, d_y, result, (cudaStream_t)stream);
}
sipg_status sipg_dot_f32(size_t n, const float* d_x, const float* d_y, float* result, void* stream) {
  return sipg::dot<float>(n, d_x, d_y, result, (cudaStream_t)stream);
}
sipg_status sipg_cg_step_f64(size_t n, double alpha, double* d_x, const double* d_p, double* d_r, const double* d_Ap,
                             void* stream) {
  return sipg::cg_step<double>(n, alpha, d_x, d_p, d_r, d_Ap, (cudaStream_t)stream);
}
sipg_status sipg_cg_step_f32(size_t n, float alpha, float* d_x, const float* d_p, float* d_r, const float* d_Ap,
                             void* stream) {
  return sipg::cg_step<float>(n, alpha, d_x, d_p, d_r, d_Ap, (cudaStream_t)stream);
}
sipg_status sipg_xpby_f64(size_t n, const double* d_x, double beta, double* d_y, void* stream) {
  return sipg::xpby<double>(n, d_x, beta, d_y, (cudaStream_t)stream);
}
sipg_status sipg_xpby_f32(size_t n, const float* d_x, float beta, float* d_y, void* stream) {
  return sipg::xpby<float>(n, d_x, beta, d_y, (cudaStream_t)stream);
}
}
