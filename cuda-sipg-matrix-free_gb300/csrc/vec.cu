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

// ---------------------------------------------------------------------------
// Dot product without allocation.
//
// Some callers cannot call cudaMalloc (or cudaMallocAsync): code whose device
// memory belongs to another allocator that reserved the whole pool up front,
// and code that must not risk an allocation's implicit synchronisation or an
// out-of-memory failure in the middle of a latency-critical sequence.  For
// them sipg_dot_f64_noalloc runs the same deterministic reduction as
// sipg_dot_f64 with its scratch in the fixed file-scope array below instead of
// a per-call allocation.  It is a chunked variant: block b reduces elements
// [b*2048, (b+1)*2048), so the scratch needs one partial sum per block and the
// vector length is bounded by the array size.
// ---------------------------------------------------------------------------
constexpr int kNoAllocChunk = 2048;     // elements per block: 256 threads x 8
constexpr int kNoAllocMaxBlocks = 8192; // partial sums the scratch holds
constexpr size_t kNoAllocMaxN = (size_t)kNoAllocChunk * kNoAllocMaxBlocks;  // 16,777,216 elements
// [0, kNoAllocMaxBlocks): block partials; then the arrival counter (as an
// unsigned int in the next double's storage); then the result.  65,552 bytes,
// held by every GPU that loads the library until the process exits.
static __device__ __align__(256) double g_noalloc_dot_scratch[kNoAllocMaxBlocks + 2];

__global__ void __launch_bounds__(kVecThreads) k_dot_chunked(const double* __restrict__ x, const double* __restrict__ y,
                                                             size_t n, double* __restrict__ scratch) {
  __shared__ double sh[32];
  double acc = 0.0;
  const size_t base = (size_t)blockIdx.x * kNoAllocChunk;
#pragma unroll
  for (int k = 0; k < kNoAllocChunk / kVecThreads; ++k) {
    const size_t i = base + (size_t)k * kVecThreads + threadIdx.x;
    if (i < n) acc = fma(x[i], y[i], acc);
  }
  const double bt = block_sum<double, kVecThreads>(acc, sh);
  ReduceScratch red;
  red.partials = scratch;
  red.counter = reinterpret_cast<unsigned int*>(scratch + kNoAllocMaxBlocks);
  red.capacity = kNoAllocMaxBlocks;
  double total;
  if (grid_sum_last<double, kVecThreads>(bt, red, gridDim.x, sh, &total) && threadIdx.x == 0)
    scratch[kNoAllocMaxBlocks + 1] = total;
}

// Device address of the scratch array, looked up once per device with that
// device current (the first call on each device does it) and kept for the
// life of the process: a cudaDeviceReset of the device would leave it stale,
// which is why the entry point is documented as unusable on a reset device.
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[128] = {};

static sipg_status noalloc_scratch(double** out) {
  int dev = 0;
  SIPG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) {
    set_error("sipg_dot_f64_noalloc: device ordinal out of range");
    return SIPG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_dot_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("sipg_dot_f64_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      return SIPG_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = static_cast<double*>(g_noalloc_ptr[dev]);
  return SIPG_OK;
}

static sipg_status dot_noalloc(size_t n, const double* x, const double* y, double* result, cudaStream_t s) {
  if (!x || !y || !result) {
    set_error("sipg_dot_f64_noalloc: null argument");
    return SIPG_ERR_INVALID;
  }
  if (n > kNoAllocMaxN) {
    set_error("sipg_dot_f64_noalloc: n = " + std::to_string(n) + " exceeds the no-allocation maximum of " +
              std::to_string(kNoAllocMaxN) + " elements (8192 blocks x 2048); use sipg_dot_f64");
    return SIPG_ERR_INVALID;
  }
  if (n == 0) {
    *result = 0.0;
    return SIPG_OK;
  }
  double* scratch = nullptr;
  sipg_status st = noalloc_scratch(&scratch);
  if (st != SIPG_OK) return st;
  const int nb = (int)((n + kNoAllocChunk - 1) / kNoAllocChunk);
  // the arrival counter must start at zero; the array keeps the last call's contents
  SIPG_CUDA_TRY(cudaMemsetAsync(scratch + kNoAllocMaxBlocks, 0, sizeof(double), s));
  k_dot_chunked<<<nb, kVecThreads, 0, s>>>(x, y, n, scratch);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  SIPG_CUDA_TRY(cudaMemcpyAsync(result, scratch + kNoAllocMaxBlocks + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
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
sipg_status sipg_dot_f64_noalloc(size_t n, const double* d_x, const double* d_y, double* result, void* stream) {
  return sipg::dot_noalloc(n, d_x, d_y, result, (cudaStream_t)stream);
}
}
