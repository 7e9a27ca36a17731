/*
 * cuda_emul.h -- lets the reference's own CUDA headers compile with g++ and
 * run on a CPU, so that its kernels (volume, flux_term6a/6b, volume_mvm,
 * alpha/beta_kernel) and its host driver (sipg_sem_2d, conjugate_gradient)
 * produce golden outputs without a GPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Included first by oracle/ref_emul.cpp, which
 * oracle/build_ref.py compiles against the reference headers.
 *
 * - the CUDA qualifiers become nothing, so kernels are plain functions and
 *   __constant__ tables plain globals;
 * - blockIdx/threadIdx/blockDim/gridDim are globals that emu::launch sets while
 *   it calls a kernel once per (block, thread) in order -- exact for these
 *   kernels, which use neither shared memory nor barriers and whose threads
 *   write disjoint outputs;
 * - device memory is host memory (cudaMalloc -> malloc, cudaMemcpy -> memmove);
 * - cublas_dot sums in index order on one thread.
 * The reference's CUDA_ERRORS.hpp and cublas_wrapper.hpp are replaced through
 * their include guards by the small equivalents below.
 */
#ifndef SIPG_CUDA_EMUL_H
#define SIPG_CUDA_EMUL_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

static dim3 blockIdx, threadIdx, blockDim, gridDim;

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };

template <class T>
static inline cudaError_t cudaMalloc(T** p, size_t n) {
  *p = (T*)std::calloc(n ? n : 1, 1);
  return *p ? 0 : 2;
}
static inline cudaError_t cudaFree(void* p) {
  std::free(p);
  return 0;
}
static inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
  std::memmove(d, s, n);
  return 0;
}
template <class T>
static inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n, size_t off = 0,
                                             cudaMemcpyKind = cudaMemcpyHostToDevice) {
  std::memcpy((char*)&sym + off, src, n);
  return 0;
}
static inline cudaError_t cudaGetLastError() { return 0; }
static inline const char* cudaGetErrorString(cudaError_t) { return "no error (CPU emulation)"; }
static inline cudaError_t cudaDeviceReset() { return 0; }
static inline cudaError_t cudaDeviceSynchronize() { return 0; }
static inline cudaError_t cudaThreadSynchronize() { return 0; }

typedef int cudaEvent_t;
static inline cudaError_t cudaEventCreate(cudaEvent_t* e) {
  *e = 0;
  return 0;
}
static inline cudaError_t cudaEventRecord(cudaEvent_t, int = 0) { return 0; }
static inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return 0; }
static inline cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) {
  *ms = 0;
  return 0;
}
static inline cudaError_t cudaEventDestroy(cudaEvent_t) { return 0; }

/* stands in for CUDA_ERRORS.hpp */
#define __CUDA_ERRORS_HPP__
namespace emu {
static inline void check(int rc, const char* what) {
  if (rc) {
    std::fprintf(stderr, "emulated CUDA call failed: %s\n", what);
    std::abort();
  }
}
}  // namespace emu
#define checkError(val) ::emu::check((int)(val), #val)

/* stands in for cublas_wrapper.hpp */
#define __CUBLAS_WRAPPER_HPP__
typedef void* cublasHandle_t;
typedef int cublasStatus_t;
static inline cublasStatus_t cublasCreate(cublasHandle_t* h) {
  *h = nullptr;
  return 0;
}
static inline cublasStatus_t cublasDestroy(cublasHandle_t) { return 0; }
template <class T>
static inline cublasStatus_t cublas_dot(cublasHandle_t, int n, const T* x, int incx, const T* y, int incy, T* result) {
  T s = 0;
  for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
  *result = s;
  return 0;
}

namespace emu {
/* kernel<<<grid, block>>>(args) is rewritten by build_ref.py as
 * ::emu::launch([&](auto&&... a) { kernel(a...); }, grid, block)(args) */
template <class F>
struct launcher {
  F f;
  dim3 g, b;
  template <class... A>
  void operator()(A&&... args) {
    gridDim = g;
    blockDim = b;
    for (unsigned bz = 0; bz < g.z; ++bz)
      for (unsigned by = 0; by < g.y; ++by)
        for (unsigned bx = 0; bx < g.x; ++bx)
          for (unsigned tz = 0; tz < b.z; ++tz)
            for (unsigned ty = 0; ty < b.y; ++ty)
              for (unsigned tx = 0; tx < b.x; ++tx) {
                blockIdx = dim3(bx, by, bz);
                threadIdx = dim3(tx, ty, tz);
                f(args...);
              }
  }
};
template <class F>
static inline launcher<F> launch(F f, dim3 g, dim3 b) {
  return launcher<F>{f, g, b};
}
}  // namespace emu

#endif
