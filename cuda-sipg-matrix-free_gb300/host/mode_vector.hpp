// mode_vector.hpp -- DoF vectors with the reference's interface and layout
// (mode_vector.hpp:37-359): value (i1,i2) of element e at
// ((i1*nompe + i2)*noe + e).  mode_vector is a shallow device handle (copied by
// value, no destructor, explicit free()); host_mode_vector owns a std::vector.
// Difference: copy(host -> device) reuses the device array when the size is
// unchanged instead of reallocating every time (mode_vector.hpp:346-357).
// Under nvcc the handle also indexes on the device, v(i1, i2, e), as the
// reference's does (mode_vector.hpp:108-120), so kernels written against the
// reference's mode_vector compile against this one unchanged.
#pragma once

#include <cuda_runtime.h>

#include <cassert>
#include <vector>

#include "sipg_host_common.hpp"

// callable from host and device code under nvcc, as the reference's default
// constructor, get_noe and get_nompe are (mode_vector.hpp:51,149-160)
#ifdef __CUDACC__
#define SIPG_HD __host__ __device__
#else
#define SIPG_HD
#endif

template <typename FLOAT_TYPE, typename INT_TYPE>
class host_mode_vector;
template <typename FLOAT_TYPE, typename INT_TYPE>
class mode_vector;
template <typename FLOAT_TYPE, typename INT_TYPE>
void copy(const mode_vector<FLOAT_TYPE, INT_TYPE>& from, host_mode_vector<FLOAT_TYPE, INT_TYPE>& to);
template <typename FLOAT_TYPE, typename INT_TYPE>
void copy(const host_mode_vector<FLOAT_TYPE, INT_TYPE>& from, mode_vector<FLOAT_TYPE, INT_TYPE>& to);

template <typename FLOAT_TYPE, typename INT_TYPE>
class mode_vector {
  INT_TYPE noe;
  INT_TYPE nompe;
  FLOAT_TYPE* device_array;

 public:
  SIPG_HD mode_vector() : noe(0), nompe(0), device_array(nullptr) {}
  // allocates noe * nompe^2 values on the device
  mode_vector(INT_TYPE _noe, INT_TYPE _nompe) : noe(_noe), nompe(_nompe), device_array(nullptr) {
    sipg_host::check_cuda(cudaMalloc(&device_array, sizeof(FLOAT_TYPE) * (size_t)noe * nompe * nompe), "cudaMalloc");
  }
  // wraps device memory owned by the caller
  mode_vector(INT_TYPE _noe, INT_TYPE _nompe, FLOAT_TYPE* d) : noe(_noe), nompe(_nompe), device_array(d) {}
  // allocates and copies from the host
  mode_vector(const host_mode_vector<FLOAT_TYPE, INT_TYPE>& h) : noe(0), nompe(0), device_array(nullptr) {
    copy(h, *this);
  }
  const FLOAT_TYPE* data() const { return device_array; }
  FLOAT_TYPE* data() { return device_array; }
  INT_TYPE size() const { return noe * nompe * nompe; }
  SIPG_HD INT_TYPE get_noe() const { return noe; }
  SIPG_HD INT_TYPE get_nompe() const { return nompe; }
  INT_TYPE HOST_DEBUG(INT_TYPE i1, INT_TYPE i2, INT_TYPE e) const { return ((i1 * nompe) + i2) * noe + e; }
#ifdef __CUDACC__
  // value (i1, i2) of element e, from device code (mode_vector.hpp:108-120):
  // the handle is passed to a kernel by value and indexed there
  __device__ inline FLOAT_TYPE& operator()(INT_TYPE i1, INT_TYPE i2, INT_TYPE e) {
    return device_array[((i1 * nompe) + i2) * noe + e];
  }
  __device__ inline const FLOAT_TYPE& operator()(INT_TYPE i1, INT_TYPE i2, INT_TYPE e) const {
    return device_array[((i1 * nompe) + i2) * noe + e];
  }
#endif
  void free() {
    if (device_array) sipg_host::check_cuda(cudaFree(device_array), "cudaFree");
    device_array = nullptr;
    noe = 0;
    nompe = 0;
  }
  friend void copy<FLOAT_TYPE, INT_TYPE>(const host_mode_vector<FLOAT_TYPE, INT_TYPE>& from,
                                         mode_vector<FLOAT_TYPE, INT_TYPE>& to);
};

template <typename FLOAT_TYPE, typename INT_TYPE>
class host_mode_vector {
  INT_TYPE noe;
  INT_TYPE nompe;
  std::vector<FLOAT_TYPE> host_vector;

 public:
  host_mode_vector() : noe(0), nompe(0) {}
  host_mode_vector(INT_TYPE _noe, INT_TYPE _nompe)
      : noe(_noe), nompe(_nompe), host_vector((size_t)_noe * _nompe * _nompe, FLOAT_TYPE(0)) {}
  host_mode_vector(const mode_vector<FLOAT_TYPE, INT_TYPE>& mv) : noe(0), nompe(0) { copy(mv, *this); }
  INT_TYPE get_noe() const { return noe; }
  INT_TYPE get_nompe() const { return nompe; }
  INT_TYPE size() const { return (INT_TYPE)host_vector.size(); }
  const FLOAT_TYPE* data() const { return host_vector.data(); }
  FLOAT_TYPE& operator()(INT_TYPE i1, INT_TYPE i2, INT_TYPE e) {
    assert(i1 < nompe && i2 < nompe && e < noe);
    return host_vector[((size_t)i1 * nompe + i2) * noe + e];
  }
  const FLOAT_TYPE& operator()(INT_TYPE i1, INT_TYPE i2, INT_TYPE e) const {
    assert(i1 < nompe && i2 < nompe && e < noe);
    return host_vector[((size_t)i1 * nompe + i2) * noe + e];
  }
  friend void copy<FLOAT_TYPE, INT_TYPE>(const mode_vector<FLOAT_TYPE, INT_TYPE>& from,
                                         host_mode_vector<FLOAT_TYPE, INT_TYPE>& to);
  friend void copy<FLOAT_TYPE, INT_TYPE>(const host_mode_vector<FLOAT_TYPE, INT_TYPE>& from,
                                         mode_vector<FLOAT_TYPE, INT_TYPE>& to);
};

template <typename FLOAT_TYPE, typename INT_TYPE>
void copy(const mode_vector<FLOAT_TYPE, INT_TYPE>& from, host_mode_vector<FLOAT_TYPE, INT_TYPE>& to) {
  to.noe = from.get_noe();
  to.nompe = from.get_nompe();
  to.host_vector.resize((size_t)from.size());
  sipg_host::check_cuda(cudaMemcpy(to.host_vector.data(), from.data(), sizeof(FLOAT_TYPE) * (size_t)from.size(),
                                   cudaMemcpyDeviceToHost),
                        "cudaMemcpy D2H");
}

template <typename FLOAT_TYPE, typename INT_TYPE>
void copy(const host_mode_vector<FLOAT_TYPE, INT_TYPE>& from, mode_vector<FLOAT_TYPE, INT_TYPE>& to) {
  const size_t n = (size_t)from.get_noe() * from.get_nompe() * from.get_nompe();
  if (!to.device_array || (size_t)to.size() != n) {
    if (to.device_array) sipg_host::check_cuda(cudaFree(to.device_array), "cudaFree");
    to.device_array = nullptr;
    sipg_host::check_cuda(cudaMalloc(&to.device_array, sizeof(FLOAT_TYPE) * n), "cudaMalloc");
  }
  to.noe = from.get_noe();
  to.nompe = from.get_nompe();
  sipg_host::check_cuda(cudaMemcpy(to.device_array, from.data(), sizeof(FLOAT_TYPE) * n, cudaMemcpyHostToDevice),
                        "cudaMemcpy H2D");
}
