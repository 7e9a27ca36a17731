// CUDA_TIMER.hpp -- event timer of the reference's interface (CUDA_TIMER.hpp:14-51):
// start()/stop() record events on the legacy stream, elapsed_millisecs() reads them.
#pragma once

#include <cuda_runtime.h>

class CUDA_TIMER {
  cudaEvent_t _start = nullptr, _stop = nullptr;
  float _elapsed_millisecs = 0.f;

 public:
  void start() {
    cudaEventCreate(&_start);
    cudaEventCreate(&_stop);
    cudaEventRecord(_start, 0);
  }
  void stop() {
    cudaEventRecord(_stop, 0);
    cudaEventSynchronize(_stop);
    cudaEventElapsedTime(&_elapsed_millisecs, _start, _stop);
    cudaEventDestroy(_start);
    cudaEventDestroy(_stop);
  }
  float elapsed_millisecs() const { return _elapsed_millisecs; }
};
