// sipg_host_common.hpp -- error handling shared by the C++ host API (the
// reference-compatible headers in this directory).  The reference exits the
// process on a CUDA error (CUDA_ERRORS.hpp:147-166); this API throws
// sipg_host::error instead, carrying the sipg_status and the message.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "sipg_gb300.h"

namespace sipg_host {

struct error : std::runtime_error {
  sipg_status status;
  error(sipg_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(sipg_status s, const char* what) {
  if (s != SIPG_OK) throw error(s, std::string(what) + ": " + sipg_last_error());
}

inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw error(SIPG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace sipg_host
