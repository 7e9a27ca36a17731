// mode_vector_kernel.cu -- a user kernel written the way the reference writes
// its kernels against mode_vector (volume_gpu_kernels.hpp:9-86: the handle
// passed by value, indexed in(i1, i2, e) on the device, grid
// (ceil(noe/128), n, n) x 128), compiled against the host API's mode_vector.
// It applies the nodal mass matrix of the SIPG-SEM basis, out(i1,i2,e) =
// (h/2)^2 w_i1 w_i2 in(i1,i2,e), with the LGL weights from the C ABI.  Prints
// one JSON line with the largest difference from the same product formed on
// the host through HOST_DEBUG indexing, relative to the largest value (exit 0
// when it is at rounding level).
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "mode_vector.hpp"
#include "sipg_gb300.h"

template <typename FLOAT_TYPE>
__global__ void mass_kernel(mode_vector<FLOAT_TYPE, int> in, mode_vector<FLOAT_TYPE, int> out, const FLOAT_TYPE* w,
                            FLOAT_TYPE scale) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int i1 = blockIdx.y, i2 = blockIdx.z;
  if (e < in.get_noe()) out(i1, i2, e) = scale * w[i1] * w[i2] * in(i1, i2, e);
}

int main() {
  const int dim = 37, p = 5, n = p + 1, noe = dim * dim;
  std::vector<double> nodes(n), w(n);
  if (sipg_lgl_table(n, nodes.data(), w.data()) != SIPG_OK) return 2;
  host_mode_vector<double, int> h_in(noe, n);
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2)
      for (int e = 0; e < noe; ++e) h_in(i1, i2, e) = U(rng);
  mode_vector<double, int> d_in(h_in), d_out(noe, n);
  double* d_w = nullptr;
  cudaMalloc(&d_w, sizeof(double) * n);
  cudaMemcpy(d_w, w.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  const double h = 1.0 / dim, scale = 0.25 * h * h;
  mass_kernel<double><<<dim3((noe + 127) / 128, n, n), 128>>>(d_in, d_out, d_w, scale);
  if (cudaDeviceSynchronize() != cudaSuccess) return 3;
  host_mode_vector<double, int> h_out(d_out);
  double maxerr = 0.0, maxref = 0.0;
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2)
      for (int e = 0; e < noe; ++e) {
        const double ref = scale * w[i1] * w[i2] * h_in.data()[d_in.HOST_DEBUG(i1, i2, e)];
        maxerr = std::fmax(maxerr, std::fabs(h_out.data()[d_out.HOST_DEBUG(i1, i2, e)] - ref));
        maxref = std::fmax(maxref, std::fabs(ref));
      }
  const double rel = maxref > 0 ? maxerr / maxref : maxerr;
  std::printf("{\"case\": \"mode_vector_kernel\", \"dim\": %d, \"p\": %d, \"max_rel_err\": %.3e}\n", dim, p, rel);
  cudaFree(d_w);
  d_in.free();
  d_out.free();
  // a wrong index gives an O(1) error; the device's products may round differently in the last bit
  return rel <= 1e-14 ? 0 : 1;
}
