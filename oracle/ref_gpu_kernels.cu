// ref_gpu_kernels.cu -- explicit instantiations of the reference's own FP64
// kernels (volume_gpu_kernels.hpp:9-86, sipg_sem_2d_gpu_kernels.hpp:189-316,
// conjugate_gradient_kernels.hpp:5-38), compiled unchanged from the reference
// headers by oracle/build_ref.py into oracle/_ref/ref_kernels.cubin for
// oracle/ref_gpu.cpp.  TEST INFRASTRUCTURE AND BASELINE ONLY.
#include <conjugate_gradient_kernels.hpp>
#include <sipg_sem_2d_gpu_kernels.hpp>
#include <volume_gpu_kernels.hpp>

template __global__ void volume<double>(int, mode_vector<double, int>, mode_vector<double, int>);
template __global__ void flux_term6a<double>(int, quadrilateral_mesh_info<double>, mode_vector<double, int>,
                                             mode_vector<double, int>, double);
template __global__ void flux_term6b<double>(int, quadrilateral_mesh_info<double>, mode_vector<double, int>,
                                             mode_vector<double, int>, double);
template __global__ void alpha_kernel<double>(int, double*, double*, double*, double*, double);
template __global__ void beta_kernel<double>(int, double*, double*, double);
