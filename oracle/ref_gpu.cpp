/*
 * ref_gpu.cpp -- runs the reference's own CUDA kernels on the GPU.
 *
 * TEST INFRASTRUCTURE AND BASELINE ONLY.  oracle/build_ref.py compiles the
 * reference's kernel headers (volume_gpu_kernels.hpp, sipg_sem_2d_gpu_kernels.hpp,
 * conjugate_gradient_kernels.hpp) unchanged for sm_103a into
 * oracle/_ref/ref_kernels.cubin.  This file (built on the GPU machine into
 * oracle/_ref/libref_gpu.so) loads that cubin with the CUDA runtime's library
 * API, fills the reference's __constant__ tables (device_const.hpp:10-18) the
 * way load_Dphi_table / load_lgl_quadrature_table do, and launches the kernels
 * with the reference's launch geometry:
 *   - refgpu_apply: sipg_sem_2d<T>::_mvm (sipg_sem_2d.hpp:167-201): volume,
 *     flux_term6a, flux_term6b on one stream, `reps` times (the timing loop of
 *     performance_tests/mvm_performance_test.cu:44-65);
 *   - refgpu_cg: conjugate_gradient<T> (conjugate_gradient_gpu.hpp:18-109):
 *     the same host loop around the reference's apply, alpha_kernel,
 *     beta_kernel and blocking cublasDdot calls.
 * It is the "reference on the same GPU" baseline; the product never uses it.
 */
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "sipg_oracle.h"

namespace {

// Kernel-parameter layouts of the reference's mode_vector<double,int>
// (mode_vector.hpp:43-46) and quadrilateral_mesh_info<double> (mesh_info.hpp:177-184).
struct RefModeVector {
  int noe;
  int nompe;
  double* device_array;
};
struct RefQuadMesh {
  int dimx;
  int dimy;
  int noe;
  double* x;
  double* y;
};

cudaLibrary_t g_lib = nullptr;
cudaKernel_t g_volume = nullptr, g_flux6a = nullptr, g_flux6b = nullptr, g_alpha = nullptr, g_beta = nullptr;
void* g_dphi = nullptr;     // d_dphi_double[4096]
void* g_weights = nullptr;  // d_lgl_weights_double[64]
void* g_nodes = nullptr;    // d_lgl_nodes_double[64]
std::string g_err;

int fail(const char* what, cudaError_t e) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return (int)e ? (int)e : 1;
}

#define TRY(call)                         \
  do {                                    \
    cudaError_t _e = (call);              \
    if (_e != cudaSuccess) return fail(#call, _e); \
  } while (0)

int load_tables(int p) {
  double nodes[64], w[64], D[64 * 64];
  if (sipg_oracle_lgl(p + 1, nodes, w) || sipg_oracle_dphi(p, D)) {
    g_err = "table construction failed";
    return 1;
  }
  TRY(cudaMemcpy(g_nodes, nodes, sizeof(double) * (p + 1), cudaMemcpyHostToDevice));
  TRY(cudaMemcpy(g_weights, w, sizeof(double) * (p + 1), cudaMemcpyHostToDevice));
  TRY(cudaMemcpy(g_dphi, D, sizeof(double) * (p + 1) * (p + 1), cudaMemcpyHostToDevice));
  return 0;
}

int launch_mvm(int p, int dim, double pen, const double* in, double* out, cudaStream_t s) {
  const int noe = dim * dim;
  RefModeVector vin{noe, p + 1, const_cast<double*>(in)}, vout{noe, p + 1, out};
  RefQuadMesh mesh{dim, dim, noe, nullptr, nullptr};  // the flux kernels never read the coordinates
  int N = p;
  const int blockD = 128;
  dim3 vg((noe + blockD - 1) / blockD, p + 1, p + 1), vb(blockD, 1, 1);
  void* vargs[] = {&N, &vin, &vout};
  TRY(cudaLaunchKernel((const void*)g_volume, vg, vb, vargs, 0, s));
  dim3 fg((dim + 31) / 32, (dim + 3) / 4, 1), fb(32, 4, 1);
  void* fargs[] = {&N, &mesh, &vin, &vout, &pen};
  TRY(cudaLaunchKernel((const void*)g_flux6a, fg, fb, fargs, 0, s));
  TRY(cudaLaunchKernel((const void*)g_flux6b, fg, fb, fargs, 0, s));
  return 0;
}

}  // namespace

extern "C" {

const char* refgpu_last_error(void) { return g_err.c_str(); }

int refgpu_init(const char* cubin) {
  if (g_lib) return 0;
  TRY(cudaLibraryLoadFromFile(&g_lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0));
  TRY(cudaLibraryGetKernel(&g_volume, g_lib, "_Z6volumeIdEvi11mode_vectorIT_iES2_"));
  TRY(cudaLibraryGetKernel(&g_flux6a, g_lib, "_Z11flux_term6aIdEvi23quadrilateral_mesh_infoIT_E11mode_vectorIS1_iES4_S1_"));
  TRY(cudaLibraryGetKernel(&g_flux6b, g_lib, "_Z11flux_term6bIdEvi23quadrilateral_mesh_infoIT_E11mode_vectorIS1_iES4_S1_"));
  TRY(cudaLibraryGetKernel(&g_alpha, g_lib, "_Z12alpha_kernelIdEviPT_S1_S1_S1_S0_"));
  TRY(cudaLibraryGetKernel(&g_beta, g_lib, "_Z11beta_kernelIdEviPT_S1_S0_"));
  size_t bytes = 0;
  TRY(cudaLibraryGetGlobal(&g_dphi, &bytes, g_lib, "d_dphi_double"));
  TRY(cudaLibraryGetGlobal(&g_weights, &bytes, g_lib, "d_lgl_weights_double"));
  TRY(cudaLibraryGetGlobal(&g_nodes, &bytes, g_lib, "d_lgl_nodes_double"));
  return 0;
}

/* out = A in with the reference kernels, `reps` times; *ms = elapsed device time. */
int refgpu_apply(int p, int dim, double pen, const double* d_in, double* d_out, int reps, float* ms) {
  if (!g_lib || p < 1 || p > 32 || dim < 1 || reps < 1) {
    g_err = "refgpu_apply: not initialised or bad arguments";
    return 1;
  }
  if (int e = load_tables(p)) return e;
  cudaEvent_t e0, e1;
  TRY(cudaEventCreate(&e0));
  TRY(cudaEventCreate(&e1));
  if (int e = launch_mvm(p, dim, pen, d_in, d_out, 0)) return e;  // warm-up
  TRY(cudaEventRecord(e0, 0));
  for (int r = 0; r < reps; ++r)
    if (int e = launch_mvm(p, dim, pen, d_in, d_out, 0)) return e;
  TRY(cudaEventRecord(e1, 0));
  TRY(cudaEventSynchronize(e1));
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TRY(cudaGetLastError());
  return 0;
}

/* The reference CG host loop (absolute tolerance on sqrt(r.r), max_it = DoF)
 * around the reference kernels and cuBLAS dots.  x holds x0 on entry. */
int refgpu_cg(int p, int dim, double pen, double* d_x, const double* d_b, double tol, int* iterations, float* ms) {
  if (!g_lib) {
    g_err = "refgpu_cg: not initialised";
    return 1;
  }
  if (int e = load_tables(p)) return e;
  const int noe = dim * dim, n = noe * (p + 1) * (p + 1);
  double *r = nullptr, *pv = nullptr, *Ap = nullptr;
  TRY(cudaMalloc(&r, sizeof(double) * n));
  TRY(cudaMalloc(&pv, sizeof(double) * n));
  TRY(cudaMalloc(&Ap, sizeof(double) * n));
  cublasHandle_t h;
  if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) {
    g_err = "cublasCreate failed";
    return 1;
  }
  cudaEvent_t e0, e1;
  TRY(cudaEventCreate(&e0));
  TRY(cudaEventCreate(&e1));
  TRY(cudaEventRecord(e0, 0));
  const int blockD = 128, grid = (n + blockD - 1) / blockD;
  double rr_old = 0, rr_new = 0, pAp = 0, norm_b = 0;
  cublasDdot(h, n, d_b, 1, d_b, 1, &norm_b);
  if (int e = launch_mvm(p, dim, pen, d_x, r, 0)) return e;
  {
    int size = n;
    double m1 = -1.0;
    const double* bb = d_b;
    void* a[] = {&size, &r, &bb, &m1};
    TRY(cudaLaunchKernel((const void*)g_beta, dim3(grid), dim3(blockD), a, 0, 0));
  }
  TRY(cudaMemcpy(pv, r, sizeof(double) * n, cudaMemcpyDeviceToDevice));
  cublasDdot(h, n, r, 1, r, 1, &rr_old);
  int it = 0;
  while (std::sqrt(rr_old) > tol && it < n) {
    if (int e = launch_mvm(p, dim, pen, pv, Ap, 0)) return e;
    cublasDdot(h, n, pv, 1, Ap, 1, &pAp);
    double alpha = rr_old / pAp;
    int size = n;
    void* a[] = {&size, &d_x, &pv, &r, &Ap, &alpha};
    TRY(cudaLaunchKernel((const void*)g_alpha, dim3(grid), dim3(blockD), a, 0, 0));
    cublasDdot(h, n, r, 1, r, 1, &rr_new);
    double beta = rr_new / rr_old;
    void* bargs[] = {&size, &pv, &r, &beta};
    TRY(cudaLaunchKernel((const void*)g_beta, dim3(grid), dim3(blockD), bargs, 0, 0));
    rr_old = rr_new;
    ++it;
  }
  TRY(cudaEventRecord(e1, 0));
  TRY(cudaEventSynchronize(e1));
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  *iterations = it;
  cublasDestroy(h);
  cudaFree(r);
  cudaFree(pv);
  cudaFree(Ap);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TRY(cudaGetLastError());
  return 0;
}
}
