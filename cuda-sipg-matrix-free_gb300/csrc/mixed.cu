// mixed.cu -- FP32/FP64 defect correction (no counterpart in the reference):
//   r = b - A x           FP64 fused apply (APPLY_RESID), r.r reduced on device
//   stop if ||r|| <= outer_tol ||b||
//   c = r / ||r||         rounded to FP32 (scaled so FP32 sees O(1) values)
//   A d = c               FP32 CG, operator and accumulation in FP32, to inner_tol
//   x += ||r|| d          FP64
// x, b, r and every outer norm stay FP64 on the device; the only host traffic
// per outer step is one small state read to test convergence.
#include <cmath>
#include <new>

#include "sipg_cg.cuh"

using namespace sipg;

namespace sipg {
cudaError_t launch_apply_f64(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>& a, const HostTables& h,
                             cudaStream_t s);

__global__ void __launch_bounds__(kVecThreads) k_scale_to_f32(const double* __restrict__ r, float* __restrict__ c,
                                                              float* __restrict__ d, size_t n,
                                                              const CgState<double>* st) {
  const double inv = 1.0 / sqrt(st->rr);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    c[i] = (float)(r[i] * inv);
    d[i] = 0.0f;
  }
}

__global__ void __launch_bounds__(kVecThreads) k_correct_f64(double* __restrict__ x, const float* __restrict__ d,
                                                             size_t n, const CgState<double>* st) {
  const double s = sqrt(st->rr);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] = fma(s, (double)d[i], x[i]);
}
}  // namespace sipg

namespace {
struct MixedBuffers {
  double* r = nullptr;
  float* c = nullptr;
  float* d = nullptr;
  CgState<double>* st = nullptr;
  CgState<double>* st_host = nullptr;
  ReduceScratch red;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ~MixedBuffers() {
    cudaFree(r);
    cudaFree(c);
    cudaFree(d);
    cudaFree(st);
    cudaFreeHost(st_host);
    cudaFree(red.partials);
    cudaFree(red.counter);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};
}  // namespace

extern "C" sipg_status sipg_solve_mixed(sipg_op* op, double* d_x, const double* d_b, const sipg_mixed_opts* opts,
                                        sipg_mixed_result* res, void* stream) {
  if (!op || !d_x || !d_b) {
    set_error("sipg_solve_mixed: null argument");
    return SIPG_ERR_INVALID;
  }
  sipg_mixed_opts o = {1e-5, 1e-10, 50, 0};
  if (opts) o = *opts;
  if (!(o.inner_tol > 0) || !(o.outer_tol > 0) || o.max_outer < 1) {
    set_error("sipg_solve_mixed: tolerances must be positive and max_outer >= 1");
    return SIPG_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  const size_t n = (size_t)op->ndof;
  MixedBuffers mb;
  const int vb = (int)std::max<size_t>(1, std::min<size_t>((n + kVecThreads - 1) / kVecThreads, 152 * 8));
  const int cap = reduce_capacity(op->dim);
  SIPG_CUDA_TRY(cudaMalloc(&mb.r, n * sizeof(double)));
  SIPG_CUDA_TRY(cudaMalloc(&mb.c, n * sizeof(float)));
  SIPG_CUDA_TRY(cudaMalloc(&mb.d, n * sizeof(float)));
  SIPG_CUDA_TRY(cudaMalloc(&mb.st, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMallocHost(&mb.st_host, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMalloc(&mb.red.partials, sizeof(double) * cap));
  SIPG_CUDA_TRY(cudaMalloc(&mb.red.counter, sizeof(unsigned int)));
  SIPG_CUDA_TRY(cudaMemsetAsync(mb.red.counter, 0, sizeof(unsigned int), s));
  SIPG_CUDA_TRY(cudaMemsetAsync(mb.st, 0, sizeof(CgState<double>), s));
  mb.red.capacity = cap;
  SIPG_CUDA_TRY(cudaEventCreate(&mb.ev0));
  SIPG_CUDA_TRY(cudaEventCreate(&mb.ev1));
  SIPG_CUDA_TRY(cudaEventRecord(mb.ev0, s));

  // ||b|| in FP64 (k_cg_init also leaves stop = 0, so the residual launch never marks "done")
  k_cg_init<double><<<vb, kVecThreads, 0, s>>>(d_b, n, mb.st, 0.0, 0, 1, mb.red);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  SIPG_CUDA_TRY(cudaMemcpyAsync(mb.st_host, mb.st, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  const double bnorm = std::sqrt(mb.st_host->bb);

  int outer = 0, inner_total = 0;
  double rel = INFINITY;
  sipg_status status = SIPG_OK;
  for (;;) {
    ApplyArgs<double> a{};
    a.in = d_x;
    a.out = mb.r;
    a.b = d_b;
    a.dim = op->dim;
    a.nu = op->pen;
    a.st = mb.st;
    a.red = mb.red;
    SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_RESID, a, op->tab, s));
    SIPG_CUDA_TRY(cudaMemcpyAsync(mb.st_host, mb.st, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
    const double rr = mb.st_host->rr;
    rel = (bnorm > 0) ? std::sqrt(rr) / bnorm : std::sqrt(rr);
    if (!std::isfinite(rel)) {
      set_error("sipg_solve_mixed: non-finite residual");
      status = SIPG_ERR_BREAKDOWN;
      break;
    }
    if (rel <= o.outer_tol || rr == 0.0) break;
    if (outer >= o.max_outer) {
      status = SIPG_ERR_NOT_CONVERGED;
      break;
    }
    k_scale_to_f32<<<vb, kVecThreads, 0, s>>>(mb.r, mb.c, mb.d, n, mb.st);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    sipg_cg_result ir;
    sipg_status is = sipg_cg_f32(op, mb.d, mb.c, (float)o.inner_tol, 1, o.max_inner, &ir, stream);
    if (is == SIPG_ERR_BREAKDOWN) {
      status = is;
      break;
    }
    if (is != SIPG_OK && is != SIPG_ERR_NOT_CONVERGED) return is;
    inner_total += ir.iterations;
    k_correct_f64<<<vb, kVecThreads, 0, s>>>(d_x, mb.d, n, mb.st);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    ++outer;
  }
  SIPG_CUDA_TRY(cudaEventRecord(mb.ev1, s));
  SIPG_CUDA_TRY(cudaEventSynchronize(mb.ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, mb.ev0, mb.ev1);
  if (res) {
    res->outer_iterations = outer;
    res->inner_iterations = inner_total;
    res->rel_residual = rel;
    res->time_ms = ms;
    res->converged = (status == SIPG_OK) ? 1 : 0;
  }
  return status;
}
