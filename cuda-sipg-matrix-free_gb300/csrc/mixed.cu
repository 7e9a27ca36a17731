// mixed.cu -- FP32 CG inside FP64 defect correction (no counterpart in the
// reference), with reliable updates.
//
// The FP64 part: x (the solution), b, the true residual r = b - A x (fused
// FP64 apply, APPLY_RESID) and the outer norms, all on the device.  The FP32
// part: the CG iteration itself (fused FP32 apply and update, graph-captured)
// on a correction e ~ A^-1 r.  Whenever the FP32 iterated residual has fallen
// by `inner_tol` relative to its largest value since the last correction
// (sqrt(r32.r32) < inner_tol * rmax), the correction is folded into x in FP64
// (x += e), r is recomputed in FP64 and rounded into the FP32 residual, and the
// FP32 CG *continues with its search direction* (beta = r_new.r_new / r_old.r_old):
// the reliable-update scheme of Sleijpen & van der Vorst (1996), as used for
// mixed-precision CG on GPUs by Clark et al. (2010).  Restarting the FP32 CG
// from scratch at every correction instead (classic iterative refinement)
// loses the Krylov space and, on this operator (condition number ~ p^4 / h^2),
// needs two orders of magnitude more FP32 iterations.
#include <cmath>
#include <new>

#include "sipg_cg.cuh"

using namespace sipg;

namespace sipg {
// FP32 iterations after which an FP64 correction is forced
constexpr int kCorrectEvery = 1000;

cudaError_t launch_apply_f64(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>& a, const HostTables& h,
                             cudaStream_t s);

// r32 = (float) r64, e = 0, and the FP32 CG state for the next run of
// iterations: on the first call p = r; afterwards beta = r_new.r_new / r_old.r_old.
__global__ void __launch_bounds__(kVecThreads)
    k_mixed_restart(const double* __restrict__ r64, float* __restrict__ r32, float* __restrict__ e, size_t n,
                    CgState<float>* st, ReduceScratch red, int first, float delta, int max_it) {
  __shared__ float sh[32];
  float acc = 0.f;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float v = (float)r64[i];
    r32[i] = v;
    e[i] = 0.f;
    acc = fmaf(v, v, acc);
  }
  const float bt = block_sum<float, kVecThreads>(acc, sh);
  float total;
  if (grid_sum_last<float, kVecThreads>(bt, red, gridDim.x, sh, &total) && threadIdx.x == 0) {
    if (first) {
      st->first = 1;
      st->it = 0;
      st->parity = 0;
      st->beta = 0.f;
      st->status = (int)SIPG_OK;
    } else {
      st->beta = total / st->rr;
      st->first = 0;
    }
    st->rr = total;
    st->rmax = sqrtf(total);
    st->delta = delta;
    st->stop = 0.f;  // the FP32 loop stops only for corrections, breakdown or max_it
    // a correction is forced after max_it more FP32 iterations even if the
    // residual stagnates above delta * rmax (FP32 rounding floor)
    st->max_it = st->it + max_it;
    st->need_update = 0;
    st->done = 0;
  }
}

__global__ void __launch_bounds__(kVecThreads) k_fold_correction(double* __restrict__ x, const float* __restrict__ e,
                                                                 size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] += (double)e[i];
}
}  // namespace sipg

namespace {
struct MixedWorkspace {
  double* r64 = nullptr;
  float* e32 = nullptr;
  CgState<double>* st64 = nullptr;
  CgState<double>* st64_host = nullptr;
  CgState<float>* st32_host = nullptr;
  ReduceScratch red64, red32;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ~MixedWorkspace() {
    cudaFree(r64);
    cudaFree(e32);
    cudaFree(st64);
    cudaFreeHost(st64_host);
    cudaFreeHost(st32_host);
    cudaFree(red64.partials);
    cudaFree(red64.counter);
    cudaFree(red32.partials);
    cudaFree(red32.counter);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};

sipg_status alloc_workspace(MixedWorkspace& m, size_t n, int cap, cudaStream_t s) {
  SIPG_CUDA_TRY(cudaMalloc(&m.r64, n * sizeof(double)));
  SIPG_CUDA_TRY(cudaMalloc(&m.e32, n * sizeof(float)));
  SIPG_CUDA_TRY(cudaMalloc(&m.st64, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMallocHost(&m.st64_host, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMallocHost(&m.st32_host, sizeof(CgState<float>)));
  ReduceScratch* reds[2] = {&m.red64, &m.red32};
  for (ReduceScratch* r : reds) {
    SIPG_CUDA_TRY(cudaMalloc(&r->partials, sizeof(double) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&r->counter, sizeof(unsigned int)));
    SIPG_CUDA_TRY(cudaMemsetAsync(r->counter, 0, sizeof(unsigned int), s));
    r->capacity = cap;
  }
  SIPG_CUDA_TRY(cudaMemsetAsync(m.st64, 0, sizeof(CgState<double>), s));
  SIPG_CUDA_TRY(cudaEventCreate(&m.ev0));
  SIPG_CUDA_TRY(cudaEventCreate(&m.ev1));
  return SIPG_OK;
}
}  // namespace

extern "C" sipg_status sipg_solve_mixed(sipg_op* op, double* d_x, const double* d_b, const sipg_mixed_opts* opts,
                                        sipg_mixed_result* res, void* stream) {
  if (!op || !d_x || !d_b) {
    set_error("sipg_solve_mixed: null argument");
    return SIPG_ERR_INVALID;
  }
  sipg_mixed_opts o = {0.1, 1e-10, 200, 0};
  if (opts) o = *opts;
  if (!(o.inner_tol > 0) || !(o.inner_tol < 1) || !(o.outer_tol > 0) || o.max_outer < 1) {
    set_error("sipg_solve_mixed: need 0 < inner_tol < 1, outer_tol > 0, max_outer >= 1");
    return SIPG_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  const size_t n = (size_t)op->ndof;
  const int vb = (int)std::max<size_t>(1, std::min<size_t>((n + kVecThreads - 1) / kVecThreads, 152 * 8));
  MixedWorkspace mw;
  sipg_status st = alloc_workspace(mw, n, reduce_capacity(op->dim), s);
  if (st != SIPG_OK) return st;
  CgF32View v32;  // the op's FP32 CG workspace, iterating on the correction e
  st = cg_f32_prepare(op, mw.e32, &v32);
  if (st != SIPG_OK) return st;
  const long long max_inner = o.max_inner > 0 ? o.max_inner : op->ndof;
  SIPG_CUDA_TRY(cudaEventRecord(mw.ev0, s));

  // ||b|| in FP64
  k_cg_init<double><<<vb, kVecThreads, 0, s>>>(d_b, n, mw.st64, 0.0, 0, 1, mw.red64);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  SIPG_CUDA_TRY(cudaMemcpyAsync(mw.st64_host, mw.st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  const double bnorm = std::sqrt(mw.st64_host->bb);

  int corrections = 0;
  long long inner_total = 0;
  double rel = INFINITY;
  sipg_status status = SIPG_OK;
  for (;;) {
    // the true residual in FP64
    ApplyArgs<double> a{};
    a.in = d_x;
    a.out = mw.r64;
    a.b = d_b;
    a.dim = op->dim;
    a.nu = op->pen;
    a.st = mw.st64;
    a.red = mw.red64;
    SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_RESID, a, op->tab, s));
    SIPG_CUDA_TRY(cudaMemcpyAsync(mw.st64_host, mw.st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
    const double rr = mw.st64_host->rr;
    rel = (bnorm > 0) ? std::sqrt(rr) / bnorm : std::sqrt(rr);
    if (!std::isfinite(rel)) {
      set_error("sipg_solve_mixed: non-finite residual");
      status = SIPG_ERR_BREAKDOWN;
      break;
    }
    if (rel <= o.outer_tol || rr == 0.0) break;
    if (corrections >= o.max_outer || inner_total >= max_inner) {
      status = SIPG_ERR_NOT_CONVERGED;
      break;
    }
    // the FP32 residual and CG state; after the first correction the search
    // direction is kept
    k_mixed_restart<<<vb, kVecThreads, 0, s>>>(mw.r64, v32.r, mw.e32, n, v32.st, mw.red32, corrections == 0 ? 1 : 0,
                                               (float)o.inner_tol, kCorrectEvery);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    const int it_before = (corrections == 0) ? 0 : mw.st32_host->it;
    // FP32 iterations until a correction is due
    for (;;) {
      st = cg_f32_launch_chunk(op, s, mw.st32_host);
      if (st != SIPG_OK) return st;
      if (mw.st32_host->done) break;
    }
    inner_total += mw.st32_host->it - it_before;
    if (mw.st32_host->status == (int)SIPG_ERR_BREAKDOWN) {
      set_error("sipg_solve_mixed: FP32 CG breakdown");
      status = SIPG_ERR_BREAKDOWN;
      break;
    }
    k_fold_correction<<<vb, kVecThreads, 0, s>>>(d_x, mw.e32, n);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    ++corrections;
  }
  SIPG_CUDA_TRY(cudaEventRecord(mw.ev1, s));
  SIPG_CUDA_TRY(cudaEventSynchronize(mw.ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, mw.ev0, mw.ev1);
  if (res) {
    res->outer_iterations = corrections;
    res->inner_iterations = (int)inner_total;
    res->rel_residual = rel;
    res->time_ms = ms;
    res->converged = (status == SIPG_OK) ? 1 : 0;
  }
  return status;
}
