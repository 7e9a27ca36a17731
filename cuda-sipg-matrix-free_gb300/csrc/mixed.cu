// mixed.cu -- the mixed-precision solve (no counterpart in the reference):
// an inner CG on the FP32 pipes inside FP64 defect correction with reliable
// updates.
//
// FP64 part: the solution x, b, the true residual r = b - A x (fused FP64
// apply, APPLY_RESID) and the outer norms, all on the device.  Inner part: a
// CG on the correction e ~ A^-1 r in one of two formats (sipg_inner_kind):
//   * INNER_F32: FP32 vectors and the FP32 apply;
//   * INNER_PAIRS: double-float pair vectors (two FP32 planes) and the
//     compensated apply (sipg_apply_df.cuh) -- FP32 instructions only, ~48
//     significant bits.
// FP32 vectors fail on this operator once its condition number approaches
// 1 / eps_32: the rounding noise of a smooth FP32 vector is spread over all
// frequencies, A amplifies it by up to kappa, and each step's correction then
// carries a residual error as large as the residual it removes (measured: 512
// x 512, p = 6, kappa ~ 2e7, no convergence in 190,000 FP32 iterations).
// Pairs push that limit to kappa ~ 1e12.
//
// Whenever the inner residual has fallen by `inner_tol` relative to its
// largest value since the last update (sqrt(r.r) < inner_tol * rmax) or after
// kCorrectEvery inner iterations, e is folded into x in FP64, r is recomputed
// in FP64 and rounded into the inner residual, and the inner CG *continues
// with its search direction* (beta = r_new.r_new / r_prev.r_prev): the
// reliable-update scheme of Sleijpen & van der Vorst (1996), as used for
// mixed-precision CG on GPUs by Clark et al. (2010).
//
// The flexible outer kind (SIPG_OUTER_FLEXIBLE) replaces the unit-step
// correction by flexible CG in FP64 (Notay, SIAM J. Sci. Comput. 22, 2000;
// FCG(1): each direction A-orthogonal to the previous one) whose
// preconditioner is the FP32 inner CG, run from zero on r / ||r|| until its
// residual fell by inner_tol.  One outer step:
//   z = ||r|| e                      (e: the FP32 inner solution)
//   gamma = z.q_prev / d_prev.q_prev,  d = z - gamma d_prev,  d.r
//   q = A d (FP64 apply),  alpha = d.r / d.q
//   x += alpha d,  r -= alpha q,  r.r           (all FP64)
// and, once ||r|| reaches the target, r = b - A x recomputed in FP64 (the
// recursion's drift) before the solve may stop.  Why FP32 suffices here but
// not for the unit step: the line search measures the correction in the
// energy norm, in which rounding a smooth correction to FP32 is an error of
// relative size ~sqrt(kappa) eps_32 (3e-4 at kappa = 2e7), while the residual
// norm sees ~kappa eps_32 (~1).
#include <cmath>
#include <new>

#include "sipg_apply_df.cuh"
#include "sipg_cg_df.cuh"
#include "sipg_fcg.cuh"

using namespace sipg;

namespace sipg {
// inner iterations after which an FP64 update is forced
constexpr int kCorrectEvery = 1000;

template <int KIND>
__global__ void __launch_bounds__(kVecThreads)
    k_mixed_restart(const double* __restrict__ r64, float* __restrict__ r, float* __restrict__ e, size_t n,
                    CgState<typename InnerScalar<KIND>::type>* st, ReduceScratch red, int first, double delta,
                    double stop, int max_it) {
  inner_restart_body<KIND>(r64, r, e, n, st, red, first, delta, stop, max_it, blockIdx.x, gridDim.x);
}

template <int KIND>
__global__ void __launch_bounds__(kVecThreads) k_mixed_fold(double* __restrict__ x, const float* __restrict__ e,
                                                            size_t n) {
  inner_fold_body<KIND>(x, e, n, blockIdx.x, gridDim.x);
}

// the FP64 kind: r = r64, e = 0, state as inner_restart_body
__global__ void __launch_bounds__(kVecThreads)
    k_mixed_restart_f64(const double* __restrict__ r64, double* __restrict__ r, double* __restrict__ e, size_t n,
                        CgState<double>* st, ReduceScratch red, int first, double delta, double stop, int max_it) {
  __shared__ double sh[32];
  double acc = 0.0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double v = r64[i];
    r[i] = v;
    e[i] = 0.0;
    acc = fma(v, v, acc);
  }
  const double bt = block_sum<double, kVecThreads>(acc, sh);
  double total;
  if (grid_sum_last<double, kVecThreads>(bt, red, gridDim.x, sh, &total) && threadIdx.x == 0) {
    if (first) {
      st->first = 1;
      st->it = 0;
      st->parity = 0;
      st->beta = 0.0;
      st->status = (int)SIPG_OK;
    } else {
      st->beta = total / st->rr_prev;
      st->first = 0;
    }
    st->rr = total;
    st->rmax = sqrt(total);
    st->delta = delta;
    st->stop = stop;
    st->max_it = st->it + max_it;
    st->need_update = 0;
    st->done = (total == 0.0) ? 1 : 0;
  }
}

__global__ void __launch_bounds__(kVecThreads) k_mixed_fold_f64(double* __restrict__ x, const double* __restrict__ e,
                                                                size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] += e[i];
}

// Condition-number estimate kappa ~ c_p dim^2 (penalty p^2; grows with larger
// penalties), from the extreme eigenvalues of the assembled operator at
// dim = 8 (the ratio kappa(8) / kappa(4) is 3.9-4.0 for every p).
double kappa_estimate(int p, int dim, double pen) {
  static const double c[9] = {0, 0.81, 4.76, 12.0, 25.9, 45.7, 75.6, 114.1, 167.1};
  const double pp = (double)p * p;
  const double scale = pen > pp ? pen / pp : 1.0;
  return c[p < 1 ? 1 : (p > 8 ? 8 : p)] * (double)dim * dim * scale;
}

int choose_inner(int requested, int p, int dim, double pen) {
  if (requested == SIPG_INNER_F32 || requested == SIPG_INNER_PAIRS || requested == SIPG_INNER_F64) return requested;
  return kappa_estimate(p, dim, pen) * std::ldexp(1.0, -24) < 0.01 ? SIPG_INNER_F32 : SIPG_INNER_PAIRS;
}
}  // namespace sipg

namespace {
// Everything one mixed solve on an op needs on the device, kept in the op
// between solves.  Inner vectors are 8 n bytes (pairs: 2 n floats; FP64: n
// doubles; FP32: the first n floats); one K-iteration graph per inner kind
// (its kernels read x only through the fold, outside the graph).
struct MixedCache {
  size_t n = 0;
  double* r64 = nullptr;
  float* r = nullptr;
  float* e = nullptr;
  float* p[2] = {nullptr, nullptr};
  float* Ap = nullptr;
  float* z = nullptr;  // two-level inner kind: z = M r
  int* nz = nullptr;       // set-up: 1 if the start vector has a non-zero entry
  int* nz_host = nullptr;
  CgState<double>* st64 = nullptr;
  CgState<float>* st32 = nullptr;   // inner state, FP32 kind
  CgState<double>* stp = nullptr;   // inner state, pairs kind
  CgState<double>* st64_host = nullptr;
  CgState<float>* st32_host = nullptr;
  CgState<double>* stp_host = nullptr;
  ReduceScratch red64{}, red32{};
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int exec_k[5] = {0, 0, 0, 0, 0};
  int exec_gen[5] = {-1, -1, -1, -1, -1};
  unsigned long long exec_launches[5] = {0, 0, 0, 0, 0};  // kernel launches one replay makes
  void* tl = nullptr;  // the op's two-level preconditioner (owned by the op)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // flexible outer kind (allocated on its first use): the FP64 direction d and
  // q = A d, and its scalars
  double* d64 = nullptr;
  double* q64 = nullptr;
  FcgState* fs = nullptr;
  ~MixedCache() {
    cudaFree(d64);
    cudaFree(q64);
    cudaFree(fs);
    for (cudaGraphExec_t g : exec)
      if (g) cudaGraphExecDestroy(g);
    if (cap) cudaStreamDestroy(cap);
    cudaFree(r64);
    cudaFree(r);
    cudaFree(e);
    cudaFree(p[0]);
    cudaFree(p[1]);
    cudaFree(Ap);
    cudaFree(z);
    cudaFree(nz);
    cudaFreeHost(nz_host);
    cudaFree(st64);
    cudaFree(st32);
    cudaFree(stp);
    cudaFreeHost(st64_host);
    cudaFreeHost(st32_host);
    cudaFreeHost(stp_host);
    cudaFree(red64.partials);
    cudaFree(red64.counter);
    cudaFree(red32.partials);
    cudaFree(red32.counter);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};

void mixed_cache_free(void* p) { delete static_cast<MixedCache*>(p); }

sipg_status fcg_alloc(MixedCache& m) {
  if (m.fs) return SIPG_OK;
  SIPG_CUDA_TRY(cudaMalloc(&m.d64, m.n * sizeof(double)));
  SIPG_CUDA_TRY(cudaMalloc(&m.q64, m.n * sizeof(double)));
  SIPG_CUDA_TRY(cudaMalloc(&m.fs, sizeof(FcgState)));
  SIPG_CUDA_TRY(cudaMemset(m.fs, 0, sizeof(FcgState)));
  return SIPG_OK;
}

int vec_grid(size_t n) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + kVecThreads - 1) / kVecThreads, 152 * 8));
}

sipg_status cache_alloc(MixedCache& m, size_t n, int cap) {
  m.n = n;
  const size_t pair_bytes = 2 * n * sizeof(float);
  SIPG_CUDA_TRY(cudaMalloc(&m.r64, n * sizeof(double)));
  SIPG_CUDA_TRY(cudaMalloc(&m.r, pair_bytes));
  SIPG_CUDA_TRY(cudaMalloc(&m.e, pair_bytes));
  SIPG_CUDA_TRY(cudaMalloc(&m.p[0], pair_bytes));
  SIPG_CUDA_TRY(cudaMalloc(&m.p[1], pair_bytes));
  SIPG_CUDA_TRY(cudaMalloc(&m.Ap, pair_bytes));
  SIPG_CUDA_TRY(cudaMalloc(&m.st64, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMalloc(&m.st32, sizeof(CgState<float>)));
  SIPG_CUDA_TRY(cudaMalloc(&m.stp, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMallocHost(&m.st64_host, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMallocHost(&m.st32_host, sizeof(CgState<float>)));
  SIPG_CUDA_TRY(cudaMallocHost(&m.stp_host, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMalloc(&m.nz, sizeof(int)));
  SIPG_CUDA_TRY(cudaMallocHost(&m.nz_host, sizeof(int)));
  ReduceScratch* reds[2] = {&m.red64, &m.red32};
  for (ReduceScratch* r : reds) {
    SIPG_CUDA_TRY(cudaMalloc(&r->partials, sizeof(double) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&r->counter, sizeof(unsigned int)));
    SIPG_CUDA_TRY(cudaMemset(r->counter, 0, sizeof(unsigned int)));
    r->capacity = cap;
  }
  SIPG_CUDA_TRY(cudaMemset(m.st64, 0, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaMemset(m.st32, 0, sizeof(CgState<float>)));
  SIPG_CUDA_TRY(cudaMemset(m.stp, 0, sizeof(CgState<double>)));
  SIPG_CUDA_TRY(cudaStreamCreateWithFlags(&m.cap, cudaStreamNonBlocking));
  SIPG_CUDA_TRY(cudaEventCreate(&m.ev0));
  SIPG_CUDA_TRY(cudaEventCreate(&m.ev1));
  return SIPG_OK;
}

sipg_status cache_get(sipg_op* op, MixedCache** out) {
  std::lock_guard<std::mutex> lk(op->mu);
  if (!op->mixed) {
    MixedCache* m = new (std::nothrow) MixedCache;
    if (!m) return SIPG_ERR_NOMEM;
    const sipg_status st = cache_alloc(*m, (size_t)op->ndof, reduce_capacity(op->dim));
    if (st != SIPG_OK) {
      delete m;
      return st;
    }
    op->mixed = m;
    op->mixed_free = mixed_cache_free;
  }
  *out = static_cast<MixedCache*>(op->mixed);
  return SIPG_OK;
}

// One inner iteration: apply in CG mode (p = r + beta p_old, A p, p.Ap,
// alpha), then e += alpha p, r -= alpha Ap, r.r, beta, stop test.
sipg_status enqueue_iteration(sipg_op* op, MixedCache& m, int kind, cudaStream_t s) {
  ApplyArgs<float> a{};
  a.in = m.r;
  a.pbuf0 = m.p[0];
  a.pbuf1 = m.p[1];
  a.out = m.Ap;
  a.dim = op->dim;
  a.nu = (float)op->pen;
  a.st = m.st32;
  a.red = m.red32;
  if (kind == SIPG_INNER_F32_TWOLEVEL) {
    // z = M r (two-level, from the corner sums of r that the restart or the
    // previous update left; r.z and beta), p = z + beta p, Ap and alpha;
    // then e += alpha p, r -= alpha Ap, the stop test on r.r and the corner
    // sums of the new r.  (Forming p inside the apply, its CG mode, was
    // slower: the FP32 apply is issue-bound and the second input vector
    // costs it more than the separate pass over p and z.)
    sipg_status pst = twolevel_enqueue(op, m.tl, m.r, m.z, m.st32, m.red32, s, true);
    if (pst != SIPG_OK) return pst;
    k_cg_direction<float><<<vec_grid(m.n), kVecThreads, 0, s>>>(m.p[0], m.z, m.n, m.st32);
    count_launch();
    a.in = m.p[0];
    SIPG_CUDA_TRY(launch_apply_f32(op->p, op->cfg32, APPLY_DOT, a, op->tab, s));
    pst = twolevel_enqueue_update(op, m.tl, m.e, m.p[0], m.p[0], m.r, m.Ap, m.st32, m.red32, s);
    if (pst != SIPG_OK) return pst;
    return SIPG_OK;
  } else if (kind == SIPG_INNER_F64) {
    k_cg_direction<double><<<vec_grid(m.n), kVecThreads, 0, s>>>((double*)m.p[0], (const double*)m.r, m.n, m.stp);
    count_launch();
    ApplyArgs<double> d{};
    d.in = (const double*)m.p[0];
    d.out = (double*)m.Ap;
    d.dim = op->dim;
    d.nu = op->pen;
    d.st = m.stp;
    d.red = m.red32;
    SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_DOT, d, op->tab, s));
    k_cg_update<double><<<vec_grid(m.n), kVecThreads, 0, s>>>((double*)m.e, (const double*)m.p[0],
                                                              (const double*)m.p[0], (double*)m.r,
                                                              (const double*)m.Ap, m.n, m.stp, m.red32);
  } else if (kind == SIPG_INNER_PAIRS) {
    // p = r + beta p (in place), then Ap and alpha, then the update
    k_cg_direction_pairs<<<vec_grid(m.n), kVecThreads, 0, s>>>(m.p[0], m.r, m.n, m.stp);
    count_launch();
    a.in = m.p[0];
    set_penalty3(a, op->pen);
    a.st = nullptr;
    a.stp = m.stp;
    SIPG_CUDA_TRY(launch_apply_df(op->p, op->cfgdf, APPLY_DOT, a, nullptr, nullptr, 0, 0, op->tab, s));
    k_cg_update_pairs<<<vec_grid(m.n), kVecThreads, 0, s>>>(m.e, m.p[0], m.p[0], m.r, m.Ap, m.n, m.stp, m.red32);
  } else {
    k_cg_direction<float><<<vec_grid(m.n), kVecThreads, 0, s>>>(m.p[0], m.r, m.n, m.st32);
    count_launch();
    a.in = m.p[0];
    SIPG_CUDA_TRY(launch_apply_f32(op->p, op->cfg32, APPLY_DOT, a, op->tab, s));
    k_cg_update<float><<<vec_grid(m.n), kVecThreads, 0, s>>>(m.e, m.p[0], m.p[0], m.r, m.Ap, m.n, m.st32, m.red32);
  }
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  return SIPG_OK;
}

sipg_status capture(sipg_op* op, MixedCache& m, int kind, int K) {
  if (m.exec[kind] && m.exec_k[kind] == K && m.exec_gen[kind] == op->tile_gen) return SIPG_OK;
  if (m.exec[kind]) {
    cudaGraphExecDestroy(m.exec[kind]);
    m.exec[kind] = nullptr;
  }
  ApplyArgs<float> none{};
  none.dim = op->dim;
  if (kind == SIPG_INNER_F64) {
    ApplyArgs<double> prep{};
    prep.dim = op->dim;
    SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_PREPARE, prep, op->tab, m.cap));
  } else if (kind == SIPG_INNER_PAIRS) {
    SIPG_CUDA_TRY(launch_apply_df(op->p, op->cfgdf, APPLY_PREPARE, none, nullptr, nullptr, 0, 0, op->tab, m.cap));
  }
  else
    SIPG_CUDA_TRY(launch_apply_f32(op->p, op->cfg32, APPLY_PREPARE, none, op->tab, m.cap));
  SIPG_CUDA_TRY(cudaStreamBeginCapture(m.cap, cudaStreamCaptureModeThreadLocal));
  sipg_status st = SIPG_OK;
  // the launches counted while capturing are the graph's, not executed ones
  const unsigned long long c0 = g_launches.load();
  for (int k = 0; k < K && st == SIPG_OK; ++k) st = enqueue_iteration(op, m, kind, m.cap);
  const unsigned long long c1 = g_launches.load();
  g_launches.fetch_sub(c1 - c0);
  m.exec_launches[kind] = c1 - c0;
  cudaGraph_t g = nullptr;
  const cudaError_t end = cudaStreamEndCapture(m.cap, &g);
  if (st != SIPG_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  SIPG_CUDA_TRY(end);
  const cudaError_t inst = cudaGraphInstantiate(&m.exec[kind], g, 0);
  cudaGraphDestroy(g);
  SIPG_CUDA_TRY(inst);
  m.exec_k[kind] = K;
  m.exec_gen[kind] = op->tile_gen;
  return SIPG_OK;
}
}  // namespace

namespace {
// What both outer kinds share for one solve.
struct Solve {
  sipg_op* op;
  MixedCache* m;
  double* x;
  const double* b;
  cudaStream_t s;
  size_t n;
  int vb;    // vector-kernel grid
  int K;     // inner iterations per graph launch
  double bnorm;
  // results
  int outer = 0;
  long long inner_total = 0;
  int fp64_applies = 0;
  double rel = INFINITY;
  bool x_zero = false;  // the start vector is zero (its residual needs no apply)
};

// The state after r = b - A x with x = 0: r.r = b.b (k_cg_init left it in bb).
__global__ void k_resid_of_zero(CgState<double>* st) { apply_finish<double, APPLY_RESID>(st, st->bb, 0); }

// flag = 1 if any x_i != 0 (every writer stores the same value)
__global__ void __launch_bounds__(kVecThreads) k_any_nonzero(const double* __restrict__ x, size_t n, int* flag) {
  bool nz = false;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    nz = nz || x[i] != 0.0;
  if (__syncthreads_or(nz) && threadIdx.x == 0) *flag = 1;
}

// r64 = b - A x in FP64 (r.r into st64, it = 0), read back: with the
// pivoted sums (APPLY_RESID_PIVOT), or the plain ones for the all-FP64
// reliable-update yardstick, whose inner iterations run the plain FP64 apply
// (checking them against the other rounding floor would only slow it down).
sipg_status true_residual(Solve& v, double* rr_out, bool plain = false) {
  MixedCache& m = *v.m;
  if (v.x_zero) {
    // x = 0: r = b exactly, r.r = b.b (from the set-up), no apply
    v.x_zero = false;
    SIPG_CUDA_TRY(cudaMemcpyAsync(m.r64, v.b, v.n * sizeof(double), cudaMemcpyDeviceToDevice, v.s));
    k_resid_of_zero<<<1, 1, 0, v.s>>>(m.st64);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    SIPG_CUDA_TRY(cudaMemcpyAsync(m.st64_host, m.st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, v.s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(v.s));
    *rr_out = m.st64_host->rr;
    return SIPG_OK;
  }
  ApplyArgs<double> a{};
  a.in = v.x;
  a.out = m.r64;
  a.b = v.b;
  a.dim = v.op->dim;
  a.nu = v.op->pen;
  a.st = m.st64;
  a.red = m.red64;
  SIPG_CUDA_TRY(launch_apply_f64(v.op->p, v.op->cfg64, plain ? APPLY_RESID : APPLY_RESID_PIVOT, a, v.op->tab, v.s));
  ++v.fp64_applies;
  SIPG_CUDA_TRY(cudaMemcpyAsync(m.st64_host, m.st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, v.s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(v.s));
  *rr_out = m.st64_host->rr;
  return SIPG_OK;
}

// Replays the inner K-iteration graph until the inner state says done.
template <typename StT>
sipg_status run_inner(Solve& v, int kind, StT* st_dev, StT* st_host) {
  for (;;) {
    SIPG_CUDA_TRY(cudaGraphLaunch(v.m->exec[kind], v.s));
    count_launch(v.m->exec_launches[kind]);
    SIPG_CUDA_TRY(cudaMemcpyAsync(st_host, st_dev, sizeof(StT), cudaMemcpyDeviceToHost, v.s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(v.s));
    if (st_host->done) return SIPG_OK;
  }
}

// Defect correction with reliable updates (see the top of this file).
sipg_status solve_reliable(Solve& v, int kind, const sipg_mixed_opts& o, long long max_inner) {
  MixedCache& m = *v.m;
  const size_t n = v.n;
  const int vb = v.vb;
  cudaStream_t s = v.s;
  // the inner loop may also stop once its own residual is under the target
  const double stop_in = 0.5 * o.outer_tol * (v.bnorm > 0 ? v.bnorm : 1.0);
  // the inner state as the host last read it
  const bool st_double = kind != SIPG_INNER_F32;  // pairs and FP64 keep FP64 scalars in stp
  auto inner_it = [&]() { return st_double ? m.stp_host->it : m.st32_host->it; };
  auto inner_status = [&]() { return st_double ? m.stp_host->status : m.st32_host->status; };
  for (;;) {
    double rr = 0;
    sipg_status st = true_residual(v, &rr, kind == SIPG_INNER_F64);
    if (st != SIPG_OK) return st;
    v.rel = (v.bnorm > 0) ? std::sqrt(rr) / v.bnorm : std::sqrt(rr);
    if (!std::isfinite(v.rel)) {
      set_error("sipg_solve_mixed: non-finite residual");
      return SIPG_ERR_BREAKDOWN;
    }
    if (v.rel <= o.outer_tol || rr == 0.0) return SIPG_OK;
    if (v.outer >= o.max_outer || v.inner_total >= max_inner) return SIPG_ERR_NOT_CONVERGED;
    // the inner residual and CG state; after the first update the direction is kept
    const int first = v.outer == 0;
    if (kind == SIPG_INNER_F64)
      k_mixed_restart_f64<<<vb, kVecThreads, 0, s>>>(m.r64, (double*)m.r, (double*)m.e, n, m.stp, m.red32, first,
                                                     o.inner_tol, stop_in, kCorrectEvery);
    else if (kind == SIPG_INNER_PAIRS)
      k_mixed_restart<INNER_PAIRS><<<vb, kVecThreads, 0, s>>>(m.r64, m.r, m.e, n, m.stp, m.red32, first,
                                                               o.inner_tol, stop_in, kCorrectEvery);
    else
      k_mixed_restart<INNER_F32><<<vb, kVecThreads, 0, s>>>(m.r64, m.r, m.e, n, m.st32, m.red32, first, o.inner_tol,
                                                             stop_in, kCorrectEvery);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    const int it_before = first ? 0 : inner_it();
    // inner iterations until an update is due (at most kCorrectEvery)
    st = st_double ? run_inner(v, kind, m.stp, m.stp_host) : run_inner(v, kind, m.st32, m.st32_host);
    if (st != SIPG_OK) return st;
    v.inner_total += inner_it() - it_before;
    if (inner_status() == (int)SIPG_ERR_BREAKDOWN) {
      set_error("sipg_solve_mixed: inner CG breakdown");
      return SIPG_ERR_BREAKDOWN;
    }
    if (kind == SIPG_INNER_F64)
      k_mixed_fold_f64<<<vb, kVecThreads, 0, s>>>(v.x, (const double*)m.e, n);
    else if (kind == SIPG_INNER_PAIRS)
      k_mixed_fold<INNER_PAIRS><<<vb, kVecThreads, 0, s>>>(v.x, m.e, n);
    else
      k_mixed_fold<INNER_F32><<<vb, kVecThreads, 0, s>>>(v.x, m.e, n);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    ++v.outer;
  }
}

// inner iterations one preconditioner solve of the flexible kind may take
constexpr int kFlexibleInnerCap = 4000;

// Flexible CG in FP64 with the FP32 inner CG as its preconditioner (see the
// top of this file).
sipg_status solve_flexible(Solve& v, int kind, const sipg_mixed_opts& o, long long max_inner) {
  MixedCache& m = *v.m;
  const size_t n = v.n;
  const int vb = v.vb;
  cudaStream_t s = v.s;
  sipg_status st = fcg_alloc(m);
  if (st != SIPG_OK) return st;
  double rr = 0;
  st = true_residual(v, &rr);
  if (st != SIPG_OK) return st;
  v.rel = (v.bnorm > 0) ? std::sqrt(rr) / v.bnorm : std::sqrt(rr);
  int first = 1;
  for (;;) {
    if (!std::isfinite(v.rel)) {
      set_error("sipg_solve_mixed: non-finite residual");
      return SIPG_ERR_BREAKDOWN;
    }
    if (v.rel <= o.outer_tol || rr == 0.0) return SIPG_OK;
    if (v.outer >= o.max_outer || v.inner_total >= max_inner) return SIPG_ERR_NOT_CONVERGED;
    // z ~ A^-1 r: the FP32 inner CG from zero on r / ||r||
    k_fcg_restart<<<vb, kVecThreads, 0, s>>>(m.r64, m.r, m.e, n, m.st64, m.fs, m.st32, m.red32, (float)o.inner_tol,
                                             kFlexibleInnerCap);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    if (kind == SIPG_INNER_F32_TWOLEVEL) {
      st = twolevel_enqueue_restrict(v.op, m.tl, m.r, s);
      if (st != SIPG_OK) return st;
    }
    st = run_inner(v, kind, m.st32, m.st32_host);
    if (st != SIPG_OK) return st;
    v.inner_total += m.st32_host->it;
    if (m.st32_host->it == 0) {
      // not one inner step (a breakdown at the first direction): no direction to search along
      set_error("sipg_solve_mixed: the FP32 inner CG made no step");
      return SIPG_ERR_BREAKDOWN;
    }
    // (an inner breakdown after some steps still leaves a usable direction)
    // d = z - gamma d_prev, q = A d, alpha = d.r / d.q, x += alpha d, r -= alpha q
    if (!first) {
      k_fcg_gamma<<<vb, kVecThreads, 0, s>>>(m.e, m.q64, n, m.st64, m.fs, m.red64);
      count_launch();
    }
    k_fcg_direction<<<vb, kVecThreads, 0, s>>>(m.e, m.d64, m.r64, n, m.st64, m.fs, m.red64, first);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    ApplyArgs<double> a{};
    a.in = m.d64;
    a.out = m.q64;
    a.dim = v.op->dim;
    a.nu = v.op->pen;
    a.st = m.st64;
    a.red = m.red64;
    SIPG_CUDA_TRY(
        launch_apply_f64(v.op->p, v.op->cfg64, v.rel > kFcgPivotRel ? APPLY_DOT_PIVOT : APPLY_DOT, a, v.op->tab, s));
    ++v.fp64_applies;
    k_cg_update<double><<<vb, kVecThreads, 0, s>>>(v.x, m.d64, m.d64, m.r64, m.q64, n, m.st64, m.red64);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    SIPG_CUDA_TRY(cudaMemcpyAsync(m.st64_host, m.st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
    ++v.outer;
    if (m.st64_host->status == (int)SIPG_ERR_BREAKDOWN) {
      set_error("sipg_solve_mixed: flexible CG breakdown (d.Ad <= 0 or a non-finite scalar)");
      return SIPG_ERR_BREAKDOWN;
    }
    rr = m.st64_host->rr;
    v.rel = (v.bnorm > 0) ? std::sqrt(rr) / v.bnorm : std::sqrt(rr);
    first = 0;
    if (v.rel <= o.outer_tol) {
      // the recursion says done: recompute b - A x in FP64; continue (a
      // fresh direction history) if the drift left it above the target
      st = true_residual(v, &rr);
      if (st != SIPG_OK) return st;
      v.rel = (v.bnorm > 0) ? std::sqrt(rr) / v.bnorm : std::sqrt(rr);
      first = 1;
    }
  }
}
}  // namespace

extern "C" sipg_status sipg_solve_mixed(sipg_op* op, double* d_x, const double* d_b, const sipg_mixed_opts* opts,
                                        sipg_mixed_result* res, void* stream) {
  if (!op || !d_x || !d_b) {
    set_error("sipg_solve_mixed: null argument");
    return SIPG_ERR_INVALID;
  }
  sipg_mixed_opts o = {0.1, 1e-10, 200, 0, SIPG_INNER_AUTO, SIPG_OUTER_AUTO};
  if (opts) o = *opts;
  if (!(o.inner_tol > 0) || !(o.inner_tol < 1) || !(o.outer_tol > 0) || o.max_outer < 1 || o.inner < 0 ||
      o.inner > 4 || o.outer < 0 || o.outer > 2) {
    set_error("sipg_solve_mixed: need 0 < inner_tol < 1, outer_tol > 0, max_outer >= 1, inner in 0..4, outer in 0..2");
    return SIPG_ERR_INVALID;
  }
  int outer = o.outer;
  if (outer == SIPG_OUTER_AUTO)
    outer = (o.inner == SIPG_INNER_PAIRS || o.inner == SIPG_INNER_F64) ? SIPG_OUTER_RELIABLE : SIPG_OUTER_FLEXIBLE;
  if (outer == SIPG_OUTER_FLEXIBLE && o.inner != SIPG_INNER_AUTO && o.inner != SIPG_INNER_F32 &&
      o.inner != SIPG_INNER_F32_TWOLEVEL) {
    set_error("sipg_solve_mixed: the flexible outer kind runs an FP32 inner CG (inner = AUTO, F32 or F32_TWOLEVEL)");
    return SIPG_ERR_INVALID;
  }
  if (outer == SIPG_OUTER_RELIABLE && o.inner == SIPG_INNER_F32_TWOLEVEL) {
    set_error("sipg_solve_mixed: the two-level-preconditioned inner CG runs under the flexible outer kind");
    return SIPG_ERR_INVALID;
  }
  const int kind = outer == SIPG_OUTER_FLEXIBLE
                       ? (o.inner == SIPG_INNER_F32 ? (int)SIPG_INNER_F32 : (int)SIPG_INNER_F32_TWOLEVEL)
                       : choose_inner(o.inner, op->p, op->dim, op->pen);
  cudaStream_t s = (cudaStream_t)stream;
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  const size_t n = (size_t)op->ndof;
  MixedCache* mp = nullptr;
  sipg_status st = cache_get(op, &mp);
  if (st != SIPG_OK) return st;
  MixedCache& m = *mp;
  if (kind == SIPG_INNER_F32_TWOLEVEL && !m.tl) {
    st = twolevel_get(op, &m.tl);
    if (st != SIPG_OK) return st;
  }
  if (kind == SIPG_INNER_F32_TWOLEVEL && !m.z) SIPG_CUDA_TRY(cudaMalloc(&m.z, n * sizeof(float)));
  const int K = n <= (1u << 20) ? 32 : 8;  // inner iterations per graph launch
  st = capture(op, m, kind, K);
  if (st != SIPG_OK) return st;
  const long long max_inner = o.max_inner > 0 ? o.max_inner : op->ndof;
  Solve v{op, &m, d_x, d_b, s, n, vec_grid(n), K, 0.0};
  SIPG_CUDA_TRY(cudaEventRecord(m.ev0, s));
  // ||b|| in FP64; the FP64 state's stop threshold outer_tol ||b||
  k_cg_init<double><<<v.vb, kVecThreads, 0, s>>>(d_b, n, m.st64, o.outer_tol, 1, 1 << 30, m.red64);
  SIPG_CUDA_TRY(cudaMemsetAsync(m.nz, 0, sizeof(int), s));
  k_any_nonzero<<<v.vb, kVecThreads, 0, s>>>(d_x, n, m.nz);
  count_launch(2);
  SIPG_CUDA_TRY(cudaGetLastError());
  SIPG_CUDA_TRY(cudaMemcpyAsync(m.st64_host, m.st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaMemcpyAsync(m.nz_host, m.nz, sizeof(int), cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  v.bnorm = std::sqrt(m.st64_host->bb);
  v.x_zero = *m.nz_host == 0;
  const sipg_status status = outer == SIPG_OUTER_FLEXIBLE ? solve_flexible(v, kind, o, max_inner)
                                                          : solve_reliable(v, kind, o, max_inner);
  if (status == SIPG_ERR_CUDA || status == SIPG_ERR_NOMEM) return status;
  SIPG_CUDA_TRY(cudaEventRecord(m.ev1, s));
  SIPG_CUDA_TRY(cudaEventSynchronize(m.ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, m.ev0, m.ev1);
  if (res) {
    res->outer_iterations = v.outer;
    res->inner_iterations = (int)v.inner_total;
    res->rel_residual = v.rel;
    res->time_ms = ms;
    res->converged = (status == SIPG_OK) ? 1 : 0;
    res->inner_kind = kind;
    res->outer_kind = outer;
    res->fp64_applies = v.fp64_applies;
  }
  return status;
}

extern "C" sipg_status sipg_residual_f64(sipg_op* op, const double* d_x, const double* d_b, double* d_r, double* rel,
                                         void* stream) {
  if (!op || !d_x || !d_b || !rel) {
    set_error("sipg_residual_f64: null argument");
    return SIPG_ERR_INVALID;
  }
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  MixedCache* mp = nullptr;
  sipg_status st = cache_get(op, &mp);
  if (st != SIPG_OK) return st;
  MixedCache& m = *mp;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t n = (size_t)op->ndof;
  k_cg_init<double><<<vec_grid(n), kVecThreads, 0, s>>>(d_b, n, m.st64, 0.0, 0, 1, m.red64);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  ApplyArgs<double> a{};
  a.in = d_x;
  a.out = d_r ? d_r : m.r64;
  a.b = d_b;
  a.dim = op->dim;
  a.nu = op->pen;
  a.st = m.st64;
  a.red = m.red64;
  SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_RESID_PIVOT, a, op->tab, s));
  SIPG_CUDA_TRY(cudaMemcpyAsync(m.st64_host, m.st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  const double bb = m.st64_host->bb, rr = m.st64_host->rr;
  *rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
  return SIPG_OK;
}
