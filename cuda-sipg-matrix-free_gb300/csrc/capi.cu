// capi.cu -- the C ABI (include/sipg_gb300.h): operator lifetime, the fused
// apply, the graph-driven conjugate gradient, host-buffer apply, tables.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "sipg_cg.cuh"

namespace sipg {

std::atomic<unsigned long long> g_launches{0};
static thread_local std::string t_last_error;
void set_error(const std::string& msg) { t_last_error = msg; }

cudaError_t launch_apply_f64_p1(const TileCfg&, int, const ApplyArgs<double>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f64_p1(const TileCfg&, int, const ApplyArgs<double>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f64_p2(const TileCfg&, int, const ApplyArgs<double>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f64_p2(const TileCfg&, int, const ApplyArgs<double>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f64_p3(const TileCfg&, int, const ApplyArgs<double>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f64_p3(const TileCfg&, int, const ApplyArgs<double>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f64_p4(const TileCfg&, int, const ApplyArgs<double>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f64_p4(const TileCfg&, int, const ApplyArgs<double>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f64_p5(const TileCfg&, int, const ApplyArgs<double>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f64_p5(const TileCfg&, int, const ApplyArgs<double>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f64_p6(const TileCfg&, int, const ApplyArgs<double>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f64_p6(const TileCfg&, int, const ApplyArgs<double>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f64_p7(const TileCfg&, int, const ApplyArgs<double>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f64_p7(const TileCfg&, int, const ApplyArgs<double>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f64_p8(const TileCfg&, int, const ApplyArgs<double>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f64_p8(const TileCfg&, int, const ApplyArgs<double>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f32_p1(const TileCfg&, int, const ApplyArgs<float>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f32_p1(const TileCfg&, int, const ApplyArgs<float>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f32_p2(const TileCfg&, int, const ApplyArgs<float>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f32_p2(const TileCfg&, int, const ApplyArgs<float>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f32_p3(const TileCfg&, int, const ApplyArgs<float>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f32_p3(const TileCfg&, int, const ApplyArgs<float>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f32_p4(const TileCfg&, int, const ApplyArgs<float>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f32_p4(const TileCfg&, int, const ApplyArgs<float>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f32_p5(const TileCfg&, int, const ApplyArgs<float>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f32_p5(const TileCfg&, int, const ApplyArgs<float>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f32_p6(const TileCfg&, int, const ApplyArgs<float>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f32_p6(const TileCfg&, int, const ApplyArgs<float>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f32_p7(const TileCfg&, int, const ApplyArgs<float>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f32_p7(const TileCfg&, int, const ApplyArgs<float>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);
cudaError_t launch_apply_f32_p8(const TileCfg&, int, const ApplyArgs<float>&, const HostTables&, cudaStream_t);
cudaError_t launch_apply_batched_f32_p8(const TileCfg&, int, const ApplyArgs<float>*, const int*, int, int,
                                          const HostTables&, cudaStream_t);

cudaError_t launch_apply_df_p1(const TileCfg&, int, const ApplyArgs<float>&, const ApplyArgs<float>*, const int*, int, int,
                                 const HostTables&, cudaStream_t);
cudaError_t launch_apply_df_p2(const TileCfg&, int, const ApplyArgs<float>&, const ApplyArgs<float>*, const int*, int, int,
                                 const HostTables&, cudaStream_t);
cudaError_t launch_apply_df_p3(const TileCfg&, int, const ApplyArgs<float>&, const ApplyArgs<float>*, const int*, int, int,
                                 const HostTables&, cudaStream_t);
cudaError_t launch_apply_df_p4(const TileCfg&, int, const ApplyArgs<float>&, const ApplyArgs<float>*, const int*, int, int,
                                 const HostTables&, cudaStream_t);
cudaError_t launch_apply_df_p5(const TileCfg&, int, const ApplyArgs<float>&, const ApplyArgs<float>*, const int*, int, int,
                                 const HostTables&, cudaStream_t);
cudaError_t launch_apply_df_p6(const TileCfg&, int, const ApplyArgs<float>&, const ApplyArgs<float>*, const int*, int, int,
                                 const HostTables&, cudaStream_t);
cudaError_t launch_apply_df_p7(const TileCfg&, int, const ApplyArgs<float>&, const ApplyArgs<float>*, const int*, int, int,
                                 const HostTables&, cudaStream_t);
cudaError_t launch_apply_df_p8(const TileCfg&, int, const ApplyArgs<float>&, const ApplyArgs<float>*, const int*, int, int,
                                 const HostTables&, cudaStream_t);

#define SIPG_DISPATCH_P(FN, P, ...) \
  switch (P) {                      \
    case 1: return FN##_p1(__VA_ARGS__); \
    case 2: return FN##_p2(__VA_ARGS__); \
    case 3: return FN##_p3(__VA_ARGS__); \
    case 4: return FN##_p4(__VA_ARGS__); \
    case 5: return FN##_p5(__VA_ARGS__); \
    case 6: return FN##_p6(__VA_ARGS__); \
    case 7: return FN##_p7(__VA_ARGS__); \
    case 8: return FN##_p8(__VA_ARGS__); \
  }                                 \
  return cudaErrorInvalidValue;

cudaError_t launch_apply_f64(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>& a, const HostTables& h,
                             cudaStream_t s) {
  SIPG_DISPATCH_P(launch_apply_f64, p, cfg, mode, a, h, s)
}
cudaError_t launch_apply_f32(int p, const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const HostTables& h,
                             cudaStream_t s) {
  SIPG_DISPATCH_P(launch_apply_f32, p, cfg, mode, a, h, s)
}
cudaError_t launch_apply_df(int p, const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const ApplyArgs<float>* insts,
                            const int* tile_start, int ninst, int total_tiles, const HostTables& h, cudaStream_t s) {
  SIPG_DISPATCH_P(launch_apply_df, p, cfg, mode, a, insts, tile_start, ninst, total_tiles, h, s)
}
cudaError_t launch_apply_batched_f64(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>* insts,
                                     const int* tile_start, int ninst, int total_tiles, const HostTables& h,
                                     cudaStream_t s) {
  SIPG_DISPATCH_P(launch_apply_batched_f64, p, cfg, mode, insts, tile_start, ninst, total_tiles, h, s)
}
cudaError_t launch_apply_batched_f32(int p, const TileCfg& cfg, int mode, const ApplyArgs<float>* insts,
                                     const int* tile_start, int ninst, int total_tiles, const HostTables& h,
                                     cudaStream_t s) {
  SIPG_DISPATCH_P(launch_apply_batched_f32, p, cfg, mode, insts, tile_start, ninst, total_tiles, h, s)
}

template <typename T>
cudaError_t launch_apply(const sipg_op* op, int mode, const ApplyArgs<T>& a, cudaStream_t s);
template <>
cudaError_t launch_apply<double>(const sipg_op* op, int mode, const ApplyArgs<double>& a, cudaStream_t s) {
  return launch_apply_f64(op->p, op->cfg64, mode, a, op->tab, s);
}
template <>
cudaError_t launch_apply<float>(const sipg_op* op, int mode, const ApplyArgs<float>& a, cudaStream_t s) {
  return launch_apply_f32(op->p, op->cfg32, mode, a, op->tab, s);
}

sipg_status rhs_f64(const sipg_op* op, int sol, const sipg_modes* modes, double* d_b, cudaStream_t s);
sipg_status err_norms_f64(const sipg_op* op, int sol, const sipg_modes* modes, const double* d_u, double* err,
                          cudaStream_t s);

// Default tile shapes: rows of 32 elements, TY rows per CTA; for FP64 on
// small meshes the per-node tile, which spreads the FP64 work over many more
// warps and SMs.
static TileCfg default_cfg(int p, int dim, bool f64) {
  TileCfg c;
  c.tx = 32;
  if (f64) {
    // 32 x TY tiles by measurement at ~16 M DoF, p = 1..8 (p = 4: 1024^2,
    // 24.5 GDoF/s with 8 rows against 23.9 with 4); TY = 2 at p = 6 and 8,
    // where a 32 x 4 tile's shared memory leaves too few CTAs per SM
    static const int kRows[9] = {4, 8, 8, 8, 8, 4, 2, 4, 2};
    c.ty = kRows[p >= 1 && p <= 8 ? p : 0];
    if (dim <= kPernodeDefaultDim) c = pernode_tile(p, dim <= kPernodeWideDim ? 0 : 1);
  } else {
    c.ty = (p == 1) ? 8 : 4;  // measured at ~16 M DoF (p = 4, 1024^2: 492 GDoF/s with 4 rows, 474 with 8)
  }
  return c;
}

static int vec_blocks(size_t n) {
  const size_t want = (n + kVecThreads - 1) / kVecThreads;
  return (int)std::max<size_t>(1, std::min<size_t>(want, 152 * 8));
}

}  // namespace sipg

using namespace sipg;

// CG workspace: vectors, device state, reduction scratch, the cached graph.
struct sipg_cg_workspace {
  int elem = 8;  // sizeof(T)
  size_t n = 0;
  void* r = nullptr;
  void* p[2] = {nullptr, nullptr};
  void* Ap = nullptr;
  void* bar = nullptr;     // the persistent small-mesh CG's barrier counter and abort flag
  void* st = nullptr;      // CgState<T>
  void* st_host = nullptr; // pinned mirror
  ReduceScratch red;
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* exec_x = nullptr;
  int exec_k = 0;
  int exec_gen = -1;  // the op's tile generation the graph was captured with
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

static void ws_free(sipg_cg_workspace* w) {
  if (!w) return;
  if (w->exec) cudaGraphExecDestroy(w->exec);
  cudaFree(w->r);
  cudaFree(w->p[0]);
  cudaFree(w->p[1]);
  cudaFree(w->Ap);
  cudaFree(w->bar);
  cudaFree(w->st);
  cudaFreeHost(w->st_host);
  cudaFree(w->red.partials);
  cudaFree(w->red.counter);
  if (w->cap) cudaStreamDestroy(w->cap);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

template <typename T>
static sipg_status ws_get(sipg_op* op, sipg_cg_workspace** out) {
  std::lock_guard<std::mutex> lk(op->mu);
  sipg_cg_workspace*& slot = (sizeof(T) == 8) ? op->ws64 : op->ws32;
  if (slot) {
    *out = slot;
    return SIPG_OK;
  }
  sipg_cg_workspace* w = new (std::nothrow) sipg_cg_workspace;
  if (!w) return SIPG_ERR_NOMEM;
  w->elem = sizeof(T);
  w->n = (size_t)op->ndof;
  const size_t bytes = w->n * sizeof(T);
  const TileCfg cfg = (sizeof(T) == 8) ? op->cfg64 : op->cfg32;
  (void)cfg;
  const int cap = reduce_capacity(op->dim);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&w->r, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&w->p[0], bytes);
  if (e == cudaSuccess) e = cudaMalloc(&w->p[1], bytes);
  if (e == cudaSuccess) e = cudaMalloc(&w->Ap, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&w->st, sizeof(CgState<T>));
  if (e == cudaSuccess) e = cudaMallocHost(&w->st_host, sizeof(CgState<T>));
  if (e == cudaSuccess) e = cudaMalloc(&w->red.partials, sizeof(double) * cap);
  if (e == cudaSuccess) e = cudaMalloc(&w->red.counter, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(w->red.counter, 0, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(w->st, 0, sizeof(CgState<T>));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&w->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev1);
  w->red.capacity = cap;
  if (e != cudaSuccess) {
    set_error(std::string("CG workspace allocation failed: ") + cudaGetErrorString(e));
    ws_free(w);
    return e == cudaErrorMemoryAllocation ? SIPG_ERR_NOMEM : SIPG_ERR_CUDA;
  }
  slot = w;
  *out = w;
  return SIPG_OK;
}

// Iterations per graph launch: small systems are launch-bound, so batch more.
static int graph_iters(long long ndof) { return ndof <= (1LL << 20) ? 32 : 8; }

// Capture K CG iterations (apply + update; the direction buffers alternate by
// the parity kept in the device state, so a chunk may stop at any iteration).
// Whether the CG iterations fuse the direction update into the apply
// (APPLY_CG: two kernels per iteration).  The per-node tile does: on the small
// meshes it serves, an iteration is a chain of short launches.  The
// element-per-thread tiles form the direction in a vector kernel instead
// (APPLY_DOT), so the apply reads one vector, not two.
template <typename T>
static bool cg_fused_direction(const sipg_op* op) {
  return sizeof(T) == 8 && is_pernode(op->cfg64, op->p);
}

template <typename T>
static sipg_status capture_iterations(sipg_op* op, sipg_cg_workspace* w, T* x, int K) {
  if (w->exec && w->exec_x == x && w->exec_k == K && w->exec_gen == op->tile_gen) return SIPG_OK;
  if (w->exec) {
    cudaGraphExecDestroy(w->exec);
    w->exec = nullptr;
  }
  {
    ApplyArgs<T> prep{};
    prep.dim = op->dim;
    SIPG_CUDA_TRY(launch_apply<T>(op, APPLY_PREPARE, prep, w->cap));
  }
  cudaGraph_t g = nullptr;
  SIPG_CUDA_TRY(cudaStreamBeginCapture(w->cap, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaSuccess;
  const int vb = vec_blocks(w->n);
  const bool fused = cg_fused_direction<T>(op);
  for (int k = 0; k < K && err == cudaSuccess; ++k) {
    ApplyArgs<T> a{};
    a.out = (T*)w->Ap;
    a.b = nullptr;
    a.dim = op->dim;
    a.nu = (T)op->pen;
    a.st = (CgState<T>*)w->st;
    a.red = w->red;
    if (fused) {
      // p_new = r + beta p_old, Ap, p.Ap, alpha in one kernel; x += alpha
      // p_new, r -= alpha Ap, r.r, beta in the next
      a.in = (const T*)w->r;
      a.pbuf0 = (T*)w->p[0];
      a.pbuf1 = (T*)w->p[1];
      err = launch_apply<T>(op, APPLY_CG, a, w->cap);
      if (err != cudaSuccess) break;
      k_cg_update<T><<<vb, kVecThreads, 0, w->cap>>>(x, (const T*)w->p[0], (const T*)w->p[1], (T*)w->r,
                                                     (const T*)w->Ap, w->n, (CgState<T>*)w->st, w->red);
    } else {
      // p = r + beta p; Ap, p.Ap, alpha; x += alpha p, r -= alpha Ap, r.r, beta
      k_cg_direction<T><<<vb, kVecThreads, 0, w->cap>>>((T*)w->p[0], (const T*)w->r, w->n, (CgState<T>*)w->st);
      err = cudaGetLastError();
      if (err != cudaSuccess) break;
      a.in = (const T*)w->p[0];
      err = launch_apply<T>(op, APPLY_DOT, a, w->cap);
      if (err != cudaSuccess) break;
      k_cg_update<T><<<vb, kVecThreads, 0, w->cap>>>(x, (const T*)w->p[0], (const T*)w->p[0], (T*)w->r,
                                                     (const T*)w->Ap, w->n, (CgState<T>*)w->st, w->red);
    }
    err = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamEndCapture(w->cap, &g);
  if (err != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    set_error(std::string("CG graph capture failed: ") + cudaGetErrorString(err != cudaSuccess ? err : e2));
    return SIPG_ERR_CUDA;
  }
  cudaError_t e3 = cudaGraphInstantiate(&w->exec, g, 0);
  cudaGraphDestroy(g);
  if (e3 != cudaSuccess) {
    w->exec = nullptr;
    set_error(std::string("CG graph instantiate failed: ") + cudaGetErrorString(e3));
    return SIPG_ERR_CUDA;
  }
  w->exec_x = x;
  w->exec_k = K;
  w->exec_gen = op->tile_gen;
  return SIPG_OK;
}

template <typename T>
static sipg_status cg_solve(sipg_op* op, T* x, const T* b, T tol, int rel, int max_it, sipg_cg_result* res,
                            cudaStream_t s) {
  if (!op || !x || !b) {
    set_error("sipg_cg: null argument");
    return SIPG_ERR_INVALID;
  }
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  sipg_cg_workspace* w = nullptr;
  sipg_status st = ws_get<T>(op, &w);
  if (st != SIPG_OK) return st;
  const long long mx = (max_it > 0) ? max_it : op->ndof;
  const int max_i = (int)std::min<long long>(mx, 2000000000LL);
  const int K = graph_iters(op->ndof);
  // small FP64 meshes on the per-node tile: one persistent kernel runs every
  // iteration (cg_small.cu); otherwise graphs of K iterations.  Measured at
  // p = 4: the persistent kernel is faster up to 32 x 32 (16^2: 1.80 against
  // 2.2 ms), slower at 64 x 64 (12.2 against 9.9 ms: hundreds of CTAs meet at
  // each grid barrier)
  const bool small = sizeof(T) == 8 && is_pernode(op->cfg64, op->p) && op->dim <= kSmallCgDim;
  if (!small) {
    st = capture_iterations<T>(op, w, x, K);
    if (st != SIPG_OK) return st;
  } else if (!w->bar) {
    SIPG_CUDA_TRY(cudaMalloc(&w->bar, 256));
  }
  SIPG_CUDA_TRY(cudaEventRecord(w->ev0, s));
  k_cg_init<T><<<vec_blocks(w->n), kVecThreads, 0, s>>>(b, w->n, (CgState<T>*)w->st, tol, rel, max_i, w->red);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  ApplyArgs<T> a{};
  a.in = x;
  a.out = (T*)w->r;
  a.b = b;
  a.dim = op->dim;
  a.nu = (T)op->pen;
  a.st = (CgState<T>*)w->st;
  a.red = w->red;
  SIPG_CUDA_TRY(launch_apply<T>(op, APPLY_RESID, a, s));
  CgState<T>* hs = (CgState<T>*)w->st_host;
  long long launched = 0;
  if (small) {
    SIPG_CUDA_TRY(cudaMemsetAsync(w->bar, 0, 256, s));
    SmallCgArgs g;
    g.x = (double*)x;
    g.r = (double*)w->r;
    g.p0 = (double*)w->p[0];
    g.p1 = (double*)w->p[1];
    g.Ap = (double*)w->Ap;
    g.st = (CgState<double>*)w->st;
    g.part_a = w->red.partials;
    g.part_b = w->red.partials + kSmallCgMaxBlocks;
    g.bar = (unsigned long long*)w->bar;
    g.abort = (int*)((char*)w->bar + 128);
    g.dim = op->dim;
    g.nu = op->pen;
    SIPG_CUDA_TRY(launch_cg_small(op->p, op->cfg64, g, op->tab, s));
    SIPG_CUDA_TRY(cudaMemcpyAsync(hs, w->st, sizeof(CgState<T>), cudaMemcpyDeviceToHost, s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs->status == (int)SIPG_ERR_CUDA) {
      set_error("sipg_cg: a grid barrier of the persistent CG gave up waiting");
      return SIPG_ERR_CUDA;
    }
  }
  for (; !small;) {
    SIPG_CUDA_TRY(cudaGraphLaunch(w->exec, s));
    count_launch((cg_fused_direction<T>(op) ? 2ULL : 3ULL) * K);
    launched += K;
    SIPG_CUDA_TRY(cudaMemcpyAsync(hs, w->st, sizeof(CgState<T>), cudaMemcpyDeviceToHost, s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs->done) break;
    if (launched > (long long)max_i + K) {  // cannot happen unless the device state is corrupt
      set_error("sipg_cg: iteration bookkeeping lost");
      return SIPG_ERR_CUDA;
    }
  }
  SIPG_CUDA_TRY(cudaEventRecord(w->ev1, s));
  SIPG_CUDA_TRY(cudaEventSynchronize(w->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, w->ev0, w->ev1);
  const bool conv = !(std::sqrt((double)hs->rr) > (double)hs->stop);
  if (res) {
    res->iterations = hs->it;
    res->rr = (double)hs->rr;
    res->stop = (double)hs->stop;
    res->time_ms = ms;
    res->converged = conv ? 1 : 0;
  }
  if (hs->status == (int)SIPG_ERR_BREAKDOWN) {
    set_error("sipg_cg: breakdown (p.Ap <= 0 or non-finite scalar)");
    return SIPG_ERR_BREAKDOWN;
  }
  return conv ? SIPG_OK : SIPG_ERR_NOT_CONVERGED;
}


// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* sipg_last_error(void) { return t_last_error.c_str(); }
const char* sipg_version(void) { return "sipg-gb300 0.1 (sm_103a)"; }
unsigned long long sipg_launch_count(void) { return g_launches.load(); }

sipg_status sipg_lgl_table(int npts, double* nodes, double* weights) {
  if (npts < 2 || npts > 64 || !nodes || !weights) {
    set_error("sipg_lgl_table: npts must be in 2..64 and pointers non-null");
    return SIPG_ERR_INVALID;
  }
  lgl_compute(npts - 1, nodes, weights);
  return SIPG_OK;
}

sipg_status sipg_dphi_table(int degree, double* D) {
  if (degree < 1 || degree > 63 || !D) {
    set_error("sipg_dphi_table: degree must be in 1..63");
    return SIPG_ERR_INVALID;
  }
  double x[64], w[64];
  lgl_compute(degree, x, w);
  dphi_compute(degree, x, D);
  return SIPG_OK;
}

sipg_status sipg_laplacian_rows_f64(int degree, double* rows) {
  if (degree < 1 || degree > SIPG_MAX_DEGREE || !rows) {
    set_error("sipg_laplacian_rows_f64: degree must be in 1..SIPG_MAX_DEGREE and rows non-null");
    return SIPG_ERR_INVALID;
  }
  HostTables t;
  if (build_host_tables(degree, &t) != 0) {
    set_error("sipg_laplacian_rows_f64: table construction failed");
    return SIPG_ERR_INVALID;
  }
  // lap(i1,i2,j1,j2) = [i2 == j2] w_i2 K(i1,j1) + [i1 == j1] w_i1 K(i2,j2) on
  // the reference element; row (i1,i2) keeps its cross pattern: the
  // diagonal, then (i1, j != i2), then (j != i1, i2)
  const int n = degree + 1, R = 2 * degree + 1;
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2) {
      double* row = rows + (size_t)(i1 * n + i2) * R;
      int r = 0;
      row[r++] = t.w[i2] * t.K[i1 * n + i1] + t.w[i1] * t.K[i2 * n + i2];
      for (int j = 0; j < n; ++j)
        if (j != i2) row[r++] = t.w[i1] * t.K[i2 * n + j];
      for (int j = 0; j < n; ++j)
        if (j != i1) row[r++] = t.w[i2] * t.K[i1 * n + j];
    }
  return SIPG_OK;
}

sipg_status sipg_square_mesh_coords(int dim, double* x, double* y) {
  if (dim < 1 || !x || !y) {
    set_error("sipg_square_mesh_coords: dim >= 1 and non-null pointers required");
    return SIPG_ERR_INVALID;
  }
  const long long noe = (long long)dim * dim;
  const double delta = 1. / (double)dim;
  double xx = 0, yy = 1;
  for (int i = 0; i < dim; ++i) {
    xx = 0;
    yy -= delta;
    for (int j = 0; j < dim; ++j) {
      const long long id = (long long)i * dim + j;
      x[0 * noe + id] = xx;
      y[0 * noe + id] = yy;
      x[1 * noe + id] = xx + delta;
      y[1 * noe + id] = yy;
      x[2 * noe + id] = xx + delta;
      y[2 * noe + id] = yy + delta;
      x[3 * noe + id] = xx;
      y[3 * noe + id] = yy + delta;
      xx += delta;
    }
  }
  return SIPG_OK;
}

sipg_status sipg_op_create(int dim, int degree, double pen, sipg_op** out) {
  if (!out) {
    set_error("sipg_op_create: null output");
    return SIPG_ERR_INVALID;
  }
  *out = nullptr;
  if (dim < 1 || dim > 65535) {
    set_error("sipg_op_create: dim must be in 1..65535");
    return SIPG_ERR_INVALID;
  }
  if (degree < 1 || degree > SIPG_MAX_P) {
    set_error("sipg_op_create: degree must be in 1..8");
    return SIPG_ERR_UNSUPPORTED;
  }
  if (!std::isfinite(pen)) {
    set_error("sipg_op_create: penalty must be finite");
    return SIPG_ERR_INVALID;
  }
  int dev = 0, major = 0, minor = 0;
  SIPG_CUDA_TRY(cudaGetDevice(&dev));
  SIPG_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  SIPG_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  if (major * 10 + minor != 103) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "sipg_op_create: device %d is sm_%d%d; this build targets sm_103a", dev, major,
                  minor);
    set_error(buf);
    return SIPG_ERR_UNSUPPORTED;
  }
  sipg_op* op = new (std::nothrow) sipg_op;
  if (!op) return SIPG_ERR_NOMEM;
  op->dim = dim;
  op->p = degree;
  op->pen = pen;
  op->device = dev;
  op->noe = (long long)dim * dim;
  op->ndof = op->noe * (degree + 1) * (degree + 1);
  build_host_tables(degree, &op->tab);
  op->cfg64 = default_cfg(degree, dim, true);
  op->cfg32 = default_cfg(degree, dim, false);
  op->cfgdf.tx = 32;
  op->cfgdf.ty = degree <= 4 ? 8 : (degree <= 7 ? 4 : 2);  // measured at ~13-16 M DoF
  // shapes the autotuner already chose for this (degree, dim) in this process
  autotune_lookup(degree, dim, SIPG_TUNE_F64, &op->cfg64);
  autotune_lookup(degree, dim, SIPG_TUNE_F32, &op->cfg32);
  autotune_lookup(degree, dim, SIPG_TUNE_PAIRS, &op->cfgdf);
  *out = op;
  return SIPG_OK;
}

sipg_status sipg_op_destroy(sipg_op* op) {
  if (!op) return SIPG_OK;
  cudaSetDevice(op->device);
  ws_free(op->ws64);
  ws_free(op->ws32);
  if (op->mixed_free) op->mixed_free(op->mixed);
  if (op->pcg_free) op->pcg_free(op->pcg);
  if (op->tl_free) op->tl_free(op->tl);
  if (op->stage_in) cudaFree(op->stage_in);
  if (op->stage_out) cudaFree(op->stage_out);
  for (cudaStream_t h : op->hs)
    if (h) cudaStreamDestroy(h);
  for (cudaEvent_t e : op->hev)
    if (e) cudaEventDestroy(e);
  delete op;
  return SIPG_OK;
}

size_t sipg_op_solve_footprint(int dim, int degree, sipg_precision prec) {
  const size_t ndof = (size_t)dim * dim * (degree + 1) * (degree + 1);
  const size_t e = prec == SIPG_F32 ? 4 : 8;
  // x, b (caller) + r, p0, p1, Ap (workspace)
  return ndof * e * 6 + 64 * 1024;
}

sipg_status sipg_apply_f64(const sipg_op* op, const double* d_in, double* d_out, void* stream) {
  if (!op || !d_in || !d_out || d_in == d_out) {
    set_error("sipg_apply_f64: null or aliased vectors");
    return SIPG_ERR_INVALID;
  }
  ApplyArgs<double> a{};
  a.in = d_in;
  a.out = d_out;
  a.dim = op->dim;
  a.nu = op->pen;
  SIPG_CUDA_TRY(launch_apply<double>(op, APPLY_PLAIN, a, (cudaStream_t)stream));
  return SIPG_OK;
}

sipg_status sipg_apply_f32(const sipg_op* op, const float* d_in, float* d_out, void* stream) {
  if (!op || !d_in || !d_out || d_in == d_out) {
    set_error("sipg_apply_f32: null or aliased vectors");
    return SIPG_ERR_INVALID;
  }
  ApplyArgs<float> a{};
  a.in = d_in;
  a.out = d_out;
  a.dim = op->dim;
  a.nu = (float)op->pen;
  SIPG_CUDA_TRY(launch_apply<float>(op, APPLY_PLAIN, a, (cudaStream_t)stream));
  return SIPG_OK;
}

sipg_status sipg_apply_pairs(const sipg_op* op, const float* d_in, float* d_out, void* stream) {
  if (!op || !d_in || !d_out || d_in == d_out) {
    set_error("sipg_apply_pairs: null or aliased vectors");
    return SIPG_ERR_INVALID;
  }
  ApplyArgs<float> a{};
  a.in = d_in;
  a.out = d_out;
  a.dim = op->dim;
  a.nu = (float)op->pen;
  set_penalty3(a, op->pen);
  SIPG_CUDA_TRY(launch_apply_df(op->p, op->cfgdf, APPLY_PLAIN, a, nullptr, nullptr, 0, 0, op->tab, (cudaStream_t)stream));
  return SIPG_OK;
}

// Copies element rows [r0, r1) of every node plane between a host and a
// device vector (node-major layout: plane k of noe values at k * noe): one
// strided copy where the plane pitch allows it, else one copy per plane.
static cudaError_t copy_rows(double* dst, const double* src, const sipg_op* op, int r0, int r1, cudaMemcpyKind kind,
                             cudaStream_t s) {
  const size_t pitch = (size_t)op->noe * sizeof(double);
  const size_t off = (size_t)r0 * op->dim, width = (size_t)(r1 - r0) * op->dim * sizeof(double);
  const int planes = (op->p + 1) * (op->p + 1);
  if (pitch <= (size_t)INT32_MAX)
    return cudaMemcpy2DAsync(dst + off, pitch, src + off, pitch, width, planes, kind, s);
  for (int k = 0; k < planes; ++k) {
    const cudaError_t e =
        cudaMemcpyAsync(dst + (size_t)k * op->noe + off, src + (size_t)k * op->noe + off, width, kind, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// y = A x with host buffers, pipelined over bands of element rows: the
// copy-in of band b + 1, the apply of band b (two compute streams, so one
// band's tail overlaps the next band's start) and the copy-out of band b - 1
// run at once.  Band b's copy-in carries one row more -- the first row of
// band b + 1, its halo below (the row above arrived with band b - 1) -- so its
// apply waits for its own copy only.  Synchronous: returns when h_out is
// written.
sipg_status sipg_apply_host_f64(sipg_op* op, const double* h_in, double* h_out, void* stream) {
  if (!op || !h_in || !h_out) {
    set_error("sipg_apply_host_f64: null argument");
    return SIPG_ERR_INVALID;
  }
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = (size_t)op->ndof * sizeof(double);
  constexpr int kMaxBands = 16;
  // equal bands of a multiple of 8 rows (every tile's rows divide 8), ~64
  // rows each.  Measured at 1024^2, p = 4, end to end: 8 bands 15.3 GDoF/s,
  // 16 bands 16.9, 32 bands 11.7; 16-row first and last bands (a faster fill
  // and drain on paper) 11.5
  int bounds[kMaxBands + 1];
  int nb = 0;
  {
    const int n = std::max(1, std::min(kMaxBands, op->dim / 64));
    const int rows = ((op->dim + n - 1) / n + 7) / 8 * 8;
    for (int r = 0; r < op->dim; r += rows) bounds[nb++] = r;
    bounds[nb] = op->dim;
  }
  std::lock_guard<std::mutex> lk(op->mu);  // the staging buffers and streams are per op
  if (!op->stage_in) SIPG_CUDA_TRY(cudaMalloc(&op->stage_in, bytes));
  if (!op->stage_out) SIPG_CUDA_TRY(cudaMalloc(&op->stage_out, bytes));
  if (!op->hs[0]) {
    for (cudaStream_t& h : op->hs) SIPG_CUDA_TRY(cudaStreamCreateWithFlags(&h, cudaStreamNonBlocking));
    for (cudaEvent_t& e : op->hev) SIPG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  cudaStream_t s_in = op->hs[0], s_out = op->hs[1];
  cudaEvent_t* ev_in = op->hev;                // [kMaxBands]: band b's rows (and its halo row) are on the device
  cudaEvent_t* ev_done = op->hev + kMaxBands;  // [kMaxBands]: band b's outputs are written
  cudaEvent_t ev_start = op->hev[2 * kMaxBands], ev_end = op->hev[2 * kMaxBands + 1];
  // everything starts after the work already queued on the caller's stream
  SIPG_CUDA_TRY(cudaEventRecord(ev_start, s));
  for (int k = 0; k < 4; ++k) SIPG_CUDA_TRY(cudaStreamWaitEvent(op->hs[k], ev_start, 0));
  for (int b = 0; b < nb; ++b) {
    const int r0 = bounds[b], r1 = std::min(op->dim, bounds[b + 1] + 1);  // + the halo row below
    SIPG_CUDA_TRY(copy_rows(op->stage_in, h_in, op, r0, r1, cudaMemcpyHostToDevice, s_in));
    SIPG_CUDA_TRY(cudaEventRecord(ev_in[b], s_in));
  }
  for (int b = 0; b < nb; ++b) {
    const int r0 = bounds[b], r1 = bounds[b + 1];
    cudaStream_t cs = op->hs[2 + (b & 1)];
    SIPG_CUDA_TRY(cudaStreamWaitEvent(cs, ev_in[b], 0));
    ApplyArgs<double> a{};
    a.in = op->stage_in;
    a.out = op->stage_out;
    a.dim = op->dim;
    a.nu = op->pen;
    a.row0 = r0;
    a.nrows = r1 - r0;
    SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_PLAIN, a, op->tab, cs));
    SIPG_CUDA_TRY(cudaEventRecord(ev_done[b], cs));
    SIPG_CUDA_TRY(cudaStreamWaitEvent(s_out, ev_done[b], 0));
    SIPG_CUDA_TRY(copy_rows(h_out, op->stage_out, op, r0, r1, cudaMemcpyDeviceToHost, s_out));
  }
  SIPG_CUDA_TRY(cudaEventRecord(ev_end, s_out));
  SIPG_CUDA_TRY(cudaStreamWaitEvent(s, ev_end, 0));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  return SIPG_OK;
}

sipg_status sipg_cg_f64(sipg_op* op, double* d_x, const double* d_b, double tol, int tol_relative, int max_it,
                        sipg_cg_result* res, void* stream) {
  return cg_solve<double>(op, d_x, d_b, tol, tol_relative, max_it, res, (cudaStream_t)stream);
}

sipg_status sipg_cg_f32(sipg_op* op, float* d_x, const float* d_b, float tol, int tol_relative, int max_it,
                        sipg_cg_result* res, void* stream) {
  return cg_solve<float>(op, d_x, d_b, tol, tol_relative, max_it, res, (cudaStream_t)stream);
}

sipg_status sipg_rhs_f64(const sipg_op* op, int sol, const sipg_modes* modes, double* d_b, void* stream) {
  if (!op || !d_b || sol < SIPG_SOL_A || sol > SIPG_SOL_MODES || (sol == SIPG_SOL_MODES && !modes) ||
      (modes && (modes->nmodes < 0 || modes->nmodes > 8))) {
    set_error("sipg_rhs_f64: invalid arguments");
    return SIPG_ERR_INVALID;
  }
  return rhs_f64(op, sol, modes, d_b, (cudaStream_t)stream);
}

sipg_status sipg_err_norms_f64(const sipg_op* op, int sol, const sipg_modes* modes, const double* d_u, double* err,
                               void* stream) {
  if (!op || !d_u || !err || sol < SIPG_SOL_A || sol > SIPG_SOL_MODES || (sol == SIPG_SOL_MODES && !modes)) {
    set_error("sipg_err_norms_f64: invalid arguments");
    return SIPG_ERR_INVALID;
  }
  return err_norms_f64(op, sol, modes, d_u, err, (cudaStream_t)stream);
}

sipg_status sipg_solve_mixed(sipg_op* op, double* d_x, const double* d_b, const sipg_mixed_opts* opts,
                             sipg_mixed_result* res, void* stream);

}  // extern "C"
