// batch.cu -- many SIPG problems solved together (no counterpart in the
// reference): many right-hand sides on one mesh, or uneven (dim, p) problems.
//
// Every instance keeps its own operator (shared between instances with the
// same dim, p and penalty), inner CG vectors (double-float pairs: the inner
// kind SIPG_INNER_PAIRS of mixed.cu, which converges at every condition
// number), FP64 residual, device CG states and reduction scratch, resident on
// the device for the life of the batch.  One inner iteration of the whole
// batch is one batched compensated apply launch per degree present
// (k_sipg_apply_df_batched: the instances' tiles concatenated into one grid)
// plus a batched direction launch before it and a batched update launch after
// it (k_cg_direction_pairs_batched, k_cg_update_pairs_batched); K iterations are
// captured once as a CUDA graph and replayed.  The mixed-precision scheme is
// the reliable-update one of mixed.cu, per instance: an instance whose inner
// residual has fallen by inner_tol stops iterating (its blocks return at once)
// until the host, between graph replays, folds its correction into x in FP64,
// recomputes its FP64 residual (batched FP64 applies over the instances that
// need it) and restarts it -- or retires it once ||b - Ax|| <= outer_tol
// ||b||.  Converged instances retire mid-batch while the others go on.
#include <algorithm>
#include <cmath>
#include <map>
#include <new>
#include <tuple>
#include <vector>

#include "sipg_cg_df.cuh"

using namespace sipg;

namespace sipg {

struct MixedInst {
  double* x64;
  const double* b64;
  double* r64;
  float* r32;  // pair vectors
  float* e;
  CgState<double>* st32;  // the inner state (FP64 scalars)
  CgState<double>* st64;
  ReduceScratch red32;
  ReduceScratch red64;
  size_t n;
  int first;
  double delta;
  double stop;  // the outer target in inner residual units
  int max_it;
  int nblk;  // blocks this instance uses (see VecInst)
};

// ||b||^2 of every listed instance into its FP64 state
__global__ void __launch_bounds__(kVecThreads) k_batch_norm_b(const MixedInst* __restrict__ insts) {
  const MixedInst m = insts[blockIdx.y];
  if ((int)blockIdx.x >= m.nblk) return;
  cg_init_body<double>(m.b64, m.n, m.st64, 0.0, 0, 1, m.red64, blockIdx.x, m.nblk);
}

// inner residual = r64 as pairs, e = 0, inner CG state for the next run (see
// inner_restart_body)
__global__ void __launch_bounds__(kVecThreads) k_batch_restart(const MixedInst* __restrict__ insts) {
  const MixedInst m = insts[blockIdx.y];
  if ((int)blockIdx.x >= m.nblk) return;
  inner_restart_body<INNER_PAIRS>(m.r64, m.r32, m.e, m.n, m.st32, m.red32, m.first, m.delta, m.stop, m.max_it,
                                  blockIdx.x, m.nblk);
}

// x64 += e
__global__ void __launch_bounds__(kVecThreads) k_batch_fold(const MixedInst* __restrict__ insts) {
  const MixedInst m = insts[blockIdx.y];
  if ((int)blockIdx.x >= m.nblk) return;
  inner_fold_body<INNER_PAIRS>(m.x64, m.e, m.n, blockIdx.x, m.nblk);
}

// park instances: the FP32 iterations skip them
__global__ void k_batch_park(const MixedInst* __restrict__ insts, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    insts[i].st32->done = 1;
    insts[i].st32->need_update = 0;
  }
}

}  // namespace sipg

namespace {

struct BInst {
  int dim = 0, p = 0;
  double pen = 0;
  sipg_op* op = nullptr;
  size_t n = 0;
  double* r64 = nullptr;
  float* r32 = nullptr;  // pair vectors (2 n floats) from here
  float* e = nullptr;
  float* p0 = nullptr;
  float* Ap = nullptr;
  CgState<double>* st32 = nullptr;  // inner state
  CgState<double>* st64 = nullptr;
  ReduceScratch red32, red64;
  int tilesdf = 0, tiles64 = 0;
};

struct BGroup {
  int p = 0;
  std::vector<int> members;
  TileCfg cfgdf, cfg64;
  ApplyArgs<float>* d_cg = nullptr;  // all members, compensated FP32 CG mode
  int* d_tilesdf = nullptr;
  int totaldf = 0;
  ApplyArgs<double>* d_res = nullptr;  // a subset, FP64 residual mode (rebuilt per round)
  int* d_tiles64 = nullptr;
};

int tiles_of(int dim, const TileCfg& c) { return apply_grid_blocks(dim, c); }

}  // namespace

struct sipg_batch {
  int n = 0;
  std::vector<BInst> inst;
  std::vector<BGroup> groups;
  std::vector<sipg_op*> owned;
  PairInst* d_vec = nullptr;
  MixedInst* d_sel = nullptr;  // selection list (capacity n)
  MixedInst* h_sel = nullptr;  // pinned
  ApplyArgs<double>* h_res = nullptr;  // pinned staging for FP64 residual args
  int* h_tiles = nullptr;              // pinned staging for tile starts
  CgState<double>* h_st32 = nullptr;   // pinned mirrors, n each
  CgState<double>* h_st64 = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
  int K = 8;
  int bpi = 1;  // blocks per instance for the vector kernels
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

static void batch_free(sipg_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (BInst& i : b->inst) {
    cudaFree(i.r64);
    cudaFree(i.r32);
    cudaFree(i.e);
    cudaFree(i.p0);
    cudaFree(i.Ap);
    cudaFree(i.st32);
    cudaFree(i.st64);
    cudaFree(i.red32.partials);
    cudaFree(i.red32.counter);
    cudaFree(i.red64.partials);
    cudaFree(i.red64.counter);
  }
  for (BGroup& g : b->groups) {
    cudaFree(g.d_cg);
    cudaFree(g.d_tilesdf);
    cudaFree(g.d_res);
    cudaFree(g.d_tiles64);
  }
  cudaFree(b->d_vec);
  cudaFree(b->d_sel);
  cudaFreeHost(b->h_sel);
  cudaFreeHost(b->h_res);
  cudaFreeHost(b->h_tiles);
  cudaFreeHost(b->h_st32);
  cudaFreeHost(b->h_st64);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  for (sipg_op* op : b->owned) sipg_op_destroy(op);
  delete b;
}

static sipg_status batch_alloc(sipg_batch* b) {
  const int n = b->n;
  b->bpi = 1;
  for (const BInst& i : b->inst) b->bpi = std::max(b->bpi, inst_blocks(i.n));
  for (BInst& i : b->inst) {
    const int cap = reduce_capacity(i.dim);
    const size_t pair_bytes = 2 * i.n * sizeof(float);
    SIPG_CUDA_TRY(cudaMalloc(&i.r64, i.n * sizeof(double)));
    SIPG_CUDA_TRY(cudaMalloc(&i.r32, pair_bytes));
    SIPG_CUDA_TRY(cudaMalloc(&i.e, pair_bytes));
    SIPG_CUDA_TRY(cudaMalloc(&i.p0, pair_bytes));
    SIPG_CUDA_TRY(cudaMalloc(&i.Ap, pair_bytes));
    SIPG_CUDA_TRY(cudaMalloc(&i.st32, sizeof(CgState<double>)));
    SIPG_CUDA_TRY(cudaMalloc(&i.st64, sizeof(CgState<double>)));
    SIPG_CUDA_TRY(cudaMemset(i.st32, 0, sizeof(CgState<double>)));
    SIPG_CUDA_TRY(cudaMemset(i.st64, 0, sizeof(CgState<double>)));
    ReduceScratch* reds[2] = {&i.red32, &i.red64};
    for (ReduceScratch* r : reds) {
      SIPG_CUDA_TRY(cudaMalloc(&r->partials, sizeof(double) * cap));
      SIPG_CUDA_TRY(cudaMalloc(&r->counter, sizeof(unsigned int)));
      SIPG_CUDA_TRY(cudaMemset(r->counter, 0, sizeof(unsigned int)));
      r->capacity = cap;
    }
  }
  // groups by degree
  std::map<int, int> gidx;
  for (int k = 0; k < n; ++k) {
    const int p = b->inst[k].p;
    if (!gidx.count(p)) {
      gidx[p] = (int)b->groups.size();
      BGroup g;
      g.p = p;
      g.cfgdf = b->inst[k].op->cfgdf;
      g.cfg64 = batched_tile(b->inst[k].op->cfg64);
      b->groups.push_back(g);
    }
    b->groups[gidx[p]].members.push_back(k);
  }
  for (BGroup& g : b->groups) {
    const int m = (int)g.members.size();
    std::vector<ApplyArgs<float>> args(m);
    std::vector<int> ts(m + 1, 0);
    for (int j = 0; j < m; ++j) {
      BInst& i = b->inst[g.members[j]];
      i.tilesdf = tiles_of(i.dim, g.cfgdf);
      i.tiles64 = tiles_of(i.dim, g.cfg64);
      ApplyArgs<float> a{};
      a.in = i.p0;  // the direction, formed by k_cg_direction_pairs_batched
      a.out = i.Ap;
      a.dim = i.dim;
      a.nu = (float)i.pen;
      set_penalty3(a, i.pen);
      a.stp = i.st32;
      a.red = i.red32;
      args[j] = a;
      ts[j + 1] = ts[j] + i.tilesdf;
    }
    g.totaldf = ts[m];
    SIPG_CUDA_TRY(cudaMalloc(&g.d_cg, sizeof(ApplyArgs<float>) * m));
    SIPG_CUDA_TRY(cudaMalloc(&g.d_tilesdf, sizeof(int) * (m + 1)));
    SIPG_CUDA_TRY(cudaMalloc(&g.d_res, sizeof(ApplyArgs<double>) * m));
    SIPG_CUDA_TRY(cudaMalloc(&g.d_tiles64, sizeof(int) * (m + 1)));
    SIPG_CUDA_TRY(cudaMemcpy(g.d_cg, args.data(), sizeof(ApplyArgs<float>) * m, cudaMemcpyHostToDevice));
    SIPG_CUDA_TRY(cudaMemcpy(g.d_tilesdf, ts.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice));
  }
  std::vector<PairInst> vec(n);
  for (int k = 0; k < n; ++k) {
    BInst& i = b->inst[k];
    PairInst v;
    v.x = i.e;
    v.pb0 = i.p0;
    v.pb1 = i.p0;
    v.r = i.r32;
    v.Ap = i.Ap;
    v.n = i.n;
    v.st = i.st32;
    v.red = i.red32;
    v.nblk = inst_blocks(i.n);
    v.pad = 0;
    vec[k] = v;
  }
  SIPG_CUDA_TRY(cudaMalloc(&b->d_vec, sizeof(PairInst) * n));
  SIPG_CUDA_TRY(cudaMemcpy(b->d_vec, vec.data(), sizeof(PairInst) * n, cudaMemcpyHostToDevice));
  SIPG_CUDA_TRY(cudaMalloc(&b->d_sel, sizeof(MixedInst) * n));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_sel, sizeof(MixedInst) * n));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_res, sizeof(ApplyArgs<double>) * n));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_tiles, sizeof(int) * (n + 1)));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_st32, sizeof(CgState<double>) * n));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_st64, sizeof(CgState<double>) * n));
  SIPG_CUDA_TRY(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
  SIPG_CUDA_TRY(cudaEventCreate(&b->ev0));
  SIPG_CUDA_TRY(cudaEventCreate(&b->ev1));
  long long total = 0;
  for (const BInst& i : b->inst) total += (long long)i.n;
  b->K = total <= (1LL << 22) ? 16 : 8;
  return SIPG_OK;
}

// K FP32 CG iterations of every instance: per degree a batched apply, then one
// batched update; captured once.
static sipg_status batch_capture(sipg_batch* b) {
  if (b->exec) return SIPG_OK;
  for (BGroup& g : b->groups)
    SIPG_CUDA_TRY(launch_apply_df(g.p, g.cfgdf, APPLY_PREPARE, ApplyArgs<float>{}, nullptr, nullptr, 0, 0,
                                  b->inst[g.members[0]].op->tab, b->cap));
  cudaGraph_t graph = nullptr;
  SIPG_CUDA_TRY(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaSuccess;
  for (int k = 0; k < b->K && err == cudaSuccess; ++k) {
    k_cg_direction_pairs_batched<<<dim3(b->bpi, b->n), kVecThreads, 0, b->cap>>>(b->d_vec);
    err = cudaGetLastError();
    for (BGroup& g : b->groups) {
      if (err != cudaSuccess) break;
      err = launch_apply_df(g.p, g.cfgdf, APPLY_DOT, ApplyArgs<float>{}, g.d_cg, g.d_tilesdf, (int)g.members.size(),
                            g.totaldf, b->inst[g.members[0]].op->tab, b->cap);
      if (err != cudaSuccess) break;
    }
    if (err != cudaSuccess) break;
    k_cg_update_pairs_batched<<<dim3(b->bpi, b->n), kVecThreads, 0, b->cap>>>(b->d_vec);
    err = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamEndCapture(b->cap, &graph);
  if (err != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    set_error(std::string("batch graph capture failed: ") + cudaGetErrorString(err != cudaSuccess ? err : e2));
    return SIPG_ERR_CUDA;
  }
  cudaError_t e3 = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e3 != cudaSuccess) {
    b->exec = nullptr;
    set_error(std::string("batch graph instantiate failed: ") + cudaGetErrorString(e3));
    return SIPG_ERR_CUDA;
  }
  return SIPG_OK;
}

// FP64 residual r = b - A x of the selected instances (batched per degree)
static sipg_status batch_residuals(sipg_batch* b, const std::vector<int>& sel, double* const* d_x,
                                   const double* const* d_b, cudaStream_t s) {
  for (BGroup& g : b->groups) {
    int m = 0;
    b->h_tiles[0] = 0;
    for (int k : sel) {
      BInst& i = b->inst[k];
      if (i.p != g.p) continue;
      ApplyArgs<double> a{};
      a.in = d_x[k];
      a.out = i.r64;
      a.b = d_b[k];
      a.dim = i.dim;
      a.nu = i.pen;
      a.st = i.st64;
      a.red = i.red64;
      b->h_res[m] = a;
      b->h_tiles[m + 1] = b->h_tiles[m] + i.tiles64;
      ++m;
    }
    if (!m) continue;
    SIPG_CUDA_TRY(cudaMemcpyAsync(g.d_res, b->h_res, sizeof(ApplyArgs<double>) * m, cudaMemcpyHostToDevice, s));
    SIPG_CUDA_TRY(cudaMemcpyAsync(g.d_tiles64, b->h_tiles, sizeof(int) * (m + 1), cudaMemcpyHostToDevice, s));
    SIPG_CUDA_TRY(launch_apply_batched_f64(g.p, g.cfg64, APPLY_RESID, g.d_res, g.d_tiles64, m, b->h_tiles[m],
                                           b->inst[g.members[0]].op->tab, s));
    // the pinned staging is reused by the next group: wait for the copies
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return SIPG_OK;
}

static int fill_sel(sipg_batch* b, const std::vector<int>& sel, double* const* d_x, const double* const* d_b,
                    int first, double delta, const std::vector<double>& stop, int max_it) {
  int m = 0;
  for (int k : sel) {
    BInst& i = b->inst[k];
    MixedInst mi;
    mi.x64 = d_x[k];
    mi.b64 = d_b[k];
    mi.r64 = i.r64;
    mi.e = i.e;
    mi.r32 = i.r32;
    mi.st32 = i.st32;
    mi.st64 = i.st64;
    mi.red32 = i.red32;
    mi.red64 = i.red64;
    mi.n = i.n;
    mi.first = first;
    mi.delta = delta;
    mi.stop = stop[k];
    mi.max_it = max_it;
    mi.nblk = inst_blocks(i.n);
    b->h_sel[m++] = mi;
  }
  return m;
}

extern "C" {

sipg_status sipg_batch_create(int n, const sipg_problem* probs, sipg_batch** out) {
  if (!out || n < 1 || !probs) {
    set_error("sipg_batch_create: need n >= 1 problems and an output pointer");
    return SIPG_ERR_INVALID;
  }
  *out = nullptr;
  sipg_batch* b = new (std::nothrow) sipg_batch;
  if (!b) return SIPG_ERR_NOMEM;
  b->n = n;
  b->inst.resize(n);
  std::map<std::tuple<int, int, double>, sipg_op*> ops;
  for (int k = 0; k < n; ++k) {
    const sipg_problem& pr = probs[k];
    const auto key = std::make_tuple(pr.dim, pr.degree, pr.pen);
    sipg_op* op = nullptr;
    if (ops.count(key)) {
      op = ops[key];
    } else {
      sipg_status s = sipg_op_create(pr.dim, pr.degree, pr.pen, &op);
      if (s != SIPG_OK) {
        batch_free(b);
        return s;
      }
      ops[key] = op;
      b->owned.push_back(op);
    }
    BInst& i = b->inst[k];
    i.dim = pr.dim;
    i.p = pr.degree;
    i.pen = pr.pen;
    i.op = op;
    i.n = (size_t)op->ndof;
  }
  sipg_status s = batch_alloc(b);
  if (s != SIPG_OK) {
    batch_free(b);
    return s;
  }
  *out = b;
  return SIPG_OK;
}

sipg_status sipg_batch_destroy(sipg_batch* b) {
  batch_free(b);
  return SIPG_OK;
}

sipg_status sipg_batch_op(const sipg_batch* b, int i, sipg_op** op) {
  if (!b || !op || i < 0 || i >= b->n) {
    set_error("sipg_batch_op: index out of range");
    return SIPG_ERR_INVALID;
  }
  *op = b->inst[i].op;
  return SIPG_OK;
}

size_t sipg_batch_footprint(const sipg_batch* b) {
  if (!b) return 0;
  size_t bytes = 0;
  for (const BInst& i : b->inst) bytes += i.n * (8 + 4 * 8) + 2 * sizeof(double) * reduce_capacity(i.dim);
  return bytes;
}

sipg_status sipg_batch_solve_mixed(sipg_batch* b, double* const* d_x, const double* const* d_b,
                                   const sipg_mixed_opts* opts, sipg_mixed_result* res, void* stream) {
  if (!b || !d_x || !d_b) {
    set_error("sipg_batch_solve_mixed: null argument");
    return SIPG_ERR_INVALID;
  }
  for (int k = 0; k < b->n; ++k)
    if (!d_x[k] || !d_b[k]) {
      set_error("sipg_batch_solve_mixed: null vector");
      return SIPG_ERR_INVALID;
    }
  sipg_mixed_opts o = {0.1, 1e-10, 200, 0};
  if (opts) o = *opts;
  if (!(o.inner_tol > 0) || !(o.inner_tol < 1) || !(o.outer_tol > 0) || o.max_outer < 1) {
    set_error("sipg_batch_solve_mixed: need 0 < inner_tol < 1, outer_tol > 0, max_outer >= 1");
    return SIPG_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int n = b->n;
  sipg_status st = batch_capture(b);
  if (st != SIPG_OK) return st;
  SIPG_CUDA_TRY(cudaEventRecord(b->ev0, s));
  std::vector<int> all(n);
  for (int k = 0; k < n; ++k) all[k] = k;
  std::vector<int> corrections(n, 0), retired(n, 0), conv(n, 0);
  std::vector<double> bnorm(n, 0.0), rel(n, INFINITY);
  std::vector<long long> max_inner(n);
  for (int k = 0; k < n; ++k) max_inner[k] = o.max_inner > 0 ? o.max_inner : (long long)b->inst[k].n;

  // ||b|| of every instance, and park every FP32 state
  std::vector<double> stop(n, 0.0);
  int m = fill_sel(b, all, d_x, d_b, 1, o.inner_tol, stop, 0);
  SIPG_CUDA_TRY(cudaMemcpyAsync(b->d_sel, b->h_sel, sizeof(MixedInst) * m, cudaMemcpyHostToDevice, s));
  k_batch_norm_b<<<dim3(b->bpi, m), kVecThreads, 0, s>>>(b->d_sel);
  k_batch_park<<<(m + 127) / 128, 128, 0, s>>>(b->d_sel, m);
  count_launch(2);
  SIPG_CUDA_TRY(cudaGetLastError());
  for (int k = 0; k < n; ++k)
    SIPG_CUDA_TRY(cudaMemcpyAsync(b->h_st64 + k, b->inst[k].st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  for (int k = 0; k < n; ++k) {
    bnorm[k] = std::sqrt(b->h_st64[k].bb);
    stop[k] = 0.5 * o.outer_tol * (bnorm[k] > 0 ? bnorm[k] : 1.0);
  }

  std::vector<int> sel = all;
  bool first_round = true;
  sipg_status status = SIPG_OK;
  for (;;) {
    if (!sel.empty()) {
      // FP64 residuals of the selected instances; retire or restart them
      st = batch_residuals(b, sel, d_x, d_b, s);
      if (st != SIPG_OK) return st;
      for (int k : sel)
        SIPG_CUDA_TRY(cudaMemcpyAsync(b->h_st64 + k, b->inst[k].st64, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
      SIPG_CUDA_TRY(cudaStreamSynchronize(s));
      std::vector<int> restart_first, restart_cont;
      for (int k : sel) {
        const double rr = b->h_st64[k].rr;
        rel[k] = bnorm[k] > 0 ? std::sqrt(rr) / bnorm[k] : std::sqrt(rr);
        const long long its = first_round ? 0 : b->h_st32[k].it;
        if (!std::isfinite(rel[k])) {
          retired[k] = 1;
          status = SIPG_ERR_BREAKDOWN;
        } else if (rel[k] <= o.outer_tol || rr == 0.0) {
          retired[k] = 1;
          conv[k] = 1;
        } else if (corrections[k] >= o.max_outer || its >= max_inner[k]) {
          retired[k] = 1;
          if (status == SIPG_OK) status = SIPG_ERR_NOT_CONVERGED;
        } else if (first_round) {
          restart_first.push_back(k);
        } else {
          restart_cont.push_back(k);
        }
      }
      for (int pass = 0; pass < 2; ++pass) {
        const std::vector<int>& list = pass ? restart_cont : restart_first;
        if (list.empty()) continue;
        m = fill_sel(b, list, d_x, d_b, pass ? 0 : 1, o.inner_tol, stop, 1000);
        SIPG_CUDA_TRY(cudaMemcpyAsync(b->d_sel, b->h_sel, sizeof(MixedInst) * m, cudaMemcpyHostToDevice, s));
        k_batch_restart<<<dim3(b->bpi, m), kVecThreads, 0, s>>>(b->d_sel);
        count_launch();
        SIPG_CUDA_TRY(cudaGetLastError());
        SIPG_CUDA_TRY(cudaStreamSynchronize(s));  // h_sel is reused
      }
      first_round = false;
    }
    bool active = false;
    for (int k = 0; k < n; ++k) active = active || !retired[k];
    if (!active) break;
    // FP32 iterations of every active instance
    SIPG_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    unsigned long long per_iter = (unsigned long long)b->groups.size() + 2;
    count_launch(per_iter * b->K);
    for (int k = 0; k < n; ++k)
      SIPG_CUDA_TRY(cudaMemcpyAsync(b->h_st32 + k, b->inst[k].st32, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
    sel.clear();
    for (int k = 0; k < n; ++k) {
      if (retired[k] || !b->h_st32[k].done) continue;
      if (b->h_st32[k].status == (int)SIPG_ERR_BREAKDOWN) {
        retired[k] = 1;
        status = SIPG_ERR_BREAKDOWN;
        continue;
      }
      sel.push_back(k);
    }
    if (!sel.empty()) {
      m = fill_sel(b, sel, d_x, d_b, 0, o.inner_tol, stop, 0);
      SIPG_CUDA_TRY(cudaMemcpyAsync(b->d_sel, b->h_sel, sizeof(MixedInst) * m, cudaMemcpyHostToDevice, s));
      k_batch_fold<<<dim3(b->bpi, m), kVecThreads, 0, s>>>(b->d_sel);
      count_launch();
      SIPG_CUDA_TRY(cudaGetLastError());
      SIPG_CUDA_TRY(cudaStreamSynchronize(s));  // h_sel is reused
      for (int k : sel) corrections[k] += 1;
    }
  }
  SIPG_CUDA_TRY(cudaEventRecord(b->ev1, s));
  SIPG_CUDA_TRY(cudaEventSynchronize(b->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  if (res)
    for (int k = 0; k < n; ++k) {
      res[k].outer_iterations = corrections[k];
      res[k].inner_iterations = b->h_st32[k].it;
      res[k].rel_residual = rel[k];
      res[k].time_ms = ms;
      res[k].converged = conv[k];
    }
  return status;
}

}  // extern "C"
