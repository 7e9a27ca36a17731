// batch.cu -- many SIPG problems solved together (no counterpart in the
// reference): many right-hand sides on one mesh, or uneven (dim, p) problems.
//
// Every instance keeps its own operator (shared between instances with the
// same dim, p and penalty), FP64 residual, direction and A d, FP32 inner CG
// vectors, device states and reduction scratch, resident on the device for
// the life of the batch.  The scheme is the flexible one of mixed.cu, per
// instance (sipg_fcg.cuh): flexible CG in FP64 around an FP32 inner CG (FP32
// values and accumulation) preconditioned by the two-level preconditioner
// (twolevel.cu; tables shared by the instances of one operator, scratch per
// instance), restarting from zero on the scaled residual.
//
// One inner iteration of the whole batch is the batched preconditioner
// (element kernels one launch per degree present, vertex-grid kernels one
// launch per level for all instances), a batched direction launch, one
// batched FP32 apply launch per degree (k_sipg_apply_batched in APPLY_DOT
// mode: the instances' tiles concatenated into one grid) and a batched update
// launch; K iterations are captured once as a CUDA graph and replayed.  An instance whose inner solve has finished
// skips the replays (its blocks return at once) until the host, between
// replays, runs its FP64 outer step together with every other instance due
// one (batched gamma / direction / FP64 apply / update launches over that
// selection) and restarts its inner solve -- or, once its FP64 residual
// b - A x (recomputed in FP64 before it may stop) is under outer_tol ||b||,
// retires it.  Converged instances retire mid-batch while the others go on.
#include <algorithm>
#include <cmath>
#include <map>
#include <new>
#include <tuple>
#include <vector>

#include "sipg_fcg.cuh"
#include "sipg_twolevel.cuh"

using namespace sipg;

namespace sipg {

// ||b||^2 and the stop threshold outer_tol ||b|| of every listed instance
__global__ void __launch_bounds__(kVecThreads) k_batch_init(const FcgInst* __restrict__ insts, double tol) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  cg_init_body<double>(v.b, v.n, v.st64, tol, 1, 1 << 30, v.red64, blockIdx.x, v.nblk);
}

// park instances: the FP32 iterations skip them
__global__ void k_batch_park(const FcgInst* __restrict__ insts, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) insts[i].st32->done = 1;
}

}  // namespace sipg

namespace {

// inner iterations one preconditioner solve may take
constexpr int kInnerCap = 4000;

struct BInst {
  int dim = 0, p = 0;
  double pen = 0;
  sipg_op* op = nullptr;
  size_t n = 0;
  double* r64 = nullptr;  // FP64: residual, direction, A d
  double* d64 = nullptr;
  double* q64 = nullptr;
  float* r32 = nullptr;   // FP32 inner: residual, solution, direction, A p
  float* e32 = nullptr;
  float* p32 = nullptr;
  float* Ap32 = nullptr;
  float* z32 = nullptr;   // preconditioned residual
  float* tls = nullptr;   // the preconditioner's scratch
  void* tl = nullptr;     // the operator's two-level preconditioner (owned by the op)
  CgState<float>* st32 = nullptr;   // (in the batch's contiguous state arrays)
  CgState<double>* st64 = nullptr;
  FcgState* fs = nullptr;
  ReduceScratch red32, red64;
  int tiles32 = 0, tiles64 = 0;
};

struct BGroup {
  int p = 0;
  std::vector<int> members;
  TileCfg cfg32, cfg64;
  ApplyArgs<float>* d_cg = nullptr;  // all members, FP32 inner CG (APPLY_DOT)
  int* d_tiles32 = nullptr;
  int total32 = 0;
  ApplyArgs<double>* d_sub = nullptr;  // a selection, FP64 residual or step (rebuilt per use)
  int* d_tiles64 = nullptr;
};

int tiles_of(int dim, const TileCfg& c) { return apply_grid_blocks(dim, c); }

}  // namespace

struct sipg_batch {
  int n = 0;
  std::vector<BInst> inst;
  std::vector<BGroup> groups;
  std::vector<sipg_op*> owned;
  CgState<float>* st32 = nullptr;   // n inner states
  CgState<double>* st64 = nullptr;  // n outer states
  FcgState* fs = nullptr;           // n flexible-step scalars
  FcgInst* d_vec = nullptr;         // every instance (the inner graph)
  TlInst* d_tl = nullptr;           // every instance's preconditioner operands, grouped by degree
  TlPlan tlplan;
  FcgInst* d_sel = nullptr;         // a selection (capacity n)
  FcgInst* h_sel = nullptr;         // pinned
  ApplyArgs<double>* h_sub = nullptr;  // pinned staging for FP64 apply args
  int* h_tiles = nullptr;              // pinned staging for tile starts
  CgState<float>* h_st32 = nullptr;    // pinned mirrors, n each
  CgState<double>* h_st64 = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
  int K = 8;
  unsigned long long graph_launches = 0;  // kernel launches one replay makes
  int bpi = 1;  // blocks per instance for the vector kernels
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

static void batch_free(sipg_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (BInst& i : b->inst) {
    cudaFree(i.r64);
    cudaFree(i.d64);
    cudaFree(i.q64);
    cudaFree(i.r32);
    cudaFree(i.e32);
    cudaFree(i.p32);
    cudaFree(i.Ap32);
    cudaFree(i.z32);
    cudaFree(i.tls);
    cudaFree(i.red32.partials);
    cudaFree(i.red32.counter);
    cudaFree(i.red64.partials);
    cudaFree(i.red64.counter);
  }
  for (BGroup& g : b->groups) {
    cudaFree(g.d_cg);
    cudaFree(g.d_tiles32);
    cudaFree(g.d_sub);
    cudaFree(g.d_tiles64);
  }
  cudaFree(b->st32);
  cudaFree(b->st64);
  cudaFree(b->fs);
  cudaFree(b->d_vec);
  cudaFree(b->d_tl);
  cudaFree(b->d_sel);
  cudaFreeHost(b->h_sel);
  cudaFreeHost(b->h_sub);
  cudaFreeHost(b->h_tiles);
  cudaFreeHost(b->h_st32);
  cudaFreeHost(b->h_st64);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  for (sipg_op* op : b->owned) sipg_op_destroy(op);
  delete b;
}

// One instance's operands (x, rhs: the caller's vectors of this solve).
static FcgInst inst_of(const sipg_batch* b, int k, double* x, const double* rhs, int first, float stop) {
  const BInst& i = b->inst[k];
  FcgInst v;
  v.x = x;
  v.b = rhs;
  v.r64 = i.r64;
  v.d64 = i.d64;
  v.q64 = i.q64;
  v.r32 = i.r32;
  v.e32 = i.e32;
  v.p32 = i.p32;
  v.Ap32 = i.Ap32;
  v.z32 = i.z32;
  v.st32 = i.st32;
  v.st64 = i.st64;
  v.fs = i.fs;
  v.red32 = i.red32;
  v.red64 = i.red64;
  v.n = i.n;
  v.nblk = inst_blocks(i.n);
  v.first = first;
  v.stop = stop;
  v.max_it = kInnerCap;
  return v;
}

static sipg_status batch_alloc(sipg_batch* b) {
  const int n = b->n;
  b->bpi = 1;
  for (const BInst& i : b->inst) b->bpi = std::max(b->bpi, inst_blocks(i.n));
  SIPG_CUDA_TRY(cudaMalloc(&b->st32, sizeof(CgState<float>) * n));
  SIPG_CUDA_TRY(cudaMalloc(&b->st64, sizeof(CgState<double>) * n));
  SIPG_CUDA_TRY(cudaMalloc(&b->fs, sizeof(FcgState) * n));
  SIPG_CUDA_TRY(cudaMemset(b->st32, 0, sizeof(CgState<float>) * n));
  SIPG_CUDA_TRY(cudaMemset(b->st64, 0, sizeof(CgState<double>) * n));
  SIPG_CUDA_TRY(cudaMemset(b->fs, 0, sizeof(FcgState) * n));
  for (int k = 0; k < n; ++k) {
    BInst& i = b->inst[k];
    const int cap = reduce_capacity(i.dim);
    SIPG_CUDA_TRY(cudaMalloc(&i.r64, i.n * sizeof(double)));
    SIPG_CUDA_TRY(cudaMalloc(&i.d64, i.n * sizeof(double)));
    SIPG_CUDA_TRY(cudaMalloc(&i.q64, i.n * sizeof(double)));
    SIPG_CUDA_TRY(cudaMalloc(&i.r32, i.n * sizeof(float)));
    SIPG_CUDA_TRY(cudaMalloc(&i.e32, i.n * sizeof(float)));
    SIPG_CUDA_TRY(cudaMalloc(&i.p32, i.n * sizeof(float)));
    SIPG_CUDA_TRY(cudaMalloc(&i.Ap32, i.n * sizeof(float)));
    SIPG_CUDA_TRY(cudaMalloc(&i.z32, i.n * sizeof(float)));
    sipg_status tst = twolevel_get(i.op, &i.tl);
    if (tst != SIPG_OK) return tst;
    SIPG_CUDA_TRY(cudaMalloc(&i.tls, twolevel_scratch_floats(i.tl) * sizeof(float)));
    i.st32 = b->st32 + k;
    i.st64 = b->st64 + k;
    i.fs = b->fs + k;
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
      g.cfg32 = batched_tile(b->inst[k].op->cfg32);
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
      i.tiles32 = tiles_of(i.dim, g.cfg32);
      i.tiles64 = tiles_of(i.dim, g.cfg64);
      ApplyArgs<float> a{};
      a.in = i.p32;  // the direction, formed by k_fcg_inner_direction_batched
      a.out = i.Ap32;
      a.dim = i.dim;
      a.nu = (float)i.pen;
      a.st = i.st32;
      a.red = i.red32;
      args[j] = a;
      ts[j + 1] = ts[j] + i.tiles32;
    }
    g.total32 = ts[m];
    SIPG_CUDA_TRY(cudaMalloc(&g.d_cg, sizeof(ApplyArgs<float>) * m));
    SIPG_CUDA_TRY(cudaMalloc(&g.d_tiles32, sizeof(int) * (m + 1)));
    SIPG_CUDA_TRY(cudaMalloc(&g.d_sub, sizeof(ApplyArgs<double>) * m));
    SIPG_CUDA_TRY(cudaMalloc(&g.d_tiles64, sizeof(int) * (m + 1)));
    SIPG_CUDA_TRY(cudaMemcpy(g.d_cg, args.data(), sizeof(ApplyArgs<float>) * m, cudaMemcpyHostToDevice));
    SIPG_CUDA_TRY(cudaMemcpy(g.d_tiles32, ts.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice));
  }
  // the preconditioner operands in degree-group order, and their launch plan
  std::vector<TlInst> htl;
  std::vector<const HostTables*> tabs;
  for (const BGroup& g : b->groups)
    for (int k : g.members) {
      BInst& i = b->inst[k];
      htl.push_back(twolevel_inst(i.tl, i.tls, i.r32, i.z32, i.st32, i.red32));
      tabs.push_back(&i.op->tab);
    }
  b->tlplan = twolevel_plan(htl.data(), tabs.data(), n);
  SIPG_CUDA_TRY(cudaMalloc(&b->d_tl, sizeof(TlInst) * n));
  SIPG_CUDA_TRY(cudaMemcpy(b->d_tl, htl.data(), sizeof(TlInst) * n, cudaMemcpyHostToDevice));
  std::vector<FcgInst> vec(n);
  for (int k = 0; k < n; ++k) vec[k] = inst_of(b, k, nullptr, nullptr, 1, 0.f);
  SIPG_CUDA_TRY(cudaMalloc(&b->d_vec, sizeof(FcgInst) * n));
  SIPG_CUDA_TRY(cudaMemcpy(b->d_vec, vec.data(), sizeof(FcgInst) * n, cudaMemcpyHostToDevice));
  SIPG_CUDA_TRY(cudaMalloc(&b->d_sel, sizeof(FcgInst) * n));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_sel, sizeof(FcgInst) * n));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_sub, sizeof(ApplyArgs<double>) * n));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_tiles, sizeof(int) * (n + 1)));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_st32, sizeof(CgState<float>) * n));
  SIPG_CUDA_TRY(cudaMallocHost(&b->h_st64, sizeof(CgState<double>) * n));
  SIPG_CUDA_TRY(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
  SIPG_CUDA_TRY(cudaEventCreate(&b->ev0));
  SIPG_CUDA_TRY(cudaEventCreate(&b->ev1));
  long long total = 0;
  for (const BInst& i : b->inst) total += (long long)i.n;
  b->K = total <= (1LL << 22) ? 16 : 8;
  return SIPG_OK;
}

// K FP32 CG iterations of every instance: per degree a batched apply, with a
// batched direction before and a batched update after; captured once.
static sipg_status batch_capture(sipg_batch* b) {
  if (b->exec) return SIPG_OK;
  for (BGroup& g : b->groups)
    SIPG_CUDA_TRY(launch_apply_batched_f32(g.p, g.cfg32, APPLY_PREPARE, nullptr, nullptr, 0, 0,
                                           b->inst[g.members[0]].op->tab, b->cap));
  cudaGraph_t graph = nullptr;
  SIPG_CUDA_TRY(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaSuccess;
  const dim3 vg(b->bpi, b->n);
  // the launches counted while capturing are the graph's, not executed ones
  const unsigned long long c0 = g_launches.load();
  for (int k = 0; k < b->K && err == cudaSuccess; ++k) {
    // z = M r (two-level), p = z + beta p, Ap and alpha, then the update
    if (twolevel_enqueue_batched(b->d_tl, b->tlplan, b->cap) != SIPG_OK) err = cudaErrorUnknown;
    if (err != cudaSuccess) break;
    k_fcg_inner_pdirection_batched<<<vg, kVecThreads, 0, b->cap>>>(b->d_vec);
    count_launch();
    err = cudaGetLastError();
    for (BGroup& g : b->groups) {
      if (err != cudaSuccess) break;
      err = launch_apply_batched_f32(g.p, g.cfg32, APPLY_DOT, g.d_cg, g.d_tiles32, (int)g.members.size(), g.total32,
                                     b->inst[g.members[0]].op->tab, b->cap);
    }
    if (err != cudaSuccess) break;
    k_fcg_inner_pupdate_batched<<<vg, kVecThreads, 0, b->cap>>>(b->d_vec);
    count_launch();
    err = cudaGetLastError();
  }
  const unsigned long long c1 = g_launches.load();
  g_launches.fetch_sub(c1 - c0);
  b->graph_launches = c1 - c0;
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

// FP64 applies of the selected instances, batched per degree: APPLY_RESID
// (r64 = b - A x, r.r) or APPLY_DOT (q = A d, alpha = d.r / d.q).
static sipg_status batch_apply64(sipg_batch* b, const std::vector<int>& sel, int mode, double* const* d_x,
                                 const double* const* d_b, cudaStream_t s) {
  for (BGroup& g : b->groups) {
    int m = 0;
    b->h_tiles[0] = 0;
    for (int k : sel) {
      BInst& i = b->inst[k];
      if (i.p != g.p) continue;
      ApplyArgs<double> a{};
      if (apply_base_mode(mode) == APPLY_RESID) {
        a.in = d_x[k];
        a.out = i.r64;
        a.b = d_b[k];
      } else {
        a.in = i.d64;
        a.out = i.q64;
      }
      a.dim = i.dim;
      a.nu = i.pen;
      a.st = i.st64;
      a.red = i.red64;
      b->h_sub[m] = a;
      b->h_tiles[m + 1] = b->h_tiles[m] + i.tiles64;
      ++m;
    }
    if (!m) continue;
    SIPG_CUDA_TRY(cudaMemcpyAsync(g.d_sub, b->h_sub, sizeof(ApplyArgs<double>) * m, cudaMemcpyHostToDevice, s));
    SIPG_CUDA_TRY(cudaMemcpyAsync(g.d_tiles64, b->h_tiles, sizeof(int) * (m + 1), cudaMemcpyHostToDevice, s));
    SIPG_CUDA_TRY(launch_apply_batched_f64(g.p, g.cfg64, mode, g.d_sub, g.d_tiles64, m, b->h_tiles[m],
                                           b->inst[g.members[0]].op->tab, s));
    // the pinned staging is reused by the next group: wait for the copies
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return SIPG_OK;
}

// Uploads the selection `sel` (with each instance's first-step flag) into d_sel.
static sipg_status upload_sel(sipg_batch* b, const std::vector<int>& sel, double* const* d_x, const double* const* d_b,
                              const std::vector<int>& first, float stop, cudaStream_t s) {
  int m = 0;
  for (int k : sel) b->h_sel[m++] = inst_of(b, k, d_x[k], d_b[k], first[k], stop);
  SIPG_CUDA_TRY(cudaMemcpyAsync(b->d_sel, b->h_sel, sizeof(FcgInst) * m, cudaMemcpyHostToDevice, s));
  return SIPG_OK;
}

static sipg_status read_states(sipg_batch* b, cudaStream_t s, bool inner, bool outer) {
  if (inner)
    SIPG_CUDA_TRY(cudaMemcpyAsync(b->h_st32, b->st32, sizeof(CgState<float>) * b->n, cudaMemcpyDeviceToHost, s));
  if (outer)
    SIPG_CUDA_TRY(cudaMemcpyAsync(b->h_st64, b->st64, sizeof(CgState<double>) * b->n, cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  return SIPG_OK;
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
  for (const BInst& i : b->inst)
    bytes += i.n * (3 * 8 + 5 * 4) + twolevel_scratch_floats(i.tl) * sizeof(float) +
             2 * sizeof(double) * reduce_capacity(i.dim) + sizeof(CgState<double>) + sizeof(CgState<float>) +
             sizeof(FcgState) + sizeof(TlInst);
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
  sipg_mixed_opts o = {1e-2, 1e-10, 200, 0, SIPG_INNER_AUTO, SIPG_OUTER_AUTO};
  if (opts) o = *opts;
  if (!(o.inner_tol > 0) || !(o.inner_tol < 1) || !(o.outer_tol > 0) || o.max_outer < 1) {
    set_error("sipg_batch_solve_mixed: need 0 < inner_tol < 1, outer_tol > 0, max_outer >= 1");
    return SIPG_ERR_INVALID;
  }
  if ((o.inner != SIPG_INNER_AUTO && o.inner != SIPG_INNER_F32_TWOLEVEL) ||
      (o.outer != SIPG_OUTER_AUTO && o.outer != SIPG_OUTER_FLEXIBLE)) {
    set_error("sipg_batch_solve_mixed: batches run the flexible outer kind with the two-level FP32 inner CG");
    return SIPG_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int n = b->n;
  sipg_status st = batch_capture(b);
  if (st != SIPG_OK) return st;
  SIPG_CUDA_TRY(cudaEventRecord(b->ev0, s));
  const float stop_in = (float)o.inner_tol;
  std::vector<int> all(n), first(n, 1), steps(n, 0), fp64(n, 0), retired(n, 0), conv(n, 0);
  for (int k = 0; k < n; ++k) all[k] = k;
  std::vector<double> bnorm(n, 0.0), rel(n, INFINITY);
  std::vector<long long> inner_total(n, 0), max_inner(n);
  for (int k = 0; k < n; ++k) max_inner[k] = o.max_inner > 0 ? o.max_inner : (long long)b->inst[k].n;
  sipg_status status = SIPG_OK;
  auto retire = [&](int k, sipg_status why) {
    retired[k] = 1;
    if (why == SIPG_OK) conv[k] = 1;
    else if (status == SIPG_OK || why == SIPG_ERR_BREAKDOWN) status = why;
  };

  // ||b||, the stop thresholds, every inner state parked; r = b - A x
  st = upload_sel(b, all, d_x, d_b, first, stop_in, s);
  if (st != SIPG_OK) return st;
  k_batch_init<<<dim3(b->bpi, n), kVecThreads, 0, s>>>(b->d_sel, o.outer_tol);
  k_batch_park<<<(n + 127) / 128, 128, 0, s>>>(b->d_sel, n);
  count_launch(2);
  SIPG_CUDA_TRY(cudaGetLastError());
  st = batch_apply64(b, all, APPLY_RESID_PIVOT, d_x, d_b, s);
  if (st != SIPG_OK) return st;
  st = read_states(b, s, false, true);
  if (st != SIPG_OK) return st;
  std::vector<int> cont;
  for (int k = 0; k < n; ++k) {
    fp64[k] = 1;
    bnorm[k] = std::sqrt(b->h_st64[k].bb);
    const double rr = b->h_st64[k].rr;
    rel[k] = bnorm[k] > 0 ? std::sqrt(rr) / bnorm[k] : std::sqrt(rr);
    if (!std::isfinite(rel[k])) retire(k, SIPG_ERR_BREAKDOWN);
    else if (rel[k] <= o.outer_tol || rr == 0.0) retire(k, SIPG_OK);
    else cont.push_back(k);
  }
  for (;;) {
    // inner restarts of the instances that go on
    if (!cont.empty()) {
      st = upload_sel(b, cont, d_x, d_b, first, stop_in, s);
      if (st != SIPG_OK) return st;
      k_fcg_restart_batched<<<dim3(b->bpi, (unsigned)cont.size()), kVecThreads, 0, s>>>(b->d_sel);
      count_launch();
      SIPG_CUDA_TRY(cudaGetLastError());
      SIPG_CUDA_TRY(cudaStreamSynchronize(s));  // h_sel is reused
    }
    bool active = false;
    for (int k = 0; k < n; ++k) active = active || !retired[k];
    if (!active) break;
    // FP32 inner iterations of every instance still in an inner solve
    SIPG_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    count_launch(b->graph_launches);
    st = read_states(b, s, true, false);
    if (st != SIPG_OK) return st;
    std::vector<int> sel;
    for (int k = 0; k < n; ++k) {
      if (retired[k] || !b->h_st32[k].done) continue;
      inner_total[k] += b->h_st32[k].it;
      if (b->h_st32[k].it == 0) retire(k, SIPG_ERR_BREAKDOWN);  // no inner step: no direction
      else sel.push_back(k);
    }
    cont.clear();
    if (sel.empty()) continue;
    // the FP64 outer step of every instance whose inner solve finished
    st = upload_sel(b, sel, d_x, d_b, first, stop_in, s);
    if (st != SIPG_OK) return st;
    const dim3 sg(b->bpi, (unsigned)sel.size());
    k_fcg_gamma_batched<<<sg, kVecThreads, 0, s>>>(b->d_sel);
    k_fcg_direction_batched<<<sg, kVecThreads, 0, s>>>(b->d_sel);
    count_launch(2);
    SIPG_CUDA_TRY(cudaGetLastError());
    {
      std::vector<int> piv, plain;
      for (int k : sel) (rel[k] > kFcgPivotRel ? piv : plain).push_back(k);
      if (!piv.empty()) st = batch_apply64(b, piv, APPLY_DOT_PIVOT, d_x, d_b, s);
      if (st == SIPG_OK && !plain.empty()) st = batch_apply64(b, plain, APPLY_DOT, d_x, d_b, s);
      if (st != SIPG_OK) return st;
    }
    k_fcg_update_batched<<<sg, kVecThreads, 0, s>>>(b->d_sel);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    st = read_states(b, s, false, true);
    if (st != SIPG_OK) return st;
    std::vector<int> chk;
    for (int k : sel) {
      steps[k] += 1;
      fp64[k] += 1;
      first[k] = 0;
      const CgState<double>& h = b->h_st64[k];
      const double r = bnorm[k] > 0 ? std::sqrt(h.rr) / bnorm[k] : std::sqrt(h.rr);
      if (h.status == (int)SIPG_ERR_BREAKDOWN || !std::isfinite(r)) {
        rel[k] = r;
        retire(k, SIPG_ERR_BREAKDOWN);
      } else if (r <= o.outer_tol) {
        chk.push_back(k);
      } else if (steps[k] >= o.max_outer || inner_total[k] >= max_inner[k]) {
        rel[k] = r;
        retire(k, SIPG_ERR_NOT_CONVERGED);
      } else {
        rel[k] = r;
        cont.push_back(k);
      }
    }
    if (!chk.empty()) {
      // the recursion says done: b - A x in FP64 decides
      st = batch_apply64(b, chk, APPLY_RESID_PIVOT, d_x, d_b, s);
      if (st != SIPG_OK) return st;
      st = read_states(b, s, false, true);
      if (st != SIPG_OK) return st;
      for (int k : chk) {
        fp64[k] += 1;
        const double rr = b->h_st64[k].rr;
        rel[k] = bnorm[k] > 0 ? std::sqrt(rr) / bnorm[k] : std::sqrt(rr);
        if (rel[k] <= o.outer_tol) {
          retire(k, SIPG_OK);
        } else if (steps[k] >= o.max_outer || inner_total[k] >= max_inner[k]) {
          retire(k, SIPG_ERR_NOT_CONVERGED);
        } else {
          first[k] = 1;  // a fresh direction history from the true residual
          cont.push_back(k);
        }
      }
    }
  }
  SIPG_CUDA_TRY(cudaEventRecord(b->ev1, s));
  SIPG_CUDA_TRY(cudaEventSynchronize(b->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  if (res)
    for (int k = 0; k < n; ++k) {
      res[k].outer_iterations = steps[k];
      res[k].inner_iterations = (int)inner_total[k];
      res[k].rel_residual = rel[k];
      res[k].time_ms = ms;
      res[k].converged = conv[k];
      res[k].inner_kind = SIPG_INNER_F32_TWOLEVEL;
      res[k].outer_kind = SIPG_OUTER_FLEXIBLE;
      res[k].fp64_applies = fp64[k];
    }
  return status;
}

}  // extern "C"
