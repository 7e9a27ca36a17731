// serve.cu -- a continuous-batching solve server on one GPU (no counterpart in
// the reference).
//
// Requests (mesh size, degree, penalty, right-hand side, relative tolerance,
// precision) wait in a FIFO queue.  Each sipg_server_step():
//   1. admits queued requests while their device footprint fits the budget,
//      a state slot is free and (mixed requests) their preparation (below)
//      has finished (a request larger than the whole budget is
//      rejected); an admitted request gets its vectors from the stream-ordered
//      pool allocator, its right-hand side built on the device, x = 0, and a
//      slot in the device state arrays;
//   2. runs K CG iterations of every active request together: for the mixed
//      requests the FP32 inner CG of the flexible mixed-precision solve
//      (sipg_fcg.cuh), preconditioned by each operator's two-level
//      preconditioner (twolevel.cu; batched over the requests, scratch per
//      request), with per degree one batched FP32 apply launch (the
//      requests' tiles concatenated); for the FP64 ones per degree one
//      batched apply (k_sipg_apply_batched); then one batched update per
//      precision --
//      requests admitted while others are mid-solve simply join the next
//      launches;
//   3. reads all active states with one copy; mixed requests whose inner
//      solve has finished take their FP64 flexible-CG step (batched gamma,
//      direction, FP64 apply and update launches; a batched FP64 residual
//      b - A x before one may stop), then retire or restart their inner
//      solve; FP64 requests that converged retire.
// Retired requests free their vectors at once (their results stay until the
// caller releases them), so memory and slots turn over while others run.
// Meshes/operators are cached and shared; all solver state stays on the device.
//
// A mixed request's operator and two-level preconditioner (host probing and
// Galerkin products, tens of milliseconds for the largest meshes) are built
// by preparation threads from submission on, in submission order, on their
// own streams; admission takes a request once its preparation is done, so
// the stepping thread never waits for it while lanes have work.
//
// Requests run in three lanes by size (up to 2^18 DoF, up to 2^22, larger),
// each with its own stream -- the smaller the solves, the higher the stream
// priority -- its own descriptor staging and its own host mirror of the
// states.  A lane's round is steps 2-3 for its requests; sipg_server_step
// finishes every lane whose round has ended and starts its next one, so a
// lane of small solves turns rounds over (and retires requests) while a lane
// of large ones is mid-round, instead of advancing one iteration per large
// solve's iteration.  The step blocks only when every lane with work is
// mid-round.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "sipg_fcg.cuh"
#include "sipg_twolevel.cuh"

using namespace sipg;

namespace sipg {
sipg_status rhs_f64(const sipg_op* op, int sol, const sipg_modes* modes, double* d_b, cudaStream_t s);

// FP64 request start: r = b (x = 0), stop = tol ||b||, p = r on the first iteration
__global__ void __launch_bounds__(kVecThreads) k_serve_init_f64(const VecInst<double>* __restrict__ insts,
                                                                const double* __restrict__ tols,
                                                                const double* const* __restrict__ bs) {
  __shared__ double sh[32];
  const VecInst<double> v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  const double* __restrict__ b = bs[blockIdx.y];
  double acc = 0.0;
  const size_t stride = (size_t)v.nblk * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < v.n; i += stride) {
    const double bi = b[i];
    v.r[i] = bi;
    v.x[i] = 0.0;
    acc = fma(bi, bi, acc);
  }
  const double bt = block_sum<double, kVecThreads>(acc, sh);
  double total;
  if (grid_sum_last<double, kVecThreads>(bt, v.red, blockIdx.x, v.nblk, sh, &total) && threadIdx.x == 0) {
    CgState<double>* st = v.st;
    st->bb = total;
    st->rr = total;
    st->stop = tols[blockIdx.y] * sqrt(total);
    st->max_it = (int)(v.n < 2000000000 ? v.n : 2000000000);  // as the reference: at most DoF iterations
    st->it = 0;
    st->first = 1;
    st->parity = 0;
    st->status = (int)SIPG_OK;
    st->need_update = 0;
    st->delta = 0.0;
    st->rmax = 0.0;
    st->done = !(sqrt(total) > st->stop);
  }
}

// mixed request start: x = 0, r64 = b, ||b||^2 and the FP64 state (stop =
// tol ||b||); the inner restart (k_fcg_restart_batched) follows on the stream
__global__ void __launch_bounds__(kVecThreads) k_serve_init_fcg(const FcgInst* __restrict__ insts,
                                                                const double* __restrict__ tols) {
  __shared__ double sh[32];
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  double acc = 0.0;
  const size_t stride = (size_t)v.nblk * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < v.n; i += stride) {
    const double bi = v.b[i];
    v.x[i] = 0.0;
    v.r64[i] = bi;
    acc = fma(bi, bi, acc);
  }
  const double bt = block_sum<double, kVecThreads>(acc, sh);
  double total;
  if (grid_sum_last<double, kVecThreads>(bt, v.red64, blockIdx.x, v.nblk, sh, &total) && threadIdx.x == 0) {
    CgState<double>* st = v.st64;
    st->bb = total;
    st->rr = total;
    st->stop = tols[blockIdx.y] * sqrt(total);
    st->max_it = 1 << 30;
    st->it = 0;
    st->first = 1;
    st->parity = 0;
    st->status = (int)SIPG_OK;
    st->need_update = 0;
    st->delta = 0.0;
    st->rmax = 0.0;
    st->done = !(sqrt(total) > st->stop);
  }
}

}  // namespace sipg

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  unsigned long long id = 0;
  sipg_request req{};
  sipg_op* op = nullptr;
  size_t n = 0;
  size_t footprint = 0;
  int slot = -1;
  // device memory: the solution (kept until release) and one pool
  // allocation carved into the solver vectors (freed at retirement)
  char* mem = nullptr;
  double* x64 = nullptr;
  size_t x_bytes = 0;
  double* b64 = nullptr;
  double* r64 = nullptr;     // mixed: FP64 residual; FP64: r
  double* d64 = nullptr;     // mixed: FP64 direction and A d
  double* q64 = nullptr;
  float* e32 = nullptr;      // mixed: FP32 inner solution, residual, direction, A p
  float* r32 = nullptr;
  float* p32 = nullptr;
  float* Ap32 = nullptr;
  float* z32 = nullptr;      // mixed: preconditioned residual
  float* tls = nullptr;      // mixed: the preconditioner's scratch
  void* tl = nullptr;        // mixed: the operator's two-level preconditioner (owned by the op)
  double* p64[2] = {nullptr, nullptr};
  double* Ap64 = nullptr;
  ReduceScratch red32, red64;
  int corrections = 0;        // mixed: flexible outer steps taken
  double rel = 1.0;           // mixed: the relative residual the last outer step or check left
  int first = 1;              // mixed: the next outer step starts a direction history
  long long inner_total = 0;  // mixed: FP32 inner iterations
  int started = 0;
  Clock::time_point t_submit, t_admit, t_done;
  sipg_request_result result{};
  int state = 0;  // 0 queued, 1 active, 2 done
  // mixed requests: the operator and its preconditioner, built by a
  // preparation thread while the request waits (0 pending, 1 done)
  std::atomic<int> prepared{0};
  sipg_status prep_status = SIPG_OK;
};

struct Slots {
  CgState<float>* d32 = nullptr;   // mixed requests' inner (FP32) states
  CgState<double>* d64 = nullptr;  // FP64 CG states, or mixed requests' outer states
  FcgState* fs = nullptr;          // mixed requests' flexible-step scalars
};

// One size class of requests (see the file comment).
struct Lane {
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;      // the end of the lane's round in flight
  bool busy = false;
  std::vector<Request*> active;  // started requests
  std::vector<Request*> fresh;   // admitted; started at the lane's next round
  // pinned mirrors of the slot states, written by this lane's copies only
  CgState<float>* h32 = nullptr;
  CgState<double>* h64 = nullptr;
  // pinned staging and device descriptor arrays (capacity max_active; tile
  // starts max_active + 16): FP32 CG applies, FP64 CG applies, FP64 residuals
  ApplyArgs<float>* h_a32 = nullptr;
  ApplyArgs<float>* d_a32 = nullptr;
  ApplyArgs<double>* h_a64 = nullptr;
  ApplyArgs<double>* d_a64 = nullptr;
  ApplyArgs<double>* h_r64 = nullptr;
  ApplyArgs<double>* d_r64 = nullptr;
  int* h_t32 = nullptr;
  int* d_t32 = nullptr;
  int* h_t64 = nullptr;
  int* d_t64 = nullptr;
  int* h_tr = nullptr;
  int* d_tr = nullptr;
  FcgInst* h_v32 = nullptr;  // the mixed requests of a round (inner kernels)
  FcgInst* d_v32 = nullptr;
  VecInst<double>* h_v64 = nullptr;
  VecInst<double>* d_v64 = nullptr;
  FcgInst* h_m = nullptr;    // a selection of mixed requests (start, outer step, restart)
  FcgInst* d_m = nullptr;
  TlInst* h_tl = nullptr;    // the round's mixed requests' preconditioner operands, by degree
  TlInst* d_tl = nullptr;
  double* h_tol = nullptr;
  double* d_tol = nullptr;
  const double** h_bptr = nullptr;
  const double** d_bptr = nullptr;
};

constexpr int kLanes = 3;
int lane_of(size_t n) { return n <= (size_t(1) << 18) ? 0 : (n <= (size_t(1) << 22) ? 1 : 2); }

}  // namespace

struct sipg_server {
  sipg_server_opts opts{};
  cudaStream_t s = nullptr;  // solution copies and releases
  Slots slots;
  std::vector<int> free_slots;
  std::deque<Request*> queue;
  std::unordered_map<unsigned long long, Request*> all;
  std::map<std::tuple<int, int, double>, sipg_op*> ops;
  unsigned long long next_id = 1;
  size_t used = 0;
  Lane lanes[kLanes];
  unsigned long long completed = 0, rejected = 0;
  double setup_ms = 0;  // admission: operator and preconditioner set-up on the stepping thread
  // preparation threads: build mixed requests' operators and preconditioners
  // (host work and probes on their own streams) while the lanes run, in
  // submission order
  int device = 0;
  std::mutex ops_mu;  // sv->ops is shared with the preparation threads
  std::mutex prep_mu;
  std::condition_variable prep_cv;
  std::deque<Request*> prep_todo;
  std::vector<std::thread> prep_workers;
  bool prep_stop = false;
  std::atomic<long long> prep_us{0};  // their busy time
};

namespace {

// grid width of a batched vector launch: the widest listed instance
int vec_bpi(size_t nmax, int) { return inst_blocks(nmax); }

size_t footprint_of(int dim, int p, int precision) {
  const size_t n = (size_t)dim * dim * (p + 1) * (p + 1);
  const size_t red = 2 * (sizeof(double) * (size_t)reduce_capacity(dim) + 256);
  if (precision == SIPG_F64) return n * (8 * 2 + 8 * 4) + red + 4096;  // x, b, r, p0, p1, Ap
  return n * (8 * 5 + 4 * 5) + twolevel_scratch_floats_for(dim) * 4 + red + 4096;  // x, b, r, d, q + FP32 e, r, p, Ap, z
}

sipg_status get_op(sipg_server* sv, int dim, int p, double pen, sipg_op** out) {
  std::lock_guard<std::mutex> lock(sv->ops_mu);
  const auto key = std::make_tuple(dim, p, pen);
  auto it = sv->ops.find(key);
  if (it != sv->ops.end()) {
    *out = it->second;
    return SIPG_OK;
  }
  sipg_op* op = nullptr;
  sipg_status st = sipg_op_create(dim, p, pen, &op);
  if (st != SIPG_OK) return st;
  sv->ops[key] = op;
  *out = op;
  return SIPG_OK;
}

// A preparation thread: takes mixed requests in submission order and builds
// each one's operator and two-level preconditioner (the first request of an
// operator builds it; later ones find it).
void prep_loop(sipg_server* sv) {
  cudaSetDevice(sv->device);
  for (;;) {
    Request* r = nullptr;
    {
      std::unique_lock<std::mutex> lock(sv->prep_mu);
      sv->prep_cv.wait(lock, [&] { return sv->prep_stop || !sv->prep_todo.empty(); });
      if (sv->prep_stop) return;
      r = sv->prep_todo.front();
      sv->prep_todo.pop_front();
    }
    const auto t0 = Clock::now();
    sipg_op* op = nullptr;
    sipg_status st = get_op(sv, r->req.dim, r->req.degree, r->req.pen, &op);
    void* tl = nullptr;
    if (st == SIPG_OK) st = twolevel_get(op, &tl);
    sv->prep_us += std::chrono::duration_cast<std::chrono::microseconds>(Clock::now() - t0).count();
    r->prep_status = st;
    r->prepared.store(1, std::memory_order_release);
  }
}

// preparation threads: up to six (a request's set-up is mostly host work,
// tens of milliseconds at the largest meshes), fewer on a small host
int prep_threads() {
  const unsigned hw = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(6u, hw / 2));
}

// Gives back what admit() took before one of its steps failed: the request
// then holds no device memory and no slot.
sipg_status admit_rollback(Request* r, cudaStream_t s, sipg_status st) {
  if (r->mem) cudaFreeAsync(r->mem, s);
  if (r->x64) cudaFreeAsync(r->x64, s);
  r->mem = nullptr;
  r->x64 = nullptr;
  return st;
}

// carve one pool allocation into the request's vectors
sipg_status admit(sipg_server* sv, Request* r, cudaStream_t s) {
  r->x_bytes = r->n * sizeof(double);
  r->x64 = nullptr;
  r->mem = nullptr;
  void* xa = nullptr;
  void* ma = nullptr;
  cudaError_t e = cudaMallocAsync(&xa, r->x_bytes, s);
  if (e == cudaSuccess) {
    r->x64 = (double*)xa;
    e = cudaMallocAsync(&ma, r->footprint - r->x_bytes, s);
    if (e == cudaSuccess) r->mem = (char*)ma;
  }
  if (e != cudaSuccess) {
    set_error(std::string("sipg_server_step: admission failed: ") + cudaGetErrorString(e));
    return admit_rollback(r, s, e == cudaErrorMemoryAllocation ? SIPG_ERR_NOMEM : SIPG_ERR_CUDA);
  }
  char* p = r->mem;
  auto take = [&](size_t bytes) {
    char* q = p;
    p += (bytes + 255) & ~size_t(255);
    return q;
  };
  const size_t n = r->n;
  const int cap = reduce_capacity(r->req.dim);
  r->b64 = (double*)take(n * 8);
  r->r64 = (double*)take(n * 8);
  if (r->req.precision == SIPG_F64) {
    r->p64[0] = (double*)take(n * 8);
    r->p64[1] = (double*)take(n * 8);
    r->Ap64 = (double*)take(n * 8);
  } else {
    r->d64 = (double*)take(n * 8);
    r->q64 = (double*)take(n * 8);
    r->e32 = (float*)take(n * 4);
    r->r32 = (float*)take(n * 4);
    r->p32 = (float*)take(n * 4);
    r->Ap32 = (float*)take(n * 4);
    r->z32 = (float*)take(n * 4);
    r->tls = (float*)take(twolevel_scratch_floats_for(r->req.dim) * 4);
  }
  r->red32.partials = (double*)take(sizeof(double) * cap);
  r->red32.counter = (unsigned int*)take(256);
  r->red32.capacity = cap;
  r->red64.partials = (double*)take(sizeof(double) * cap);
  r->red64.counter = (unsigned int*)take(256);
  r->red64.capacity = cap;
  e = cudaMemsetAsync(r->red32.counter, 0, 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(r->red64.counter, 0, 4, s);
  if (e != cudaSuccess) {
    set_error(std::string("sipg_server_step: admission failed: ") + cudaGetErrorString(e));
    return admit_rollback(r, s, SIPG_ERR_CUDA);
  }
  const sipg_modes* modes = (r->req.sol == SIPG_SOL_MODES) ? &r->req.modes : nullptr;
  sipg_status st = rhs_f64(r->op, r->req.sol, modes, r->b64, s);
  if (st != SIPG_OK) return admit_rollback(r, s, st);
  if (r->req.precision != SIPG_F64) {
    // the operator's preconditioner, built on its first mixed request (synchronous)
    st = twolevel_get(r->op, &r->tl);
    if (st != SIPG_OK) return admit_rollback(r, s, st);
  }
  r->slot = sv->free_slots.back();
  sv->free_slots.pop_back();
  sv->used += r->footprint;
  r->state = 1;
  r->started = 0;
  r->t_admit = Clock::now();
  return SIPG_OK;
}

void retire(sipg_server* sv, Request* r, cudaStream_t s, sipg_status status, int iterations, double rel) {
  r->t_done = Clock::now();
  r->result.status = status;
  r->result.iterations = iterations;
  r->result.corrections = r->corrections;
  r->result.rel_residual = rel;
  r->result.queue_ms = std::chrono::duration<double, std::milli>(r->t_admit - r->t_submit).count();
  r->result.latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  r->result.done = 1;
  cudaFreeAsync(r->mem, s);
  r->mem = nullptr;
  sv->used -= r->footprint - r->x_bytes;  // the solution stays until release
  sv->free_slots.push_back(r->slot);
  r->slot = -1;
  r->state = 2;
  sv->completed++;
}

ApplyArgs<float> cg_args32(const Request* r, sipg_server* sv) {
  ApplyArgs<float> a{};
  a.in = r->p32;  // the direction, formed by k_fcg_inner_direction_batched
  a.out = r->Ap32;
  a.dim = r->req.dim;
  a.nu = (float)r->req.pen;
  a.st = sv->slots.d32 + r->slot;
  a.red = r->red32;
  return a;
}

ApplyArgs<double> cg_args64(const Request* r, sipg_server* sv) {
  ApplyArgs<double> a{};
  a.in = r->r64;
  a.pbuf0 = r->p64[0];
  a.pbuf1 = r->p64[1];
  a.out = r->Ap64;
  a.dim = r->req.dim;
  a.nu = r->req.pen;
  a.st = sv->slots.d64 + r->slot;
  a.red = r->red64;
  return a;
}

// inner iterations one preconditioner solve may take
constexpr int kInnerCap = 4000;

FcgInst fcg_of(const Request* r, sipg_server* sv) {
  FcgInst v;
  v.x = r->x64;
  v.b = r->b64;
  v.r64 = r->r64;
  v.d64 = r->d64;
  v.q64 = r->q64;
  v.r32 = r->r32;
  v.e32 = r->e32;
  v.p32 = r->p32;
  v.Ap32 = r->Ap32;
  v.z32 = r->z32;
  v.st32 = sv->slots.d32 + r->slot;
  v.st64 = sv->slots.d64 + r->slot;
  v.fs = sv->slots.fs + r->slot;
  v.red32 = r->red32;
  v.red64 = r->red64;
  v.n = r->n;
  v.nblk = inst_blocks(r->n);
  v.first = r->first;
  v.stop = (float)sv->opts.inner_tol;
  v.max_it = kInnerCap;
  return v;
}

// A list of requests grouped by degree, packed into one descriptor array
// (group g's arguments from `off`, its tile starts from `toff`).
struct GroupLaunch {
  int p;
  int key;  // the caller's split of a degree's requests (0 unless it asks for one)
  TileCfg cfg;
  int off, m, toff, total;
  const HostTables* tab;
};

// The requests of `list` grouped by (degree, key(request)), their apply
// arguments in h_a and tile offsets in h_t.
template <typename T, typename Build, typename Key>
std::vector<GroupLaunch> pack_groups(const std::vector<Request*>& list, ApplyArgs<T>* h_a, int* h_t, Build build,
                                     Key key) {
  std::map<std::pair<int, int>, std::vector<Request*>> by_p;
  for (Request* r : list) by_p[{r->req.degree, key(r)}].push_back(r);
  std::vector<GroupLaunch> out;
  int off = 0, toff = 0;
  for (auto& kv : by_p) {
    const std::vector<Request*>& g = kv.second;
    GroupLaunch gl;
    gl.p = kv.first.first;
    gl.key = kv.first.second;
    gl.cfg = batched_tile((sizeof(T) == 8) ? g[0]->op->cfg64 : g[0]->op->cfg32);
    gl.off = off;
    gl.m = (int)g.size();
    gl.toff = toff;
    gl.tab = &g[0]->op->tab;
    h_t[toff] = 0;
    for (int j = 0; j < gl.m; ++j) {
      h_a[off + j] = build(g[j]);
      h_t[toff + j + 1] = h_t[toff + j] + apply_grid_blocks(g[j]->req.dim, gl.cfg);
    }
    gl.total = h_t[toff + gl.m];
    off += gl.m;
    toff += gl.m + 1;
    out.push_back(gl);
  }
  return out;
}
template <typename T, typename Build>
std::vector<GroupLaunch> pack_groups(const std::vector<Request*>& list, ApplyArgs<T>* h_a, int* h_t, Build build) {
  return pack_groups<T>(list, h_a, h_t, build, [](const Request*) { return 0; });
}

template <typename T>
sipg_status upload_groups(const std::vector<GroupLaunch>& gs, const ApplyArgs<T>* h_a, ApplyArgs<T>* d_a, const int* h_t,
                          int* d_t, cudaStream_t s) {
  if (gs.empty()) return SIPG_OK;
  const GroupLaunch& last = gs.back();
  SIPG_CUDA_TRY(cudaMemcpyAsync(d_a, h_a, sizeof(ApplyArgs<T>) * (last.off + last.m), cudaMemcpyHostToDevice, s));
  SIPG_CUDA_TRY(cudaMemcpyAsync(d_t, h_t, sizeof(int) * (last.toff + last.m + 1), cudaMemcpyHostToDevice, s));
  return SIPG_OK;
}

// Launches every group in `mode` (groups of key 1: in mode_key1 when that is given).
template <typename T>
sipg_status launch_groups(const std::vector<GroupLaunch>& gs, int mode, const ApplyArgs<T>* d_a, const int* d_t,
                          cudaStream_t s, int mode_key1 = -1) {
  for (const GroupLaunch& g : gs) {
    const int mode_g = (g.key == 1 && mode_key1 >= 0) ? mode_key1 : mode;
    cudaError_t e = (sizeof(T) == 8)
                        ? launch_apply_batched_f64(g.p, g.cfg, mode_g, (const ApplyArgs<double>*)(d_a + g.off),
                                                   d_t + g.toff, g.m, g.total, *g.tab, s)
                        : launch_apply_batched_f32(g.p, g.cfg, mode_g, (const ApplyArgs<float>*)(d_a + g.off),
                                                   d_t + g.toff, g.m, g.total, *g.tab, s);
    SIPG_CUDA_TRY(e);
  }
  return SIPG_OK;
}

sipg_status server_alloc(sipg_server* sv) {
  const int cap = sv->opts.max_active;
  SIPG_CUDA_TRY(cudaStreamCreateWithFlags(&sv->s, cudaStreamNonBlocking));
  {
    // requests take their vectors from the device's default memory pool
    // (stream-ordered); let it keep up to the budget mapped between
    // synchronisations instead of returning it to the driver each time, so
    // that an admission reuses memory rather than mapping it again
    int dev = 0;
    cudaMemPool_t pool = nullptr;
    SIPG_CUDA_TRY(cudaGetDevice(&dev));
    sv->device = dev;
    SIPG_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, dev));
    unsigned long long keep = 0;  // the attribute is a 64-bit unsigned value
    SIPG_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    if (keep < (unsigned long long)sv->opts.budget_bytes) {
      keep = (unsigned long long)sv->opts.budget_bytes;
      SIPG_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
  }
  SIPG_CUDA_TRY(cudaMalloc(&sv->slots.d32, sizeof(CgState<float>) * cap));
  SIPG_CUDA_TRY(cudaMalloc(&sv->slots.d64, sizeof(CgState<double>) * cap));
  SIPG_CUDA_TRY(cudaMalloc(&sv->slots.fs, sizeof(FcgState) * cap));
  SIPG_CUDA_TRY(cudaMemset(sv->slots.d32, 0, sizeof(CgState<float>) * cap));
  SIPG_CUDA_TRY(cudaMemset(sv->slots.d64, 0, sizeof(CgState<double>) * cap));
  SIPG_CUDA_TRY(cudaMemset(sv->slots.fs, 0, sizeof(FcgState) * cap));
  int least = 0, greatest = 0;  // numerically: greatest priority is the lowest value
  SIPG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  for (int k = 0; k < kLanes; ++k) {
    Lane& L = sv->lanes[k];
    const int prio = greatest + (least - greatest) * k / (kLanes - 1);
    SIPG_CUDA_TRY(cudaStreamCreateWithPriority(&L.s, cudaStreamNonBlocking, prio));
    SIPG_CUDA_TRY(cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h32, sizeof(CgState<float>) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h64, sizeof(CgState<double>) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_a32, sizeof(ApplyArgs<float>) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_a32, sizeof(ApplyArgs<float>) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_a64, sizeof(ApplyArgs<double>) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_a64, sizeof(ApplyArgs<double>) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_r64, sizeof(ApplyArgs<double>) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_r64, sizeof(ApplyArgs<double>) * cap));
    int** tiles_h[3] = {&L.h_t32, &L.h_t64, &L.h_tr};
    int** tiles_d[3] = {&L.d_t32, &L.d_t64, &L.d_tr};
    for (int t = 0; t < 3; ++t) {
      SIPG_CUDA_TRY(cudaMallocHost(tiles_h[t], sizeof(int) * (cap + 16)));
      SIPG_CUDA_TRY(cudaMalloc(tiles_d[t], sizeof(int) * (cap + 16)));
    }
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_v32, sizeof(FcgInst) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_v32, sizeof(FcgInst) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_v64, sizeof(VecInst<double>) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_v64, sizeof(VecInst<double>) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_m, sizeof(FcgInst) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_m, sizeof(FcgInst) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_tl, sizeof(TlInst) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_tl, sizeof(TlInst) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_tol, sizeof(double) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_tol, sizeof(double) * cap));
    SIPG_CUDA_TRY(cudaMallocHost(&L.h_bptr, sizeof(double*) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&L.d_bptr, sizeof(double*) * cap));
  }
  for (int k = cap - 1; k >= 0; --k) sv->free_slots.push_back(k);
  return SIPG_OK;
}

void server_free(sipg_server* sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lock(sv->prep_mu);
    sv->prep_stop = true;
  }
  sv->prep_cv.notify_all();
  for (std::thread& t : sv->prep_workers) t.join();
  sv->prep_workers.clear();
  for (Lane& L : sv->lanes)
    if (L.s) cudaStreamSynchronize(L.s);
  if (sv->s) cudaStreamSynchronize(sv->s);
  // every request, queued or not, is in sv->all (submit enters it there first)
  for (auto& kv : sv->all) {
    if (kv.second->mem) cudaFreeAsync(kv.second->mem, sv->s);
    if (kv.second->x64) cudaFreeAsync(kv.second->x64, sv->s);
    delete kv.second;
  }
  sv->all.clear();
  sv->queue.clear();
  sv->prep_todo.clear();
  if (sv->s) cudaStreamSynchronize(sv->s);
  cudaFree(sv->slots.d32);
  cudaFree(sv->slots.d64);
  cudaFree(sv->slots.fs);
  for (Lane& L : sv->lanes) {
    cudaFreeHost(L.h32);
    cudaFreeHost(L.h64);
    cudaFreeHost(L.h_a32);
    cudaFree(L.d_a32);
    cudaFreeHost(L.h_a64);
    cudaFree(L.d_a64);
    cudaFreeHost(L.h_r64);
    cudaFree(L.d_r64);
    cudaFreeHost(L.h_t32);
    cudaFree(L.d_t32);
    cudaFreeHost(L.h_t64);
    cudaFree(L.d_t64);
    cudaFreeHost(L.h_tr);
    cudaFree(L.d_tr);
    cudaFreeHost(L.h_v32);
    cudaFree(L.d_v32);
    cudaFreeHost(L.h_v64);
    cudaFree(L.d_v64);
    cudaFreeHost(L.h_m);
    cudaFree(L.d_m);
    cudaFreeHost(L.h_tl);
    cudaFree(L.d_tl);
    cudaFreeHost(L.h_tol);
    cudaFree(L.d_tol);
    cudaFreeHost(L.h_bptr);
    cudaFree(L.d_bptr);
    if (L.ev) cudaEventDestroy(L.ev);
    if (L.s) cudaStreamDestroy(L.s);
  }
  for (auto& kv : sv->ops) sipg_op_destroy(kv.second);
  if (sv->s) cudaStreamDestroy(sv->s);
  delete sv;
}

int active_count(const sipg_server* sv) {
  int n = 0;
  for (const Lane& L : sv->lanes) n += (int)(L.active.size() + L.fresh.size());
  return n;
}

// Starts the lane's admitted requests (x = 0, r = b; one batched launch per
// precision) and moves them to its active list.  Synchronous on the lane's
// stream (its staging is reused for the round that follows).
sipg_status lane_start(sipg_server* sv, Lane& L) {
  int m32 = 0, m64 = 0;
  size_t nmax32 = 0, nmax64 = 0;
  for (Request* r : L.fresh) {
    if (r->req.precision == SIPG_F64) {
      VecInst<double> v;
      v.x = r->x64;
      v.pb0 = r->p64[0];
      v.pb1 = r->p64[1];
      v.r = r->r64;
      v.Ap = r->Ap64;
      v.n = r->n;
      v.st = sv->slots.d64 + r->slot;
      v.red = r->red64;
      v.nblk = inst_blocks(r->n);
      v.pad = 0;
      L.h_v64[m64] = v;
      L.h_tol[m64] = r->req.tol;
      L.h_bptr[m64] = r->b64;
      nmax64 = std::max(nmax64, r->n);
      ++m64;
    } else {
      r->first = 1;
      L.h_m[m32++] = fcg_of(r, sv);
      nmax32 = std::max(nmax32, r->n);
    }
  }
  // the mixed requests' tolerances follow the FP64 ones in the staging
  {
    int j = 0;
    for (Request* r : L.fresh)
      if (r->req.precision != SIPG_F64) L.h_tol[m64 + j++] = r->req.tol;
  }
  if (m64 + m32) SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_tol, L.h_tol, sizeof(double) * (m64 + m32), cudaMemcpyHostToDevice, L.s));
  if (m64) {
    SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_v64, L.h_v64, sizeof(VecInst<double>) * m64, cudaMemcpyHostToDevice, L.s));
    SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_bptr, L.h_bptr, sizeof(double*) * m64, cudaMemcpyHostToDevice, L.s));
    k_serve_init_f64<<<dim3(vec_bpi(nmax64, m64), m64), kVecThreads, 0, L.s>>>(L.d_v64, L.d_tol, L.d_bptr);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
  }
  if (m32) {
    SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_m, L.h_m, sizeof(FcgInst) * m32, cudaMemcpyHostToDevice, L.s));
    const dim3 g(vec_bpi(nmax32, m32), m32);
    k_serve_init_fcg<<<g, kVecThreads, 0, L.s>>>(L.d_m, L.d_tol + m64);
    k_fcg_restart_batched<<<g, kVecThreads, 0, L.s>>>(L.d_m);
    count_launch(2);
    SIPG_CUDA_TRY(cudaGetLastError());
  }
  SIPG_CUDA_TRY(cudaStreamSynchronize(L.s));
  L.active.insert(L.active.end(), L.fresh.begin(), L.fresh.end());
  L.fresh.clear();
  return SIPG_OK;
}

// Queues a round for the lane: iters_per_step CG iterations of its active
// requests (per precision: one batched launch per degree and kernel), the
// copy of the slot states into the lane's mirrors, and the lane's event.
sipg_status lane_launch(sipg_server* sv, Lane& L) {
  std::vector<Request*> a32, a64;
  for (Request* r : L.active) (r->req.precision == SIPG_F64 ? a64 : a32).push_back(r);
  size_t nmax32 = 0, nmax64 = 0;
  for (int j = 0; j < (int)a32.size(); ++j) {
    Request* r = a32[j];
    L.h_v32[j] = fcg_of(r, sv);
    nmax32 = std::max(nmax32, r->n);
  }
  for (int j = 0; j < (int)a64.size(); ++j) {
    Request* r = a64[j];
    VecInst<double> v;
    v.x = r->x64;
    v.pb0 = r->p64[0];
    v.pb1 = r->p64[1];
    v.r = r->r64;
    v.Ap = r->Ap64;
    v.n = r->n;
    v.st = sv->slots.d64 + r->slot;
    v.red = r->red64;
    v.nblk = inst_blocks(r->n);
    v.pad = 0;
    L.h_v64[j] = v;
    nmax64 = std::max(nmax64, r->n);
  }
  TlPlan tlplan;
  if (!a32.empty()) {
    SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_v32, L.h_v32, sizeof(FcgInst) * a32.size(), cudaMemcpyHostToDevice, L.s));
    // the preconditioner operands, grouped by degree
    std::vector<Request*> byp(a32);
    std::stable_sort(byp.begin(), byp.end(),
                     [](const Request* x, const Request* y) { return x->req.degree < y->req.degree; });
    std::vector<const HostTables*> tabs;
    for (size_t j = 0; j < byp.size(); ++j) {
      Request* r = byp[j];
      L.h_tl[j] = twolevel_inst(r->tl, r->tls, r->r32, r->z32, sv->slots.d32 + r->slot, r->red32);
      tabs.push_back(&r->op->tab);
    }
    tlplan = twolevel_plan(L.h_tl, tabs.data(), (int)byp.size());
    SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_tl, L.h_tl, sizeof(TlInst) * byp.size(), cudaMemcpyHostToDevice, L.s));
  }
  if (!a64.empty())
    SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_v64, L.h_v64, sizeof(VecInst<double>) * a64.size(), cudaMemcpyHostToDevice, L.s));
  const std::vector<GroupLaunch> g32 =
      pack_groups<float>(a32, L.h_a32, L.h_t32, [&](const Request* r) { return cg_args32(r, sv); });
  const std::vector<GroupLaunch> g64 =
      pack_groups<double>(a64, L.h_a64, L.h_t64, [&](const Request* r) { return cg_args64(r, sv); });
  {
    sipg_status st = upload_groups<float>(g32, L.h_a32, L.d_a32, L.h_t32, L.d_t32, L.s);
    if (st == SIPG_OK) st = upload_groups<double>(g64, L.h_a64, L.d_a64, L.h_t64, L.d_t64, L.s);
    if (st != SIPG_OK) return st;
  }
  for (int k = 0; k < sv->opts.iters_per_step; ++k) {
    if (!a32.empty()) {
      const dim3 vg(vec_bpi(nmax32, (int)a32.size()), (unsigned)a32.size());
      sipg_status st = twolevel_enqueue_batched(L.d_tl, tlplan, L.s);
      if (st != SIPG_OK) return st;
      k_fcg_inner_pdirection_batched<<<vg, kVecThreads, 0, L.s>>>(L.d_v32);
      count_launch();
      SIPG_CUDA_TRY(cudaGetLastError());
      st = launch_groups<float>(g32, APPLY_DOT, L.d_a32, L.d_t32, L.s);
      if (st != SIPG_OK) return st;
      k_fcg_inner_pupdate_batched<<<vg, kVecThreads, 0, L.s>>>(L.d_v32);
      count_launch();
      SIPG_CUDA_TRY(cudaGetLastError());
    }
    if (!a64.empty()) {
      sipg_status st = launch_groups<double>(g64, APPLY_CG, L.d_a64, L.d_t64, L.s);
      if (st != SIPG_OK) return st;
      k_cg_update_batched<double><<<dim3(vec_bpi(nmax64, (int)a64.size()), (unsigned)a64.size()), kVecThreads, 0,
                                    L.s>>>(L.d_v64);
      count_launch();
      SIPG_CUDA_TRY(cudaGetLastError());
    }
  }
  const int cap = sv->opts.max_active;
  SIPG_CUDA_TRY(cudaMemcpyAsync(L.h32, sv->slots.d32, sizeof(CgState<float>) * cap, cudaMemcpyDeviceToHost, L.s));
  SIPG_CUDA_TRY(cudaMemcpyAsync(L.h64, sv->slots.d64, sizeof(CgState<double>) * cap, cudaMemcpyDeviceToHost, L.s));
  SIPG_CUDA_TRY(cudaEventRecord(L.ev, L.s));
  L.busy = true;
  return SIPG_OK;
}

// After a lane's round: FP64 requests that are done retire; mixed requests
// whose inner solve finished take their flexible-CG step in FP64 (batched,
// synchronously on the lane's stream), then retire -- after b - A x in FP64
// confirms the target -- or restart their inner solve.
sipg_status lane_finish(sipg_server* sv, Lane& L) {
  std::vector<Request*> keep, fix;
  for (Request* r : L.active) {
    if (r->req.precision == SIPG_F64) {
      const CgState<double>& h = L.h64[r->slot];
      if (h.done) {
        const bool conv = !(std::sqrt(h.rr) > h.stop);
        const double rel = h.bb > 0 ? std::sqrt(h.rr / h.bb) : 0.0;
        retire(sv, r, L.s,
               h.status == (int)SIPG_ERR_BREAKDOWN ? SIPG_ERR_BREAKDOWN : (conv ? SIPG_OK : SIPG_ERR_NOT_CONVERGED),
               h.it, rel);
      } else {
        keep.push_back(r);
      }
      continue;
    }
    const CgState<float>& h32 = L.h32[r->slot];
    if (!h32.done) {
      keep.push_back(r);
      continue;
    }
    r->inner_total += h32.it;
    if (h32.it == 0) {
      // no inner step: a zero residual (b = 0 or x exact) retires, else there is no direction
      const CgState<double>& h = L.h64[r->slot];
      const double rel = h.bb > 0 ? std::sqrt(h.rr / h.bb) : 0.0;
      retire(sv, r, L.s, h.rr == 0.0 ? SIPG_OK : SIPG_ERR_BREAKDOWN, (int)r->inner_total, rel);
      continue;
    }
    fix.push_back(r);
  }
  if (!fix.empty()) {
    const int cap = sv->opts.max_active;
    int m = 0;
    size_t nmax = 0;
    for (Request* r : fix) {
      L.h_m[m++] = fcg_of(r, sv);
      nmax = std::max(nmax, r->n);
    }
    const dim3 g(vec_bpi(nmax, m), m);
    SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_m, L.h_m, sizeof(FcgInst) * m, cudaMemcpyHostToDevice, L.s));
    k_fcg_gamma_batched<<<g, kVecThreads, 0, L.s>>>(L.d_m);
    k_fcg_direction_batched<<<g, kVecThreads, 0, L.s>>>(L.d_m);
    count_launch(2);
    SIPG_CUDA_TRY(cudaGetLastError());
    // q = A d in FP64, alpha = d.r / d.q
    const std::vector<GroupLaunch> gq = pack_groups<double>(fix, L.h_r64, L.h_tr, [&](const Request* r) {
      ApplyArgs<double> a{};
      a.in = r->d64;
      a.out = r->q64;
      a.dim = r->req.dim;
      a.nu = r->req.pen;
      a.st = sv->slots.d64 + r->slot;
      a.red = r->red64;
      return a;
    }, [](const Request* r) { return r->rel > kFcgPivotRel ? 1 : 0; });
    sipg_status st = upload_groups<double>(gq, L.h_r64, L.d_r64, L.h_tr, L.d_tr, L.s);
    if (st == SIPG_OK) st = launch_groups<double>(gq, APPLY_DOT, L.d_r64, L.d_tr, L.s, APPLY_DOT_PIVOT);
    if (st != SIPG_OK) return st;
    k_fcg_update_batched<<<g, kVecThreads, 0, L.s>>>(L.d_m);
    count_launch();
    SIPG_CUDA_TRY(cudaGetLastError());
    SIPG_CUDA_TRY(cudaMemcpyAsync(L.h64, sv->slots.d64, sizeof(CgState<double>) * cap, cudaMemcpyDeviceToHost, L.s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(L.s));
    std::vector<Request*> cont, chk;
    for (Request* r : fix) {
      r->corrections++;
      r->first = 0;
      const CgState<double>& h = L.h64[r->slot];
      const double rel = h.bb > 0 ? std::sqrt(h.rr / h.bb) : std::sqrt(h.rr);
      if (!std::isfinite(rel) || h.status == (int)SIPG_ERR_BREAKDOWN) {
        retire(sv, r, L.s, SIPG_ERR_BREAKDOWN, (int)r->inner_total, rel);
      } else if (rel <= r->req.tol) {
        chk.push_back(r);
      } else if (r->corrections >= 1000) {
        retire(sv, r, L.s, SIPG_ERR_NOT_CONVERGED, (int)r->inner_total, rel);
      } else {
        r->rel = rel;
        cont.push_back(r);
      }
    }
    if (!chk.empty()) {
      // the recursion says done: b - A x in FP64 decides
      const std::vector<GroupLaunch> gr = pack_groups<double>(chk, L.h_r64, L.h_tr, [&](const Request* r) {
        ApplyArgs<double> a{};
        a.in = r->x64;
        a.out = r->r64;
        a.b = r->b64;
        a.dim = r->req.dim;
        a.nu = r->req.pen;
        a.st = sv->slots.d64 + r->slot;
        a.red = r->red64;
        return a;
      });
      st = upload_groups<double>(gr, L.h_r64, L.d_r64, L.h_tr, L.d_tr, L.s);
      if (st == SIPG_OK) st = launch_groups<double>(gr, APPLY_RESID_PIVOT, L.d_r64, L.d_tr, L.s);
      if (st != SIPG_OK) return st;
      SIPG_CUDA_TRY(
          cudaMemcpyAsync(L.h64, sv->slots.d64, sizeof(CgState<double>) * cap, cudaMemcpyDeviceToHost, L.s));
      SIPG_CUDA_TRY(cudaStreamSynchronize(L.s));
      for (Request* r : chk) {
        const CgState<double>& h = L.h64[r->slot];
        const double rel = h.bb > 0 ? std::sqrt(h.rr / h.bb) : std::sqrt(h.rr);
        if (rel <= r->req.tol) {
          retire(sv, r, L.s, SIPG_OK, (int)r->inner_total, rel);
        } else if (r->corrections >= 1000 || !std::isfinite(rel)) {
          retire(sv, r, L.s, std::isfinite(rel) ? SIPG_ERR_NOT_CONVERGED : SIPG_ERR_BREAKDOWN, (int)r->inner_total,
                 rel);
        } else {
          r->first = 1;  // a fresh direction history from the true residual
          r->rel = rel;
          cont.push_back(r);
        }
      }
    }
    if (!cont.empty()) {
      m = 0;
      nmax = 0;
      for (Request* r : cont) {
        L.h_m[m++] = fcg_of(r, sv);
        nmax = std::max(nmax, r->n);
      }
      SIPG_CUDA_TRY(cudaMemcpyAsync(L.d_m, L.h_m, sizeof(FcgInst) * m, cudaMemcpyHostToDevice, L.s));
      k_fcg_restart_batched<<<dim3(vec_bpi(nmax, m), m), kVecThreads, 0, L.s>>>(L.d_m);
      count_launch();
      SIPG_CUDA_TRY(cudaGetLastError());
      for (Request* r : cont) keep.push_back(r);
    }
    // the pinned staging (h_m) is rewritten by the lane's next round
    SIPG_CUDA_TRY(cudaStreamSynchronize(L.s));
  }
  L.active = keep;
  return SIPG_OK;
}

}  // namespace

extern "C" {

sipg_status sipg_server_create(const sipg_server_opts* opts, sipg_server** out) {
  if (!out) return SIPG_ERR_INVALID;
  *out = nullptr;
  sipg_server* sv = new (std::nothrow) sipg_server;
  if (!sv) return SIPG_ERR_NOMEM;
  sipg_server_opts o = {150ull << 30, 256, 8, 1e-2};
  if (opts) o = *opts;
  if (o.max_active < 1 || o.max_active > 4096 || o.iters_per_step < 1 || !(o.inner_tol > 0 && o.inner_tol < 1)) {
    set_error("sipg_server_create: need 1 <= max_active <= 4096, iters_per_step >= 1, 0 < inner_tol < 1");
    delete sv;
    return SIPG_ERR_INVALID;
  }
  sv->opts = o;
  sipg_status st = server_alloc(sv);
  if (st != SIPG_OK) {
    server_free(sv);
    return st;
  }
  for (int k = 0, n = prep_threads(); k < n; ++k) sv->prep_workers.emplace_back(prep_loop, sv);
  *out = sv;
  return SIPG_OK;
}

sipg_status sipg_server_destroy(sipg_server* sv) {
  server_free(sv);
  return SIPG_OK;
}

sipg_status sipg_server_submit(sipg_server* sv, const sipg_request* req, unsigned long long* id) {
  if (!sv || !req || !id) return SIPG_ERR_INVALID;
  if (req->dim < 1 || req->degree < 1 || req->degree > SIPG_MAX_DEGREE || !(req->tol > 0) ||
      req->sol < SIPG_SOL_A || req->sol > SIPG_SOL_MODES || (req->precision != SIPG_F64 && req->precision != SIPG_F32)) {
    set_error("sipg_server_submit: invalid request");
    return SIPG_ERR_INVALID;
  }
  Request* r = new (std::nothrow) Request;
  if (!r) return SIPG_ERR_NOMEM;
  r->id = sv->next_id++;
  r->req = *req;
  r->n = (size_t)req->dim * req->dim * (req->degree + 1) * (req->degree + 1);
  r->footprint = footprint_of(req->dim, req->degree, req->precision);
  r->t_submit = Clock::now();
  sv->all[r->id] = r;
  *id = r->id;
  if (r->footprint > sv->opts.budget_bytes) {
    r->result.status = SIPG_ERR_REJECTED;
    r->result.done = 1;
    r->state = 2;
    sv->rejected++;
    set_error("sipg_server_submit: request footprint exceeds the memory budget");
    return SIPG_ERR_REJECTED;
  }
  sv->queue.push_back(r);
  if (r->req.precision != SIPG_F64) {
    {
      std::lock_guard<std::mutex> lock(sv->prep_mu);
      sv->prep_todo.push_back(r);
    }
    sv->prep_cv.notify_one();
  } else {
    r->prepared.store(1, std::memory_order_release);
  }
  return SIPG_OK;
}

sipg_status sipg_server_step(sipg_server* sv, int* n_active, int* n_completed) {
  if (!sv) return SIPG_ERR_INVALID;
  const unsigned long long done_before = sv->completed;
  // 1. admission, FIFO over all lanes
  while (!sv->queue.empty() && !sv->free_slots.empty()) {
    Request* r = sv->queue.front();
    if (sv->used + r->footprint > sv->opts.budget_bytes) break;  // FIFO: wait for memory
    if (!r->prepared.load(std::memory_order_acquire)) break;     // FIFO: its preparation is still running
    const auto t_setup = Clock::now();
    sipg_status st = r->prep_status;
    if (st == SIPG_OK) st = get_op(sv, r->req.dim, r->req.degree, r->req.pen, &r->op);
    if (st != SIPG_OK) {
      // the request retires with the error; the server goes on
      sv->queue.pop_front();
      r->t_admit = r->t_done = Clock::now();
      r->result.status = st;
      r->result.done = 1;
      r->result.latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
      r->state = 2;
      sv->rejected++;
      continue;
    }
    Lane& L = sv->lanes[lane_of(r->n)];
    st = admit(sv, r, L.s);
    sv->setup_ms += std::chrono::duration<double, std::milli>(Clock::now() - t_setup).count();
    sv->queue.pop_front();
    if (st != SIPG_OK) {
      // the request holds nothing (admit rolled back); it retires with the
      // error rather than being admitted again at the next step
      r->t_admit = r->t_done = Clock::now();
      r->result.status = st;
      r->result.done = 1;
      r->result.latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
      r->state = 2;
      sv->rejected++;
      if (st == SIPG_ERR_NOMEM) continue;  // the pool is short now; later requests may still fit
      return st;
    }
    L.fresh.push_back(r);
  }
  // 2. every lane whose round has ended: its results, then its next round;
  // if every lane with work is mid-round, wait for the one of the smallest
  // solves and take it
  for (int pass = 0; pass < 2; ++pass) {
    bool progressed = false;
    for (Lane& L : sv->lanes) {
      if (L.busy) {
        const cudaError_t q = cudaEventQuery(L.ev);
        if (q == cudaErrorNotReady) continue;
        SIPG_CUDA_TRY(q);
        L.busy = false;
        sipg_status st = lane_finish(sv, L);
        if (st != SIPG_OK) return st;
        progressed = true;
      }
      if (!L.fresh.empty()) {
        sipg_status st = lane_start(sv, L);
        if (st != SIPG_OK) return st;
        progressed = true;
      }
      if (!L.active.empty()) {
        sipg_status st = lane_launch(sv, L);
        if (st != SIPG_OK) return st;
      }
    }
    if (progressed) break;
    bool waited = false;
    for (Lane& L : sv->lanes)
      if (L.busy) {
        SIPG_CUDA_TRY(cudaEventSynchronize(L.ev));
        waited = true;
        break;
      }
    if (!waited) break;
  }
  if (n_active) *n_active = active_count(sv);
  if (n_completed) *n_completed = (int)(sv->completed - done_before);
  return SIPG_OK;
}

sipg_status sipg_server_poll(sipg_server* sv, unsigned long long id, sipg_request_result* out) {
  if (!sv || !out) return SIPG_ERR_INVALID;
  auto it = sv->all.find(id);
  if (it == sv->all.end()) {
    set_error("sipg_server_poll: unknown request id");
    return SIPG_ERR_INVALID;
  }
  *out = it->second->result;
  return SIPG_OK;
}

sipg_status sipg_server_release(sipg_server* sv, unsigned long long id) {
  if (!sv) return SIPG_ERR_INVALID;
  auto it = sv->all.find(id);
  if (it == sv->all.end() || it->second->state != 2) {
    set_error("sipg_server_release: unknown or unfinished request");
    return SIPG_ERR_INVALID;
  }
  Request* r = it->second;
  if (r->x64) {
    cudaFreeAsync(r->x64, sv->s);
    sv->used -= r->x_bytes;
  }
  delete r;
  sv->all.erase(it);
  return SIPG_OK;
}

sipg_status sipg_server_solution(sipg_server* sv, unsigned long long id, double* h_x, size_t n) {
  if (!sv || !h_x) return SIPG_ERR_INVALID;
  auto it = sv->all.find(id);
  if (it == sv->all.end() || it->second->state != 2 || !it->second->x64 || n != it->second->n) {
    set_error("sipg_server_solution: unknown, unfinished or released request, or wrong length");
    return SIPG_ERR_INVALID;
  }
  SIPG_CUDA_TRY(cudaMemcpyAsync(h_x, it->second->x64, n * sizeof(double), cudaMemcpyDeviceToHost, sv->s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(sv->s));
  return SIPG_OK;
}

sipg_status sipg_server_stats(const sipg_server* sv, sipg_server_stats_t* out) {
  if (!sv || !out) return SIPG_ERR_INVALID;
  out->queued = (int)sv->queue.size();
  out->active = active_count(sv);
  out->completed = sv->completed;
  out->rejected = sv->rejected;
  out->bytes_in_use = sv->used;
  out->setup_ms = sv->setup_ms;
  out->prep_ms = sv->prep_us.load() / 1e3;
  return SIPG_OK;
}

}  // extern "C"
