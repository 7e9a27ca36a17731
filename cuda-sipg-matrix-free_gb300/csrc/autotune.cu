// autotune.cu -- picks the apply tile shape per operator by timing (no
// counterpart in the reference, whose kernels use one fixed geometry).
//
// A tile is TX = 32 elements along a mesh row (a warp's loads of one node are
// 32 consecutive values) by TY rows, with one or two threads per element; a
// CTA holds TX * TY elements and their (p+1)^2 nodal blocks in shared memory.
// For FP64 on small meshes there is also the per-node tile (a few elements
// per CTA, one thread per output node), which spreads the thin FP64 pipe's
// work over many more warps and SMs.
// TY trades halo overhead (TX + TY halo elements per tile) and reduction
// partials against shared memory per CTA and so resident CTAs per SM; a
// second thread per element doubles the resident warps at the same shared
// memory, which pays where the apply waits on latency (the compensated one)
// rather than on a pipe (FP64).  The best choice depends on the degree, the
// mesh size (how many waves of CTAs fill the 152 SMs) and the arithmetic.  The
// tuner times each candidate on the operator itself -- a few applies on
// scratch vectors -- keeps the fastest, and remembers it for (degree, dim,
// kind) in a process-wide table that new operators consult at creation.  Every tile
// shape computes each output from the same operations in the same order, so
// the apply's result does not depend on the choice (CG reductions sum
// per-block partials, whose grouping does change with TY).
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "sipg_internal.cuh"

using namespace sipg;

namespace sipg {

namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, TileCfg> g_tuned;  // (p, dim, kind) -> shape

// (elements per row, rows, threads per element): two threads per element only
// for the compensated apply (the one limited by latency rather than a pipe);
// the FP64 apply also tries the two per-node tiles (threads per element
// (p+1)^2)
constexpr int kCandidates[5][3] = {{32, 2, 1}, {32, 4, 1}, {32, 8, 1}, {32, 2, 2}, {32, 4, 2}};

template <typename T>
cudaError_t run_apply(const sipg_op* op, int prec, const TileCfg& cfg, const void* in, void* out, cudaStream_t s) {
  ApplyArgs<T> a{};
  a.in = (const T*)in;
  a.out = (T*)out;
  a.dim = op->dim;
  a.nu = (T)op->pen;
  if constexpr (sizeof(T) == 8) {
    return launch_apply_f64(op->p, cfg, APPLY_PLAIN, a, op->tab, s);
  } else {
    set_penalty3(a, op->pen);
    if (prec == SIPG_TUNE_PAIRS) return launch_apply_df(op->p, cfg, APPLY_PLAIN, a, nullptr, nullptr, 0, 0, op->tab, s);
    return launch_apply_f32(op->p, cfg, APPLY_PLAIN, a, op->tab, s);
  }
}

// average ms per apply of one candidate, or a negative value if it cannot run
template <typename T>
float time_candidate(const sipg_op* op, int prec, int tx, int ty, int tpe, const void* in, void* out, cudaStream_t s,
                     cudaEvent_t e0, cudaEvent_t e1, int reps) {
  TileCfg cfg;
  cfg.tx = tx;
  cfg.ty = ty;
  cfg.tpe = tpe;
  if (run_apply<T>(op, prec, cfg, in, out, s) != cudaSuccess) {
    cudaGetLastError();  // a launch-configuration error (shared memory); clear it
    return -1.f;
  }
  if (run_apply<T>(op, prec, cfg, in, out, s) != cudaSuccess) return -1.f;
  cudaEventRecord(e0, s);
  for (int k = 0; k < reps; ++k)
    if (run_apply<T>(op, prec, cfg, in, out, s) != cudaSuccess) return -1.f;
  cudaEventRecord(e1, s);
  if (cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  return ms / reps;
}

template <typename T>
TileCfg tune_one(const sipg_op* op, int prec, const void* in, void* out, cudaStream_t s, cudaEvent_t e0,
                 cudaEvent_t e1, float* best_ms) {
  const int reps = (int)std::max<long long>(3, std::min<long long>(50, (long long)(2.0e7 / (double)op->ndof)));
  TileCfg best;
  best.ty = 0;
  float bms = 0.f;
  std::vector<TileCfg> cands;
  for (const auto& c : kCandidates) {
    if (c[2] != 1 && prec != SIPG_TUNE_PAIRS) continue;
    TileCfg t;
    t.tx = c[0];
    t.ty = c[1];
    t.tpe = c[2];
    cands.push_back(t);
  }
  if (prec == SIPG_TUNE_F64) {
    cands.push_back(pernode_tile(op->p, 0));
    cands.push_back(pernode_tile(op->p, 1));
  }
  for (const TileCfg& c : cands) {
    const float ms = time_candidate<T>(op, prec, c.tx, c.ty, c.tpe, in, out, s, e0, e1, reps);
    if (ms > 0.f && (best.ty == 0 || ms < bms)) {
      best = c;
      bms = ms;
    }
  }
  if (best_ms) *best_ms = bms;
  return best;
}
}  // namespace

bool autotune_lookup(int p, int dim, int prec, TileCfg* cfg) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find(std::make_tuple(p, dim, prec));
  if (it == g_tuned.end()) return false;
  *cfg = it->second;
  return true;
}

}  // namespace sipg

extern "C" {

sipg_status sipg_op_autotune(sipg_op* op, void* stream, sipg_tile_choice* out) {
  if (!op) {
    set_error("sipg_op_autotune: null op");
    return SIPG_ERR_INVALID;
  }
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  cudaStream_t s = (cudaStream_t)stream;
  void* in = nullptr;
  void* outv = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const size_t bytes = (size_t)op->ndof * sizeof(double);
  sipg_status st = SIPG_OK;
  TileCfg ty[3];
  for (TileCfg& c : ty) c.ty = 0;
  float ms[3] = {0.f, 0.f, 0.f};
  cudaError_t e = cudaMalloc(&in, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&outv, bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(in, 0, bytes, s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    ty[SIPG_TUNE_F64] = tune_one<double>(op, SIPG_TUNE_F64, in, outv, s, e0, e1, &ms[SIPG_TUNE_F64]);
    ty[SIPG_TUNE_F32] = tune_one<float>(op, SIPG_TUNE_F32, in, outv, s, e0, e1, &ms[SIPG_TUNE_F32]);
    ty[SIPG_TUNE_PAIRS] = tune_one<float>(op, SIPG_TUNE_PAIRS, in, outv, s, e0, e1, &ms[SIPG_TUNE_PAIRS]);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    set_error(std::string("sipg_op_autotune: ") + cudaGetErrorString(e));
    st = e == cudaErrorMemoryAllocation ? SIPG_ERR_NOMEM : SIPG_ERR_CUDA;
  } else if (!ty[0].ty || !ty[1].ty || !ty[2].ty) {
    set_error("sipg_op_autotune: no tile shape could be launched");
    st = SIPG_ERR_CUDA;
  }
  cudaFree(in);
  cudaFree(outv);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st != SIPG_OK) return st;
  {
    std::lock_guard<std::mutex> lk(op->mu);
    op->cfg64 = ty[SIPG_TUNE_F64];
    op->cfg32 = ty[SIPG_TUNE_F32];
    op->cfgdf = ty[SIPG_TUNE_PAIRS];
    op->tile_gen++;
  }
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (int k = 0; k < 3; ++k) g_tuned[std::make_tuple(op->p, op->dim, k)] = ty[k];
  }
  if (out) {
    for (int k = 0; k < 3; ++k) {
      out->elements_per_row[k] = ty[k].tx;
      out->rows[k] = ty[k].ty;
      out->threads_per_element[k] = ty[k].tpe;
      out->ms_per_apply[k] = ms[k];
    }
  }
  return SIPG_OK;
}

sipg_status sipg_op_set_tile(sipg_op* op, int kind, int elements_per_row, int rows, int threads_per_element) {
  if (!op || kind < 0 || kind > 2) {
    set_error("sipg_op_set_tile: null op or kind not 0..2");
    return SIPG_ERR_INVALID;
  }
  const int p = op->p;
  const bool pernode = kind == SIPG_TUNE_F64 && threads_per_element == (p + 1) * (p + 1);
  bool ok;
  if (pernode) {
    ok = rows == pernode_ey(p) && (elements_per_row == pernode_ex(p, 0) || elements_per_row == pernode_ex(p, 1));
  } else {
    const bool tpe_ok =
        threads_per_element == 1 || (threads_per_element == 2 && kind == SIPG_TUNE_PAIRS && rows != 8);
    ok = elements_per_row == 32 && (rows == 2 || rows == 4 || rows == 8) && tpe_ok;
  }
  if (!ok) {
    set_error("sipg_op_set_tile: a tile is 32 elements per row by 2, 4 or 8 rows with 1 thread per element (2 for "
              "the pairs apply with 2 or 4 rows), or, for FP64, the per-node tile: "
              "(p+1)^2 threads per element, " +
              std::to_string(pernode_ex(p, 0)) + " or " + std::to_string(pernode_ex(p, 1)) + " elements per row, " +
              std::to_string(pernode_ey(p)) + " rows");
    return SIPG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(op->mu);
  TileCfg& c = kind == SIPG_TUNE_F64 ? op->cfg64 : (kind == SIPG_TUNE_F32 ? op->cfg32 : op->cfgdf);
  c.tx = elements_per_row;
  c.ty = rows;
  c.tpe = threads_per_element;
  op->tile_gen++;
  return SIPG_OK;
}

sipg_status sipg_op_get_tile(const sipg_op* op, int kind, int* elements_per_row, int* rows,
                             int* threads_per_element) {
  if (!op || !rows || kind < 0 || kind > 2) {
    set_error("sipg_op_get_tile: bad argument");
    return SIPG_ERR_INVALID;
  }
  const TileCfg& c = kind == SIPG_TUNE_F64 ? op->cfg64 : (kind == SIPG_TUNE_F32 ? op->cfg32 : op->cfgdf);
  *rows = c.ty;
  if (elements_per_row) *elements_per_row = c.tx;
  if (threads_per_element) *threads_per_element = c.tpe;
  return SIPG_OK;
}

}  // extern "C"
