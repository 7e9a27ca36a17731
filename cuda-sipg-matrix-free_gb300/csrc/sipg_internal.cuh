// sipg_internal.cuh -- shared definitions of the GB300 SIPG-SEM library:
// per-degree operator tables (passed to kernels by value, so they live in the
// kernel-parameter constant bank and no process-global __constant__ state
// exists), the operator object, CG device state, error plumbing.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>

#include "sipg_gb300.h"

#define SIPG_MAX_P SIPG_MAX_DEGREE
#define SIPG_MAX_N (SIPG_MAX_P + 1)

namespace sipg {

// ---------------------------------------------------------------------------
// Degree-P tables.  w: LGL weights; D0[i] = derivative of basis i at node 0,
// DN[i] = at node P (the face columns of the reference's D table,
// device_const.hpp:216-234); K[a*n+b] = sum_k w_k D[a][k] D[b][k], the 1-D
// stiffness that the reference's volume kernel recomputes per thread
// (volume_gpu_kernels.hpp:46-80).
// ---------------------------------------------------------------------------
template <typename T, int P>
struct Tab {
  static constexpr int N1 = P + 1;
  T w[N1];
  T WH[N1];  // w / 2 (exact): the lifted jump's weight on an interior face
  T D0[N1];
  T DN[N1];
  T K[N1 * N1];
  T KW[N1 * N1 * N1];  // KW[(a * N1 + i) * N1 + b] = w_b K[a][i]: the weighted stiffness of the column form
};

// Host-side double tables for one degree (filled by tables.cpp).
struct HostTables {
  int p;
  double nodes[SIPG_MAX_N];
  double w[SIPG_MAX_N];
  double D[SIPG_MAX_N * SIPG_MAX_N];  // D[mode*n+node]
  double K[SIPG_MAX_N * SIPG_MAX_N];
};
int build_host_tables(int p, HostTables* t);  // 0 on success
// LGL nodes/weights and the derivative matrix for any degree 1..63 (host).
int lgl_compute(int N, double* x, double* w);
int dphi_compute(int N, const double* x, double* D);

template <typename T, int P>
inline Tab<T, P> make_tab(const HostTables& h) {
  Tab<T, P> t;
  const int n = P + 1;
  for (int i = 0; i < n; ++i) {
    t.w[i] = (T)h.w[i];
    t.WH[i] = (T)(0.5 * h.w[i]);
    t.D0[i] = (T)h.D[i * n + 0];
    t.DN[i] = (T)h.D[i * n + P];
  }
  for (int i = 0; i < n * n; ++i) t.K[i] = (T)h.K[i];
  for (int a = 0; a < n; ++a)
    for (int i = 0; i < n; ++i)
      for (int b = 0; b < n; ++b) t.KW[(a * n + i) * n + b] = (T)(h.w[b] * h.K[a * n + i]);
  return t;
}

// ---------------------------------------------------------------------------
// CG state kept on the device (one per solve); scalars of type T.
// ---------------------------------------------------------------------------
template <typename T>
struct CgState {
  T rr;      // r.r of the current residual (the reference's rr_old)
  T pAp;     // p.Ap of the current direction
  T alpha;   // rr / pAp
  T beta;    // rr_new / rr_old
  T stop;    // absolute stop threshold on sqrt(r.r)
  T bb;      // b.b (for relative tolerances)
  T rmax;    // reliable updates: largest sqrt(rr) since the last FP64 correction
  T delta;   // reliable updates: correct when sqrt(rr) < delta * rmax (0: never)
  int it;    // iterations done
  int max_it;
  int done;  // 1 once sqrt(rr) <= stop, it == max_it, breakdown, or an update is due
  int first; // 1 before the first direction p = r is formed
  int status;  // SIPG_OK / SIPG_ERR_BREAKDOWN
  int parity;  // which direction buffer holds the current p
  int need_update;  // reliable updates: an FP64 correction is due
  int pad;
  T rr_prev;  // r.r before the last update (beta after a forced correction)
  T pad2;
  T rres;     // preconditioned CG: r.r of the residual (its stop test; rr holds r.z)
  T pad3;
};

// Deterministic grid reduction scratch: per-block partials, reduced in a fixed
// order by whichever block arrives last.
struct ReduceScratch {
  double* partials = nullptr;  // capacity entries
  unsigned int* counter = nullptr;
  int capacity = 0;
};

// Kernel modes of the fused apply.
enum ApplyMode : int {
  APPLY_PREPARE = -1,  // set kernel attributes only (before a graph capture)
  APPLY_PLAIN = 0,  // y = A u
  APPLY_CG = 1,     // u = r + beta p_old (u = r on the first iteration); p_new = u; y = A u; pAp -> alpha;
                    // the parity of the direction buffers flips
  APPLY_RESID = 2,  // y = b - A u; r.r -> rr, stop/done set
  APPLY_DOT = 3,    // y = A p for a direction p formed beforehand (k_cg_direction*); p.Ap -> alpha
  // FP64: APPLY_RESID / APPLY_DOT with every zero-sum contraction taken over
  // differences from one value of its element line (the FP32 apply always
  // does this): the residual checks and outer steps of the mixed solvers,
  // where a smooth iterate's rounding in the plain sums would put a floor
  // near 1e-10 under the true relative residual at 1024^2, p = 4.  The FP64
  // CG and the plain apply keep the plain sums.  (The per-node FP64 tile of
  // small meshes runs the plain modes for these.)
  APPLY_RESID_PIVOT = 4,
  APPLY_DOT_PIVOT = 5
};
// The plain mode a pivoted one computes.
__host__ __device__ constexpr int apply_base_mode(int mode) {
  return mode == APPLY_RESID_PIVOT ? APPLY_RESID : (mode == APPLY_DOT_PIVOT ? APPLY_DOT : mode);
}

template <typename T>
struct ApplyArgs {
  const T* in;     // u (PLAIN, RESID) or r (CG)
  T* pbuf0;        // CG: the two direction buffers; CgState::parity says which
  T* pbuf1;        //     holds the previous direction, the other gets the new one
  T* out;          // y
  const T* b;      // RESID: right-hand side
  int dim;
  T nu;            // penalty (the reference's `pen`)
  T nu_lo, nu_lo2;  // compensated apply: pen as three floats nu + nu_lo + nu_lo2
  CgState<T>* st;  // CG / RESID
  ReduceScratch red;
  CgState<double>* stp;  // compensated apply, CG mode: the inner state (FP64 scalars)
  // a band of element rows [row0, row0 + nrows) (nrows = 0: the whole mesh),
  // row0 a multiple of the tile's rows; the FP64 applies (element and
  // per-node tiles) honour it
  int row0, nrows;
};

// The penalty of a compensated apply as three floats (nu + nu_lo + nu_lo2).
inline void set_penalty3(ApplyArgs<float>& a, double pen) {
  a.nu = (float)pen;
  const double r1 = pen - (double)a.nu;
  a.nu_lo = (float)r1;
  a.nu_lo2 = (float)(r1 - (double)a.nu_lo);
}

// Tile shape chosen for one (precision, degree).
struct TileCfg {
  int tx = 32, ty = 4;
  int tpe = 1;  // threads per element: 1, 2 (the compensated apply), or (p+1)^2
                // (the per-node FP64 tile for small meshes)
};

// The per-node FP64 tile (one thread per output node): tx x ty elements per
// CTA, shape 0 the smallest, shape 1 twice as wide.
__host__ __device__ constexpr int pernode_ey(int p) { return p == 1 ? 4 : 2; }
__host__ __device__ constexpr int pernode_ex(int p, int shape) { return (p <= 2 ? 4 : 2) * (shape ? 2 : 1); }
// FP64 operators up to kPernodeDefaultDim elements per edge start with the
// per-node tile (measured faster than 32-element rows up to there), shape 1
// above kPernodeWideDim
constexpr int kPernodeDefaultDim = 128;
constexpr int kPernodeWideDim = 32;
inline bool is_pernode(const TileCfg& c, int p) { return c.tpe == (p + 1) * (p + 1); }
inline TileCfg pernode_tile(int p, int shape) {
  TileCfg c;
  c.tx = pernode_ex(p, shape);
  c.ty = pernode_ey(p);
  c.tpe = (p + 1) * (p + 1);
  return c;
}

// Launch the fused apply for degree p (dispatches on p and the tile shape).
// Returns cudaGetLastError() of the launch.
cudaError_t launch_apply_f64(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>& a, const HostTables& h,
                             cudaStream_t s);
cudaError_t launch_apply_f32(int p, const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const HostTables& h,
                             cudaStream_t s);
// The same for many operators of degree p in one launch (instances' tiles
// concatenated, tile_start[i] = first tile of instance i; device arrays).
cudaError_t launch_apply_batched_f64(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>* insts,
                                     const int* tile_start, int ninst, int total_tiles, const HostTables& h,
                                     cudaStream_t s);
cudaError_t launch_apply_batched_f32(int p, const TileCfg& cfg, int mode, const ApplyArgs<float>* insts,
                                     const int* tile_start, int ninst, int total_tiles, const HostTables& h,
                                     cudaStream_t s);
// The compensated FP32 apply on double-float vectors (2 n floats: the hi
// plane, then the lo plane): one operator (insts == nullptr) or a batch of
// degree-p operators; modes APPLY_PREPARE / PLAIN / CG.
cudaError_t launch_apply_df(int p, const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const ApplyArgs<float>* insts,
                            const int* tile_start, int ninst, int total_tiles, const HostTables& h, cudaStream_t s);
// The persistent CG of small FP64 meshes (cg_small.cu): operands, and its
// launch for an operator whose FP64 tile is a per-node one.  At most
// kSmallCgMaxBlocks CTAs (two partial slots each in the reduction scratch).
struct SmallCgArgs {
  double* x;
  double* r;
  double* p0;
  double* p1;
  double* Ap;
  CgState<double>* st;  // read at the start (after the residual kernel), written back at the end
  double* part_a;       // [gridDim.x] p.Ap partials
  double* part_b;       // [gridDim.x] r.r partials
  unsigned long long* bar;  // barrier arrivals (zero at launch)
  int* abort;           // raised when a barrier wait gives up (zero at launch)
  int dim;
  double nu;
};
constexpr int kSmallCgMaxBlocks = 152 * 8;
constexpr int kSmallCgDim = 32;  // meshes up to this many elements per edge use it
cudaError_t launch_cg_small(int p, const TileCfg& cfg, const SmallCgArgs& g, const HostTables& h, cudaStream_t s);

// Tile shapes the autotuner chose for (degree, dim, precision) in this
// process; false if none (autotune.cu).
bool autotune_lookup(int p, int dim, int prec, TileCfg* cfg);
// Number of blocks the apply launches for this tile shape.
// The tile a batched launch uses: batched kernels compile 32-element rows
// only, so an operator tuned to the per-node FP64 tile joins a batch with the
// 32 x 4 tile.
inline TileCfg batched_tile(TileCfg c) {
  if (c.tx != 32) c = TileCfg{};
  return c;
}
inline int apply_grid_blocks(int dim, const TileCfg& c) {
  return ((dim + c.tx - 1) / c.tx) * ((dim + c.ty - 1) / c.ty);
}
// Reduction-scratch entries that cover every element-per-thread tile shape
// (the one with the fewest elements is 32 x 2), every vector kernel grid (at
// most 152 * 8) and 16 resident per-node CTAs per SM (the per-node apply caps
// its grid at the scratch).
inline int reduce_capacity(int dim) {
  const int a = ((dim + 31) / 32) * ((dim + 1) / 2);
  return a > 152 * 16 ? a : 152 * 16;
}


// ---------------------------------------------------------------------------
// Error plumbing and launch accounting.
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
extern std::atomic<unsigned long long> g_launches;
inline void count_launch(unsigned long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

#define SIPG_CUDA_TRY(call)                                                                      \
  do {                                                                                           \
    cudaError_t _e = (call);                                                                     \
    if (_e != cudaSuccess) {                                                                     \
      ::sipg::set_error(std::string(#call) + " failed: " + cudaGetErrorString(_e));              \
      return (_e == cudaErrorMemoryAllocation) ? SIPG_ERR_NOMEM : SIPG_ERR_CUDA;                 \
    }                                                                                            \
  } while (0)

}  // namespace sipg

// ---------------------------------------------------------------------------
// The operator object behind the opaque sipg_op handle.
// ---------------------------------------------------------------------------
struct sipg_cg_workspace;


struct sipg_op {
  int dim = 0, p = 0;
  double pen = 0;
  int device = 0;
  long long noe = 0, ndof = 0;
  sipg::HostTables tab;
  sipg::TileCfg cfg64, cfg32, cfgdf;  // FP64, FP32 and compensated-FP32 apply tiles
  int tile_gen = 0;                    // bumped when a tile shape changes (graphs re-capture)
  std::mutex mu;  // guards the lazily allocated workspaces below
  sipg_cg_workspace* ws64 = nullptr;
  sipg_cg_workspace* ws32 = nullptr;
  double* stage_in = nullptr;  // host-buffer apply staging (device)
  double* stage_out = nullptr;
  // the host-buffer apply's pipeline: copy-in, copy-out and two compute
  // streams, and per band events
  cudaStream_t hs[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t hev[2 * 16 + 2] = {};
  void* mixed = nullptr;  // the mixed-precision solver's cached workspace
  void (*mixed_free)(void*) = nullptr;
  void* pcg = nullptr;  // the block-Jacobi preconditioner and PCG workspace
  void (*pcg_free)(void*) = nullptr;
  void* tl = nullptr;  // the two-level preconditioner of the mixed solve (twolevel.cu)
  void (*tl_free)(void*) = nullptr;
};

namespace sipg {
// The operator's two-level preconditioner (block-Jacobi + vertex-grid
// multigrid, twolevel.cu), built on first use: synchronous, not during stream
// capture.
sipg_status twolevel_get(sipg_op* op, void** handle);
// Enqueues z = M r on s in FP32; with st (an inner PCG state) every kernel is
// skipped once st->done and the last one sets st->rr = r.z and beta.  With
// cp_ready the restriction of r is already in place (twolevel_enqueue_restrict,
// or the update below) and is not enqueued again.
sipg_status twolevel_enqueue(const sipg_op* op, const void* handle, const float* r, float* z, CgState<float>* st,
                             const ReduceScratch& red, cudaStream_t s, bool cp_ready);
sipg_status twolevel_enqueue_restrict(const sipg_op* op, const void* handle, const float* r, cudaStream_t s);
// The inner PCG update x += alpha p, r -= alpha Ap (p by the state's parity
// from pb0 / pb1; the same pointer twice for a direction kept in place), r.r
// and the stop test, fused with the restriction of the new r.
sipg_status twolevel_enqueue_update(const sipg_op* op, const void* handle, float* x, const float* pb0,
                                    const float* pb1, float* r, const float* Ap, CgState<float>* st,
                                    const ReduceScratch& red, cudaStream_t s);
}  // namespace sipg
