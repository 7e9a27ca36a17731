// sipg_fcg.cuh -- device steps of the flexible mixed-precision solve (no
// counterpart in the reference): flexible CG in FP64 (Notay, SIAM J. Sci.
// Comput. 22, 2000, truncated to one previous direction) whose
// preconditioner is an FP32 CG run from zero on the scaled residual.
//
// One outer step, for each instance:
//   restart   r32 = r64 / ||r64||, e = 0, fresh FP32 CG state        (16 B/DoF)
//   (inner)   FP32 CG iterations on A e = r32 until its residual fell by
//             the inner tolerance                                    (40 B/DoF each)
//   gamma     z = ||r64|| e;  gamma = z.q_prev / d_prev.q_prev        (12 B/DoF)
//   direction d = z - gamma d_prev (first: d = z);  d.r              (28 B/DoF)
//   FP64 apply q = A d; alpha = d.r / d.q (APPLY_DOT)                (16 B/DoF)
//   update    x += alpha d, r64 -= alpha q, r.r (cg_update_body)     (48 B/DoF)
// The FP64 CgState of an instance carries r.r after the update and d.r
// before the apply (APPLY_DOT's alpha = rr / pAp); pAp = d.q stays there for
// the next step's gamma.  Each body works on the grid-stride slice of block
// `bid` of `nblocks` and reduces deterministically (grid_sum_last), so the
// single-solve kernels (bid = blockIdx.x) and the batched ones (one instance
// per blockIdx.y, nblk blocks each) give the same iterates.
#pragma once

#include "sipg_cg.cuh"

namespace sipg {

// Scalars of the flexible outer loop beside its FP64 CgState.
struct FcgState {
  double zscale;  // ||r64|| at the inner restart: z = zscale * e
  double gamma;   // z.q_prev / d_prev.q_prev
};

__device__ __forceinline__ void fcg_restart_body(const double* __restrict__ r64, float* __restrict__ r,
                                                 float* __restrict__ e, size_t n, const CgState<double>* st64,
                                                 FcgState* fs, CgState<float>* st, const ReduceScratch& red,
                                                 float stop, int max_it, int bid, int nblocks) {
  __shared__ float sh[32];
  const double rr = st64->rr;
  const double inv = rr > 0.0 ? 1.0 / sqrt(rr) : 1.0;
  float acc = 0.f;
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float h = (float)(r64[i] * inv);
    r[i] = h;
    e[i] = 0.f;
    acc = fmaf(h, h, acc);
  }
  const float bt = block_sum<float, kVecThreads>(acc, sh);
  float total;
  if (grid_sum_last<float, kVecThreads>(bt, red, bid, nblocks, sh, &total) && threadIdx.x == 0) {
    st->first = 1;
    st->it = 0;
    st->parity = 0;
    st->beta = 0.f;
    st->status = (int)SIPG_OK;
    st->rr = total;
    st->rres = total;  // the preconditioned inner solve's stop test reads r.r here
    st->rmax = sqrtf(total);
    st->delta = 0.f;  // no reliable updates inside a preconditioner solve
    st->stop = stop;
    st->max_it = max_it;
    st->need_update = 0;
    st->done = (total == 0.f) ? 1 : 0;
    fs->zscale = rr > 0.0 ? sqrt(rr) : 1.0;
  }
}

__device__ __forceinline__ void fcg_gamma_body(const float* __restrict__ e, const double* __restrict__ q, size_t n,
                                               const CgState<double>* st64, FcgState* fs, const ReduceScratch& red,
                                               int bid, int nblocks) {
  __shared__ double sh[32];
  const double zs = fs->zscale;
  double acc = 0.0;
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride)
    acc = fma((double)e[i] * zs, q[i], acc);
  const double bt = block_sum<double, kVecThreads>(acc, sh);
  double total;
  if (grid_sum_last<double, kVecThreads>(bt, red, bid, nblocks, sh, &total) && threadIdx.x == 0)
    fs->gamma = total / st64->pAp;
}

__device__ __forceinline__ void fcg_direction_body(const float* __restrict__ e, double* __restrict__ d,
                                                   const double* __restrict__ r, size_t n, CgState<double>* st64,
                                                   const FcgState* fs, const ReduceScratch& red, int first, int bid,
                                                   int nblocks) {
  __shared__ double sh[32];
  const double zs = fs->zscale;
  const double g = first ? 0.0 : fs->gamma;
  double acc = 0.0;
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double z = (double)e[i] * zs;
    const double di = first ? z : fma(-g, d[i], z);
    d[i] = di;
    acc = fma(di, r[i], acc);
  }
  const double bt = block_sum<double, kVecThreads>(acc, sh);
  double total;
  if (grid_sum_last<double, kVecThreads>(bt, red, bid, nblocks, sh, &total) && threadIdx.x == 0) {
    st64->rr_prev = st64->rr;  // r.r, kept for the host's progress check
    st64->rr = total;
    st64->parity = 0;
    st64->done = 0;
    if (!isfinite(total)) {
      st64->status = (int)SIPG_ERR_BREAKDOWN;
      st64->done = 1;
    }
  }
}

// The update of a preconditioned inner CG (rr holds r.z, set by the
// preconditioner's last kernel): x += alpha p, r -= alpha Ap, rres = r.r,
// it++, and the stop test on sqrt(rres).
template <typename T>
__device__ __forceinline__ void pcg_update_body(T* __restrict__ x, const T* __restrict__ p, T* __restrict__ r,
                                                const T* __restrict__ Ap, size_t n, CgState<T>* st,
                                                const ReduceScratch& red, int bid, int nblocks) {
  __shared__ T sh[32];
  if (*(volatile int*)&st->done) return;
  const T alpha = st->alpha;
  T acc = T(0);
  const size_t stride = (size_t)nblocks * blockDim.x;
  size_t head = 0;  // FP32 with 16-byte aligned vectors: four per thread and step
  if constexpr (sizeof(T) == 4) {
    if (aligned16(x, p, r, Ap)) {
      head = n & ~size_t(3);
      float4* __restrict__ x4 = reinterpret_cast<float4*>(x);
      float4* __restrict__ r4 = reinterpret_cast<float4*>(r);
      const float4* __restrict__ p4 = reinterpret_cast<const float4*>(p);
      const float4* __restrict__ a4 = reinterpret_cast<const float4*>(Ap);
      for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < head / 4; i += stride) {
        const float4 pv = p4[i], av = a4[i];
        float4 xv = x4[i], rv = r4[i];
        xv.x = fmaf(alpha, pv.x, xv.x);
        xv.y = fmaf(alpha, pv.y, xv.y);
        xv.z = fmaf(alpha, pv.z, xv.z);
        xv.w = fmaf(alpha, pv.w, xv.w);
        rv.x = fmaf(-alpha, av.x, rv.x);
        rv.y = fmaf(-alpha, av.y, rv.y);
        rv.z = fmaf(-alpha, av.z, rv.z);
        rv.w = fmaf(-alpha, av.w, rv.w);
        x4[i] = xv;
        r4[i] = rv;
        acc = fmaf(rv.x, rv.x, acc);
        acc = fmaf(rv.y, rv.y, acc);
        acc = fmaf(rv.z, rv.z, acc);
        acc = fmaf(rv.w, rv.w, acc);
      }
    }
  }
  for (size_t i = head + (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] = fma(alpha, p[i], x[i]);
    const T ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    acc = fma(ri, ri, acc);
  }
  const T bt = block_sum<T, kVecThreads>(acc, sh);
  T total;
  if (grid_sum_last<T, kVecThreads>(bt, red, bid, nblocks, sh, &total) && threadIdx.x == 0)
    pcg_update_bookkeep<T>(st, total);
}

// The FP64 product q = A d of a flexible step is taken with pivoted sums
// (APPLY_DOT_PIVOT) while the step starts from a relative residual above
// this, plain sums (APPLY_DOT) below it.  Plain sums round at the scale of
// |d|, pivoted ones at the scale of its differences: at the first steps d is
// as large as the solution and plain rounding would leave a floor near 1e-10
// in the recursively updated residual; once the residual is below 1e-2, |d|
// is about that fraction of the solution and the plain rounding is that much
// smaller.  The closing check b - A x always uses pivoted sums.
constexpr double kFcgPivotRel = 1e-2;

// ---- one solve ----

static __global__ void __launch_bounds__(kVecThreads)
    k_fcg_restart(const double* __restrict__ r64, float* __restrict__ r, float* __restrict__ e, size_t n,
                  const CgState<double>* st64, FcgState* fs, CgState<float>* st, ReduceScratch red, float stop,
                  int max_it) {
  fcg_restart_body(r64, r, e, n, st64, fs, st, red, stop, max_it, blockIdx.x, gridDim.x);
}

static __global__ void __launch_bounds__(kVecThreads)
    k_pcg_update_f32(float* __restrict__ x, const float* __restrict__ p, float* __restrict__ r,
                     const float* __restrict__ Ap, size_t n, CgState<float>* st, ReduceScratch red) {
  pcg_update_body<float>(x, p, r, Ap, n, st, red, blockIdx.x, gridDim.x);
}

static __global__ void __launch_bounds__(kVecThreads)
    k_fcg_gamma(const float* __restrict__ e, const double* __restrict__ q, size_t n, const CgState<double>* st64,
                FcgState* fs, ReduceScratch red) {
  fcg_gamma_body(e, q, n, st64, fs, red, blockIdx.x, gridDim.x);
}

static __global__ void __launch_bounds__(kVecThreads)
    k_fcg_direction(const float* __restrict__ e, double* __restrict__ d, const double* __restrict__ r, size_t n,
                    CgState<double>* st64, const FcgState* fs, ReduceScratch red, int first) {
  fcg_direction_body(e, d, r, n, st64, fs, red, first, blockIdx.x, gridDim.x);
}

// ---- many instances (instance = blockIdx.y, nblk blocks each) ----

// One instance's operands of the flexible solve.
struct FcgInst {
  double* x;        // FP64 solution
  const double* b;  // FP64 right-hand side
  double* r64;      // FP64 residual
  double* d64;      // FP64 direction
  double* q64;      // A d
  float* r32;       // FP32 inner residual
  float* e32;       // FP32 inner solution
  float* p32;       // FP32 inner direction
  float* Ap32;      // FP32 inner A p
  float* z32;       // FP32 preconditioned residual (two-level inner kind)
  CgState<float>* st32;
  CgState<double>* st64;
  FcgState* fs;
  ReduceScratch red32, red64;
  size_t n;
  int nblk;
  int first;  // flexible step: the first direction of a (re)start
  float stop;  // inner tolerance (the inner residual starts at norm 1)
  int max_it;  // inner iterations per preconditioner solve
};

static __global__ void __launch_bounds__(kVecThreads) k_fcg_restart_batched(const FcgInst* __restrict__ insts) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  fcg_restart_body(v.r64, v.r32, v.e32, v.n, v.st64, v.fs, v.st32, v.red32, v.stop, v.max_it, blockIdx.x, v.nblk);
}

static __global__ void __launch_bounds__(kVecThreads) k_fcg_gamma_batched(const FcgInst* __restrict__ insts) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk || v.first) return;
  fcg_gamma_body(v.e32, v.q64, v.n, v.st64, v.fs, v.red64, blockIdx.x, v.nblk);
}

static __global__ void __launch_bounds__(kVecThreads) k_fcg_direction_batched(const FcgInst* __restrict__ insts) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  fcg_direction_body(v.e32, v.d64, v.r64, v.n, v.st64, v.fs, v.red64, v.first, blockIdx.x, v.nblk);
}

static __global__ void __launch_bounds__(kVecThreads) k_fcg_update_batched(const FcgInst* __restrict__ insts) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  cg_update_body<double>(v.x, v.d64, v.d64, v.r64, v.q64, v.n, v.st64, v.red64, blockIdx.x, v.nblk);
}

// The inner FP32 CG of many instances: p = r (first) or p = r + beta p, and
// the update e += alpha p, r -= alpha Ap with r.r and the stop test;
// instances whose inner solve is done skip both.
static __global__ void __launch_bounds__(kVecThreads) k_fcg_inner_direction_batched(const FcgInst* __restrict__ insts) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  const CgState<float>* st = v.st32;
  if (*(volatile const int*)&st->done) return;
  const bool first = st->first != 0;
  const float beta = st->beta;
  const size_t stride = (size_t)v.nblk * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < v.n; i += stride)
    v.p32[i] = first ? v.r32[i] : fmaf(beta, v.p32[i], v.r32[i]);
}

static __global__ void __launch_bounds__(kVecThreads) k_fcg_inner_update_batched(const FcgInst* __restrict__ insts) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  cg_update_body<float>(v.e32, v.p32, v.p32, v.r32, v.Ap32, v.n, v.st32, v.red32, blockIdx.x, v.nblk);
}

// The same for the two-level-preconditioned inner CG: p = z + beta p (first:
// p = z; z, r.z and beta come from the preconditioner), and the update with
// the stop test on r.r (pcg_update_body).
static __global__ void __launch_bounds__(kVecThreads)
    k_fcg_inner_pdirection_batched(const FcgInst* __restrict__ insts) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  const CgState<float>* st = v.st32;
  if (*(volatile const int*)&st->done) return;
  cg_direction_body<float>(v.p32, v.z32, v.n, st->first != 0, st->beta, blockIdx.x, v.nblk);
}

static __global__ void __launch_bounds__(kVecThreads) k_fcg_inner_pupdate_batched(const FcgInst* __restrict__ insts) {
  const FcgInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  pcg_update_body<float>(v.e32, v.p32, v.r32, v.Ap32, v.n, v.st32, v.red32, blockIdx.x, v.nblk);
}

}  // namespace sipg
