// sipg_cg_df.cuh -- the vector kernels of the mixed-precision solvers' inner
// CG: FP32 vectors with FP32 scalars (kind INNER_F32) or double-float pair
// vectors (2 n floats, hi plane then lo plane) with FP64 scalars (kind
// INNER_PAIRS); the FP64 hand-over at a reliable update; and the folding of
// the accumulated correction into the FP64 solution.
//
// The inner CG iterates on a correction e ~ A^-1 r64 of the FP64 solution:
// e += alpha p, r -= alpha Ap (sipg_cg.cuh bookkeeping).  At a reliable update
// the host folds x64 += e, recomputes r64 = b - A x64 in FP64, and restarts the
// inner residual from r64 with the search direction kept (beta = r_new.r_new
// / r_prev.r_prev).
#pragma once

#include "sipg_cg.cuh"
#include "sipg_df.cuh"

namespace sipg {

enum InnerKind : int { INNER_F32 = 1, INNER_PAIRS = 2 };

template <int KIND>
struct InnerScalar {
  using type = float;
};
template <>
struct InnerScalar<INNER_PAIRS> {
  using type = double;
};

// Per-instance operands of the batched pair update (instance = blockIdx.y);
// pointers are pair vectors, n the values per vector.
struct PairInst {
  float* x;
  float* pb0;
  float* pb1;
  float* r;
  float* Ap;
  size_t n;
  CgState<double>* st;
  ReduceScratch red;
  int nblk;
  int pad;
};

// e += alpha p, r -= alpha Ap on pair vectors (alpha FP64, applied as a
// double-float coefficient); r.r from double-float products.
__device__ __forceinline__ void cg_update_pairs_body(float* __restrict__ x, const float* __restrict__ pb0,
                                                     const float* __restrict__ pb1, float* __restrict__ r,
                                                     const float* __restrict__ Ap, size_t n, CgState<double>* st,
                                                     const ReduceScratch& red, int bid, int nblocks) {
  __shared__ double sh[32];
  if (*(volatile int*)&st->done) return;
  const double alpha = st->alpha;
  const float ah = (float)alpha, al = (float)(alpha - (double)ah);
  const float* __restrict__ p = st->parity ? pb1 : pb0;
  df acc = df_zero();
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) {
    df xi{x[i], x[n + i]};
    xi = df_mac2(xi, ah, al, df{p[i], p[n + i]});
    const float s = __fadd_rn(xi.hi, xi.lo);
    x[i] = s;
    x[n + i] = __fsub_rn(xi.lo, __fsub_rn(s, xi.hi));
    df ri{r[i], r[n + i]};
    ri = df_mac2(ri, -ah, -al, df{Ap[i], Ap[n + i]});
    const float rs = __fadd_rn(ri.hi, ri.lo);
    const float rl = __fsub_rn(ri.lo, __fsub_rn(rs, ri.hi));
    r[i] = rs;
    r[n + i] = rl;
    acc = df_mac2(acc, rs, rl, df{rs, rl});
  }
  const double bt = block_sum<double, kVecThreads>((double)acc.hi + (double)acc.lo, sh);
  double total;
  if (grid_sum_last<double, kVecThreads>(bt, red, bid, nblocks, sh, &total) && threadIdx.x == 0)
    cg_bookkeep<double>(st, total);
}

// p = r (first iteration after a start) or p = r + beta p, in place, on pair
// vectors (beta FP64 as a double-float coefficient).  Runs before the
// APPLY_DOT apply of the same iteration.
__device__ __forceinline__ void cg_direction_pairs_body(float* __restrict__ p, const float* __restrict__ r, size_t n,
                                                        const CgState<double>* st, int bid, int nblocks) {
  if (*(volatile const int*)&st->done) return;
  const bool first = st->first != 0;
  const double beta = st->beta;
  const float bh = (float)beta, bl = (float)(beta - (double)bh);
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) {
    const df ri{r[i], r[n + i]};
    df v = ri;
    if (!first) {
      v = df_mac2(ri, bh, bl, df{p[i], p[n + i]});
      const float s = __fadd_rn(v.hi, v.lo);
      v = df{s, __fsub_rn(v.lo, __fsub_rn(s, v.hi))};
    }
    p[i] = v.hi;
    p[n + i] = v.lo;
  }
}

// (templates only so that every translation unit may instantiate them)
template <int KIND = INNER_PAIRS>
__global__ void __launch_bounds__(kVecThreads)
    k_cg_direction_pairs(float* __restrict__ p, const float* __restrict__ r, size_t n, const CgState<double>* st) {
  cg_direction_pairs_body(p, r, n, st, blockIdx.x, gridDim.x);
}

template <int KIND = INNER_PAIRS>
__global__ void __launch_bounds__(kVecThreads)
    k_cg_direction_pairs_batched(const PairInst* __restrict__ insts) {
  const PairInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  cg_direction_pairs_body(v.pb0, v.r, v.n, v.st, blockIdx.x, v.nblk);
}

template <int KIND = INNER_PAIRS>
__global__ void __launch_bounds__(kVecThreads)
    k_cg_update_pairs(float* __restrict__ x, const float* __restrict__ pb0, const float* __restrict__ pb1,
                      float* __restrict__ r, const float* __restrict__ Ap, size_t n, CgState<double>* st,
                      ReduceScratch red) {
  cg_update_pairs_body(x, pb0, pb1, r, Ap, n, st, red, blockIdx.x, gridDim.x);
}

template <int KIND = INNER_PAIRS>
__global__ void __launch_bounds__(kVecThreads) k_cg_update_pairs_batched(const PairInst* __restrict__ insts) {
  const PairInst v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  cg_update_pairs_body(v.x, v.pb0, v.pb1, v.r, v.Ap, v.n, v.st, v.red, blockIdx.x, v.nblk);
}

// Inner restart after an FP64 residual: r = r64 in the inner format, e = 0,
// and the inner CG state for the next run of iterations (first: p = r; else
// beta = r.r / r_prev.r_prev, the direction kept).  The run stops at a
// reliable update (sqrt(r.r) < delta * its max), at `stop`, at breakdown, or
// after max_it more iterations.
template <int KIND>
__device__ __forceinline__ void inner_restart_body(const double* __restrict__ r64, float* __restrict__ r,
                                                   float* __restrict__ e, size_t n,
                                                   CgState<typename InnerScalar<KIND>::type>* st,
                                                   const ReduceScratch& red, int first, double delta, double stop,
                                                   int max_it, int bid, int nblocks) {
  using S = typename InnerScalar<KIND>::type;
  __shared__ S sh[32];
  S acc = S(0);
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double v = r64[i];
    const float h = (float)v;
    r[i] = h;
    e[i] = 0.f;
    if (KIND == INNER_PAIRS) {
      r[n + i] = (float)(v - (double)h);
      e[n + i] = 0.f;
      acc = fma((S)v, (S)v, acc);
    } else {
      acc = fma((S)h, (S)h, acc);
    }
  }
  const S bt = block_sum<S, kVecThreads>(acc, sh);
  S total;
  if (grid_sum_last<S, kVecThreads>(bt, red, bid, nblocks, sh, &total) && threadIdx.x == 0) {
    if (first) {
      st->first = 1;
      st->it = 0;
      st->parity = 0;
      st->beta = S(0);
      st->status = (int)SIPG_OK;
    } else {
      st->beta = total / st->rr_prev;
      st->first = 0;
    }
    st->rr = total;
    st->rmax = sqrt(total);
    st->delta = (S)delta;
    st->stop = (S)stop;
    st->max_it = st->it + max_it;
    st->need_update = 0;
    st->done = (total == S(0)) ? 1 : 0;
  }
}

// x64 += e
template <int KIND>
__device__ __forceinline__ void inner_fold_body(double* __restrict__ x, const float* __restrict__ e, size_t n, int bid,
                                                int nblocks) {
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) {
    double v = (double)e[i];
    if (KIND == INNER_PAIRS) v += (double)e[n + i];
    x[i] += v;
  }
}

}  // namespace sipg
