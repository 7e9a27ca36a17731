// sipg_cg.cuh -- conjugate-gradient building blocks: the vector update with
// its fused r.r reduction, the solve set-up, and the host driver that runs the
// iterations as CUDA graphs with every scalar kept on the device.
//
// One iteration is two kernels (the reference's is three kernels plus two
// blocking cuBLAS dots, conjugate_gradient_gpu.hpp:69-99):
//   k_sipg_apply<APPLY_CG>:  p = r + beta p_old (first: p = r), Ap = A p,
//                            pAp reduced, alpha = rr / pAp        (32 B/DoF)
//   k_cg_update:             x += alpha p, r -= alpha Ap, rr' reduced,
//                            beta = rr'/rr, it++, done test        (48 B/DoF)
// The direction is double-buffered (p_old, p_new alternate), so a CTA reading
// a neighbour's halo never sees a half-updated direction.
#pragma once

#include "sipg_apply.cuh"

namespace sipg {

constexpr int kVecThreads = 256;

// True if every pointer is 16-byte aligned (float4 access).
template <typename... Ps>
__device__ __forceinline__ bool aligned16(const Ps*... ps) {
  return ((reinterpret_cast<uintptr_t>(ps) & 15u) | ...) == 0;
}

// The iteration bookkeeping after r.r of the updated residual is known (one
// thread): it, beta, the stop test, or a reliable update due.
template <typename T>
__device__ __forceinline__ void cg_bookkeep(CgState<T>* st, T total) {
  const T rn = sqrt(total);
  st->it += 1;
  st->first = 0;
  st->rr_prev = st->rr;
  if (st->delta > T(0) && rn < st->delta * st->rmax) {
    // reliable update due: keep rr (the previous r.r, for beta after the
    // correction) and stop; the host replaces r by the FP64 residual
    st->need_update = 1;
    st->done = 1;
  } else {
    const T rr_old = st->rr;
    st->beta = total / rr_old;
    st->rr = total;
    st->rmax = fmax(st->rmax, rn);
    st->done = !(rn > st->stop && st->it < st->max_it);
  }
  if (!isfinite(total)) {
    st->status = (int)SIPG_ERR_BREAKDOWN;
    st->done = 1;
  }
}

// The preconditioned inner CG's bookkeeping once r.r of the updated residual
// is known (one thread): it, the stop test on sqrt(r.r).
template <typename T>
__device__ __forceinline__ void pcg_update_bookkeep(CgState<T>* st, T total) {
  st->rres = total;
  st->it += 1;
  st->first = 0;
  st->done = !(sqrt(total) > st->stop && st->it < st->max_it);
  if (!isfinite(total)) {
    st->status = (int)SIPG_ERR_BREAKDOWN;
    st->done = 1;
  }
}

// x += alpha p, r -= alpha Ap, r.r reduced; then the bookkeeping.  Block
// `bid` of `nblocks` works on a grid-stride slice of the vectors.
template <typename T>
__device__ __forceinline__ void cg_update_body(T* __restrict__ x, const T* __restrict__ pb0, const T* __restrict__ pb1,
                                               T* __restrict__ r, const T* __restrict__ Ap, size_t n, CgState<T>* st,
                                               const ReduceScratch& red, int bid, int nblocks) {
  __shared__ T sh[32];
  if (*(volatile int*)&st->done) return;
  const T alpha = st->alpha;
  const T* __restrict__ p = st->parity ? pb1 : pb0;  // the direction the apply just wrote
  T acc = T(0);
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] = fma(alpha, p[i], x[i]);
    const T ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    acc = fma(ri, ri, acc);
  }
  const T bt = block_sum<T, kVecThreads>(acc, sh);
  T total;
  if (grid_sum_last<T, kVecThreads>(bt, red, bid, nblocks, sh, &total) && threadIdx.x == 0) cg_bookkeep<T>(st, total);
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_cg_update(T* __restrict__ x, const T* __restrict__ pb0,
                                                           const T* __restrict__ pb1, T* __restrict__ r,
                                                           const T* __restrict__ Ap, size_t n, CgState<T>* st,
                                                           ReduceScratch red) {
  cg_update_body<T>(x, pb0, pb1, r, Ap, n, st, red, blockIdx.x, gridDim.x);
}

// p = r on the first iteration of a solve, else p = r + beta p, in place:
// the direction of an APPLY_DOT iteration.  Forming it here rather than in
// the apply (APPLY_CG) costs one more pass over p and r but lets the apply --
// whose occupancy shared memory caps at a few CTAs per SM -- read one vector
// instead of two, which hides most of its load latency.
template <typename T>
__device__ __forceinline__ void cg_direction_body(T* __restrict__ p, const T* __restrict__ r, size_t n, bool first,
                                                  T beta, int bid, int nblocks) {
  const size_t stride = (size_t)nblocks * blockDim.x;
  size_t head = 0;  // FP32 with 16-byte aligned vectors: four per thread and step
  if constexpr (sizeof(T) == 4) {
    if (aligned16(p, r)) {
      head = n & ~size_t(3);
      float4* __restrict__ p4 = reinterpret_cast<float4*>(p);
      const float4* __restrict__ r4 = reinterpret_cast<const float4*>(r);
      for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < head / 4; i += stride) {
        const float4 rv = r4[i];
        if (first) {
          p4[i] = rv;
        } else {
          float4 pv = p4[i];
          pv.x = fmaf(beta, pv.x, rv.x);
          pv.y = fmaf(beta, pv.y, rv.y);
          pv.z = fmaf(beta, pv.z, rv.z);
          pv.w = fmaf(beta, pv.w, rv.w);
          p4[i] = pv;
        }
      }
    }
  }
  for (size_t i = head + (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride)
    p[i] = first ? r[i] : fma(beta, p[i], r[i]);
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_cg_direction(T* __restrict__ p, const T* __restrict__ r, size_t n,
                                                              const CgState<T>* st) {
  if (*(volatile const int*)&st->done) return;
  cg_direction_body<T>(p, r, n, st->first != 0, st->beta, blockIdx.x, gridDim.x);
}

// Per-instance vector operands of a batch (instance = blockIdx.y).  Each
// instance uses its own nblk blocks (the rest of the grid row returns at
// once), so its reductions -- and so its iterates -- do not depend on which
// other instances share the launch.
template <typename T>
struct VecInst {
  T* x;
  T* pb0;
  T* pb1;
  T* r;
  T* Ap;
  size_t n;
  CgState<T>* st;
  ReduceScratch red;
  int nblk;
  int pad;
};

// Blocks one instance of n values uses in the batched vector kernels.
inline int inst_blocks(size_t n) {
  const size_t b = (n + 2047) / 2048;
  return (int)(b < 1 ? 1 : (b > 64 ? 64 : b));
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_cg_update_batched(const VecInst<T>* __restrict__ insts) {
  const VecInst<T> v = insts[blockIdx.y];
  if ((int)blockIdx.x >= v.nblk) return;
  cg_update_body<T>(v.x, v.pb0, v.pb1, v.r, v.Ap, v.n, v.st, v.red, blockIdx.x, v.nblk);
}

// b.b, and the stop threshold: tol (absolute) or tol*||b|| (relative).
template <typename T>
__device__ __forceinline__ void cg_init_body(const T* __restrict__ b, size_t n, CgState<T>* st, T tol, int rel,
                                             int max_it, const ReduceScratch& red, int bid, int nblocks) {
  __shared__ T sh[32];
  T acc = T(0);
  const size_t stride = (size_t)nblocks * blockDim.x;
  for (size_t i = (size_t)bid * blockDim.x + threadIdx.x; i < n; i += stride) acc = fma(b[i], b[i], acc);
  const T bt = block_sum<T, kVecThreads>(acc, sh);
  T total;
  if (grid_sum_last<T, kVecThreads>(bt, red, bid, nblocks, sh, &total) && threadIdx.x == 0) {
    st->bb = total;
    st->stop = rel ? tol * sqrt(total) : tol;
    st->max_it = max_it;
    st->it = 0;
    st->done = 0;
    st->first = 1;
    st->status = (int)SIPG_OK;
    st->parity = 0;
    st->need_update = 0;
    st->delta = T(0);
    st->rmax = T(0);
    st->alpha = st->beta = st->pAp = T(0);
  }
}

template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_cg_init(const T* __restrict__ b, size_t n, CgState<T>* st, T tol,
                                                         int rel, int max_it, ReduceScratch red) {
  cg_init_body<T>(b, n, st, tol, rel, max_it, red, blockIdx.x, gridDim.x);
}

}  // namespace sipg
