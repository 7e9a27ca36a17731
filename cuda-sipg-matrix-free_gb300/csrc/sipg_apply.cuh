// sipg_apply.cuh -- the fused SIPG-SEM operator apply for sm_103a.
//
// One kernel computes y = A u for a TX x TY tile of elements per CTA (one
// thread per element): the tensor-product LGL volume term, the lifting of the
// face jumps, and the interior / boundary (Nitsche) face terms -- everything the
// reference does in three passes over HBM (volume, flux_term6a, flux_term6b in
// sipg_sem_2d.hpp:167-201) in one.
//
// Face-centric formulation.  Every face has a "0-side" element that touches it
// with node index 0 (x faces: the right element's i1 = 0; y faces: the upper
// element's i2 = 0) and an "N-side" element that touches it with node index P.
// With u0/uN the two traces, d0 = sum_i D[i][0] u0side(i), dN = sum_i D[i][P]
// uNside(i) the two one-sided normal derivatives, kappa = 1/2 inside and 1 on
// the boundary (where the missing side counts as zero), each face stores
//     J_j = kappa w_j (u0 - uN)                 (the lifted jump)
//     Q_j = w_j (kappa (d0 + dN) + nu (u0 - uN)) (consistency + penalty)
// The 0-side element adds Q_j to its face node, the N-side element subtracts
// it, and both lift J_j with D[.][0] / D[.][P].  This is algebraically the
// reference's e, f, g, h and a, b, c, d of sipg_sem_2d_gpu_kernels.hpp:209-247
// and :277-312, computed once per face instead of once per side.
//
// Phases of a CTA (all smem; halo elements are read from global/L2 and only
// their one relevant face is computed):
//   0  load the tile's nodal blocks into smem (coalesced along x);
//   1a write the 0-side data (u0, d0) of every face;
//   1b the N-side element of each face combines them into (J, Q);
//   2  each thread forms its n^2 outputs in registers: w_j K u along rows and
//      columns plus the lifting, then the face corrections, then the epilogue
//      (store, and in the CG modes a deterministic grid reduction).
#pragma once

#include "sipg_internal.cuh"

namespace sipg {

template <typename A>
__device__ __forceinline__ A warp_sum(A v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block; the result is valid in linear thread 0.  NT % 32 == 0.
template <typename A, int NT>
__device__ __forceinline__ A block_sum(A v, A* sh) {
  const int t = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;  // linear thread id
  v = warp_sum(v);
  if ((t & 31) == 0) sh[t >> 5] = v;
  __syncthreads();
  A s = A(0);
  if (t < 32) {
    s = (t < NT / 32) ? sh[t] : A(0);
    s = warp_sum(s);
  }
  return s;
}

// Deterministic grid reduction: every block stores its partial, the block that
// arrives last sums all partials in index order.  Returns true in the last
// block; *total is then valid in linear thread 0 of that block.
template <typename A, int NT>
__device__ __forceinline__ bool grid_sum_last(A block_total, const ReduceScratch& red, int bid, int nblocks, A* sh,
                                              A* total) {
  __shared__ int s_last;
  const int t = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;  // linear thread id
  if (t == 0) {
    red.partials[bid] = (double)block_total;
    __threadfence();
    const unsigned prev = atomicAdd(red.counter, 1u);
    s_last = (prev == (unsigned)(nblocks - 1));
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  A s = A(0);
  for (int i = t; i < nblocks; i += NT) s += (A)__ldcg(red.partials + i);
  s = block_sum<A, NT>(s, sh);
  if (t == 0) {
    *total = s;
    *red.counter = 0u;  // ready for the next launch on this scratch
  }
  return true;
}

// The same with the block id of a one-dimensional or two-dimensional grid.
template <typename A, int NT>
__device__ __forceinline__ bool grid_sum_last(A block_total, const ReduceScratch& red, int nblocks, A* sh, A* total) {
  return grid_sum_last<A, NT>(block_total, red, (int)(blockIdx.y * gridDim.x + blockIdx.x), nblocks, sh, total);
}

// Where the column form reads its weighted stiffness KW (n^3 values): from
// the kernel parameters (constant bank), or from shared memory where the
// table read with a per-row index overflows the constant cache.  Measured
// for FP64 at ~16 M DoF: shared memory pays at p = 8 (5.8 KB; 15.8 -> 17.0
// GDoF/s), not at p = 6 or 7 (2.7 and 4 KB).
template <typename T, int P>
struct KwInSmem {
  static constexpr bool value = P >= 8;
};

// Where a thread keeps its element's nodal block: only the owning thread
// reads it (halo elements come from global memory, neighbours exchange face
// values only), so where the n^2 values fit in registers -- FP32 up to p = 6
// (the row form, fully unrolled; measured: p = 4 426 -> 492 GDoF/s, p = 6
// 316 -> 366) -- they stay there, and the tile's shared memory holds the
// faces alone.
template <typename T, int P>
struct NodalInRegs {
  static constexpr bool value = sizeof(T) == 4 && P <= 6;
};

template <typename T, int P, int TX, int TY>
struct ApplySmem {
  static constexpr int N1 = P + 1, NN = N1 * N1, TE = TX * TY;
  static constexpr int US = NodalInRegs<T, P>::value ? 0 : NN * TE;  // nodal values of the tile
  static constexpr int XF = TY * 2 * N1 * (TX + 1);  // x faces [TY][2][N1][TX+1]
  static constexpr int YF = (TY + 1) * 2 * N1 * TX;  // y faces [TY+1][2][N1][TX]
  static constexpr int KW = KwInSmem<T, P>::value ? N1 * N1 * N1 : 0;
  static constexpr size_t bytes = (size_t)(US + XF + YF + KW) * sizeof(T);
};

// Phase-2 form per (precision, degree): the column form for FP64 (whose n^2
// outputs would not fit in registers beyond small p, and whose FP64 pipe is
// the bottleneck anyway), the all-register form for FP32 up to p = 6.
template <typename T, int P>
struct ApplyColumnForm {
  static constexpr bool value = (sizeof(T) == 8) || (P >= 7);
  // Unroll limits that keep FP64 at high degree out of register spills: the
  // phase-0 load batch, the halo face loop, and the phase-2 column loop.
  static constexpr int load_unroll = (sizeof(T) == 8 && P >= 5) ? 2 * (P + 1) : (P + 1) * (P + 1);
  static constexpr int halo_unroll = (sizeof(T) == 8 && P >= 5) ? 1 : (P + 1);
  static constexpr int col_unroll = (sizeof(T) == 8 && P >= 5) ? 1 : (P + 1);
};

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

// J and Q of one face node (kappa = 1/2 inside, 1 on the boundary, where the
// missing side's values are zero).  The products and the sum are explicitly
// rounded: where a kernel calls this with literal constants (a boundary
// face), the compiler would otherwise fold fma(1, s, nu * jmp) into s + nu *
// jmp and contract that into one FMA -- a last-bit difference from the same
// face computed with runtime values by another tile shape.
template <typename T>
__device__ __forceinline__ void face_combine(T w, T wh, T nu, bool interior, T u0, T d0, T uN, T dN, T& J,
                                             T& Q) {
  const T kap = interior ? T(0.5) : T(1);
  const T jmp = u0 - uN;
  J = mul_rn(interior ? wh : w, jmp);  // kappa w from the table: wh = w / 2
  Q = mul_rn(w, fma(kap, add_rn(d0, dN), mul_rn(nu, jmp)));
}

// The face corrections of output (i1, j) as the start of its chain: +Q of
// the x face it is the 0-side of (i1 = 0), -Q of the one it is the N-side of
// (i1 = P), then likewise for the y faces (j = 0, j = P); zero elsewhere.
// qx0 / qxN / qy0 / qyN are those four faces' Q at this node.
template <typename T, int N>
__device__ __forceinline__ T face_seed(int i1, int j, T qx0, T qxN, T qy0, T qyN) {
  T s = T(0);
  if (i1 == 0) s = qx0;
  if (i1 == N) s = -qxN;
  const bool xface = (i1 == 0) || (i1 == N);
  if (j == 0) s = xface ? s + qy0 : qy0;
  if (j == N) s = xface ? s - qyN : -qyN;
  return s;
}

// The reduced total of a CG / residual apply, in the block that summed it
// (one thread): alpha = rr / p.Ap (and the direction parity flip) after a CG
// or DOT apply; the start of a solve after r = b - A x.
template <typename T, int MODE>
__device__ __forceinline__ void apply_finish(CgState<T>* st, T total, int par) {
  if (MODE == APPLY_CG || MODE == APPLY_DOT) {
    const T alpha = st->rr / total;
    st->pAp = total;
    st->alpha = alpha;
    if (MODE == APPLY_CG) st->parity = 1 - par;  // every block read the parity before arriving here
    if (!(total > T(0)) || !isfinite(alpha)) {
      st->status = (int)SIPG_ERR_BREAKDOWN;
      st->done = 1;
    }
  } else {  // APPLY_RESID: r = b - A x, start of a CG solve
    st->rr = total;
    st->it = 0;
    st->first = 1;
    st->status = (int)SIPG_OK;
    st->done = !(sqrt(total) > st->stop && 0 < st->max_it);
    if (!isfinite(total)) {
      st->status = (int)SIPG_ERR_BREAKDOWN;
      st->done = 1;
    }
  }
}

// One CTA's work: tile (bx, by) of the operator in `a`; `bid` / `nblocks` name
// the block among the blocks that reduce into a.red (CG / residual modes).
template <typename T, int P, int TX, int TY, int MODE>
__device__ __forceinline__ void apply_tile(const ApplyArgs<T>& a, const Tab<T, P>& tb, int bx, int by, int bid,
                                           int nblocks) {
  constexpr int N = P, N1 = P + 1, NN = N1 * N1, TE = TX * TY;
  constexpr bool kCols = ApplyColumnForm<T, P>::value;
  constexpr int BASE = apply_base_mode(MODE);
  // FP32 (and the FP64 *_PIVOT modes): every sum whose coefficients add up to zero (a derivative row D, a
  // stiffness row K = D^T W D) is taken over differences from one value of
  // the line, v_i - v_0, which leaves it unchanged in exact arithmetic and
  // drops the part common to the line exactly.  Rounding then scales with
  // the variation of u across an element (h |grad u|), not with u itself: on
  // a smooth vector the FP32 operator's relative error falls from
  // ~kappa eps_32 (~1 at 512 x 512, p = 6) to ~dim eps_32, which is what an
  // FP32 inner solve needs to see the smooth modes.  (The other FP64 modes
  // keep the plain sums: their results stay bit-identical to the unpivoted
  // kernel's.)
  constexpr bool kPivot = sizeof(T) == 4 || MODE != BASE;
  using S = ApplySmem<T, P, TX, TY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T red_sh[32];
  T* __restrict__ us = reinterpret_cast<T*>(smem_raw);
  T* __restrict__ xf = us + S::US;
  T* __restrict__ yf = xf + S::XF;
  T* __restrict__ kws = yf + S::YF;  // KW, when KwInSmem
  constexpr bool kKwSmem = KwInSmem<T, P>::value;
  auto KWv = [&](int k) -> T { return kKwSmem ? kws[k] : tb.KW[k]; };

  constexpr bool kDot = (BASE == APPLY_CG || BASE == APPLY_DOT);  // p.Ap -> alpha
  if (kDot) {
    if (*(volatile int*)&a.st->done) return;  // converged: the launch is a no-op
  }

  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
  const int dim = a.dim;
  const int x0 = bx * TX, y0 = a.row0 + by * TY;
  const int gx = x0 + tx, gy = y0 + ty;
  const bool act = (gx < dim) && (gy < dim);
  const size_t noe = (size_t)dim * dim;
  const size_t e = (size_t)gy * dim + gx;

  bool first = true;
  T beta = T(0);
  int par = 0;
  if (BASE == APPLY_CG) {
    first = a.st->first != 0;
    beta = a.st->beta;
    par = a.st->parity;
  }
  const T* __restrict__ pold = par ? a.pbuf1 : a.pbuf0;
  T* __restrict__ pnew = par ? a.pbuf0 : a.pbuf1;
  // value k of element ee as the operator sees it (CG: p = r + beta p_old)
  auto ld = [&](int k, size_t ee) -> T {
    const T r = __ldg(a.in + (size_t)k * noe + ee);
    if (BASE == APPLY_CG) return first ? r : fma(beta, __ldg(pold + (size_t)k * noe + ee), r);
    return r;
  };
  constexpr bool kRegs = NodalInRegs<T, P>::value;
  static_assert(!kRegs || !kCols, "register-resident nodal blocks: row form only");
  T ureg[kRegs ? NN : 1];  // the element's nodal block, when kRegs
  auto U = [&](int i1, int i2) -> T& { return kRegs ? ureg[kRegs ? i1 * N1 + i2 : 0] : us[(i1 * N1 + i2) * TE + t]; };
  // a read that the compiler may not hoist out of the column loop (keeps the
  // column form's register footprint at O(n) instead of O(n^2))
  auto Uv = [&](int i1, int i2) -> T { return ((volatile T*)us)[(i1 * N1 + i2) * TE + t]; };
  auto XFr = [&](int row, int comp, int j, int fx) -> T& { return xf[((row * 2 + comp) * N1 + j) * (TX + 1) + fx]; };
  auto YFr = [&](int frow, int comp, int j, int col) -> T& { return yf[((frow * 2 + comp) * N1 + j) * TX + col]; };
  const T nu = a.nu;
  auto combine = [&](int j, bool interior, T u0, T d0, T uN, T dN, T& J, T& Q) {
    face_combine<T>(tb.w[j], tb.WH[j], nu, interior, u0, d0, uN, dN, J, Q);
  };

  // ---- phase 0: the tile's nodal blocks -> smem --------------------------
  // (loads only: CG mode writes the new direction in phase 2, so that no
  // store sits between loads the compiler could otherwise batch)
  if (kKwSmem)
    for (int k = t; k < N1 * N1 * N1; k += TE) kws[k] = tb.KW[k];
#pragma unroll(ApplyColumnForm<T, P>::load_unroll)
  for (int k = 0; k < NN; ++k) {
    const T v = act ? ld(k, e) : T(0);
    if (kRegs) ureg[kRegs ? k : 0] = v;
    else us[k * TE + t] = v;
  }
  __syncthreads();

  // ---- phase 1a: 0-side data (u0, d0) -------------------------------------
  if (act) {
#pragma unroll
    for (int j = 0; j < N1; ++j) {  // LEFT face of this element (x face slot tx)
      T d = T(0);
      const T pv = kPivot ? U(0, j) : T(0);
#pragma unroll
      for (int i = 0; i < N1; ++i) d = fma(tb.D0[i], kPivot ? U(i, j) - pv : U(i, j), d);
      XFr(ty, 0, j, tx) = U(0, j);
      XFr(ty, 1, j, tx) = d;
    }
#pragma unroll
    for (int j = 0; j < N1; ++j) {  // DOWN face (y face slot ty+1)
      T d = T(0);
      const T pv = kPivot ? U(j, 0) : T(0);
#pragma unroll
      for (int i = 0; i < N1; ++i) d = fma(tb.D0[i], kPivot ? U(j, i) - pv : U(j, i), d);
      YFr(ty + 1, 0, j, tx) = U(j, 0);
      YFr(ty + 1, 1, j, tx) = d;
    }
  }
  if (t < TX) {  // halo above: element (y0-1, x0+t), its DOWN face
    const int hx = x0 + t;
    if (y0 > 0 && hx < dim) {
      const size_t he = (size_t)(y0 - 1) * dim + hx;
#pragma unroll(ApplyColumnForm<T, P>::halo_unroll)
      for (int j = 0; j < N1; ++j) {
        T d = T(0), u0 = T(0);
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const T v = ld(j * N1 + i, he);
          if (i == 0) u0 = v;
          d = fma(tb.D0[i], kPivot ? v - u0 : v, d);
        }
        YFr(0, 0, j, t) = u0;
        YFr(0, 1, j, t) = d;
      }
    }
  } else if (t < TX + TY) {  // halo right: element (y0+r, x0+TX), its LEFT face
    const int r = t - TX, hy = y0 + r, hx = x0 + TX;
    if (hx < dim && hy < dim) {
      const size_t he = (size_t)hy * dim + hx;
#pragma unroll(ApplyColumnForm<T, P>::halo_unroll)
      for (int j = 0; j < N1; ++j) {
        T d = T(0), u0 = T(0);
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const T v = ld(i * N1 + j, he);
          if (i == 0) u0 = v;
          d = fma(tb.D0[i], kPivot ? v - u0 : v, d);
        }
        XFr(r, 0, j, TX) = u0;
        XFr(r, 1, j, TX) = d;
      }
    }
  }
  __syncthreads();

  // ---- phase 1b: N-side combines (J, Q) -----------------------------------
  if (act) {
    const bool rint = gx < dim - 1;  // RIGHT face is interior
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      T dN = T(0);
      const T pv = kPivot ? U(0, j) : T(0);
#pragma unroll
      for (int i = 0; i < N1; ++i) dN = fma(tb.DN[i], kPivot ? U(i, j) - pv : U(i, j), dN);
      const T u0 = rint ? XFr(ty, 0, j, tx + 1) : T(0);
      const T d0 = rint ? XFr(ty, 1, j, tx + 1) : T(0);
      T J, Q;
      combine(j, rint, u0, d0, U(N, j), dN, J, Q);
      XFr(ty, 0, j, tx + 1) = J;
      XFr(ty, 1, j, tx + 1) = Q;
    }
    const bool uint_ = gy > 0;  // UP face is interior
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      T dN = T(0);
      const T pv = kPivot ? U(j, 0) : T(0);
#pragma unroll
      for (int i = 0; i < N1; ++i) dN = fma(tb.DN[i], kPivot ? U(j, i) - pv : U(j, i), dN);
      const T u0 = uint_ ? YFr(ty, 0, j, tx) : T(0);
      const T d0 = uint_ ? YFr(ty, 1, j, tx) : T(0);
      T J, Q;
      combine(j, uint_, u0, d0, U(j, N), dN, J, Q);
      YFr(ty, 0, j, tx) = J;
      YFr(ty, 1, j, tx) = Q;
    }
    if (gx == 0) {  // LEFT face on the domain boundary: 0-side only
#pragma unroll
      for (int j = 0; j < N1; ++j) {
        T J, Q;
        combine(j, false, XFr(ty, 0, j, tx), XFr(ty, 1, j, tx), T(0), T(0), J, Q);
        XFr(ty, 0, j, tx) = J;
        XFr(ty, 1, j, tx) = Q;
      }
    }
    if (gy == dim - 1) {  // DOWN face on the domain boundary
#pragma unroll
      for (int j = 0; j < N1; ++j) {
        T J, Q;
        combine(j, false, YFr(ty + 1, 0, j, tx), YFr(ty + 1, 1, j, tx), T(0), T(0), J, Q);
        YFr(ty + 1, 0, j, tx) = J;
        YFr(ty + 1, 1, j, tx) = Q;
      }
    }
  }
  if (t < TX) {  // halo below: element (y0+TY, x0+t) is the N-side (its UP face) of y face TY
    const int hx = x0 + t, hy = y0 + TY;
    if (hy < dim && hx < dim) {
      const size_t he = (size_t)hy * dim + hx;
#pragma unroll(ApplyColumnForm<T, P>::halo_unroll)
      for (int j = 0; j < N1; ++j) {
        T dN = T(0), uN = T(0), v0 = T(0);
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const T v = ld(j * N1 + i, he);
          if (i == 0) v0 = v;
          if (i == N) uN = v;
          dN = fma(tb.DN[i], kPivot ? v - v0 : v, dN);
        }
        T J, Q;
        combine(j, true, YFr(TY, 0, j, t), YFr(TY, 1, j, t), uN, dN, J, Q);
        YFr(TY, 0, j, t) = J;
        YFr(TY, 1, j, t) = Q;
      }
    }
  } else if (t < TX + TY) {  // halo left: element (y0+r, x0-1) is the N-side (its RIGHT face) of x face 0
    const int r = t - TX, hy = y0 + r;
    if (x0 > 0 && hy < dim) {
      const size_t he = (size_t)hy * dim + (x0 - 1);
#pragma unroll(ApplyColumnForm<T, P>::halo_unroll)
      for (int j = 0; j < N1; ++j) {
        T dN = T(0), uN = T(0), v0 = T(0);
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const T v = ld(i * N1 + j, he);
          if (i == 0) v0 = v;
          if (i == N) uN = v;
          dN = fma(tb.DN[i], kPivot ? v - v0 : v, dN);
        }
        T J, Q;
        combine(j, true, XFr(r, 0, j, 0), XFr(r, 1, j, 0), uN, dN, J, Q);
        XFr(r, 0, j, 0) = J;
        XFr(r, 1, j, 0) = Q;
      }
    }
  }
  __syncthreads();

  // ---- phase 2: outputs ---------------------------------------------------
  // Row form: w_j sum_i K(i1,i) u(i,j) + D[i1][0] J_L,j + D[i1][P] J_R,j.
  // Column form: w_i1 sum_i K(i2,i) u(i1,i) + D[i2][0] J_D,i1 + D[i2][P] J_U,i1.
  // (The column form reads w_b K(a,i) from KW and accumulates every term
  // into one chain per output.)
  // Then the face nodes get +Q (0-side) / -Q (N-side).  kCols computes one
  // output column at a time (n live accumulators; the row contractions read
  // smem n times) -- the register-light form; otherwise all n^2 outputs stay in
  // registers and every value is read from smem twice.
  T acc = T(0);
  if (act) {
    if (kCols) {
      T eJ[N1], fJ[N1];
#pragma unroll
      for (int j = 0; j < N1; ++j) {
        eJ[j] = XFr(ty, 0, j, tx);
        fJ[j] = XFr(ty, 0, j, tx + 1);
      }
#pragma unroll(ApplyColumnForm<T, P>::col_unroll)
      for (int i1 = 0; i1 < N1; ++i1) {
        T o[N1], c[N1];
        // each output starts from its face corrections (+-Q) and x-face
        // lifting, then takes the weighted volume sums (w folded into KW)
        // and the y-face lifting: 2n + 4 FP64 operations (+1 at corners)
#pragma unroll
        for (int j = 0; j < N1; ++j) {
          const bool xf = (i1 == 0) || (i1 == N);
          const T seed = face_seed<T, N>(i1, j, xf ? XFr(ty, 1, j, tx) : T(0), xf ? XFr(ty, 1, j, tx + 1) : T(0),
                                         (j == 0) ? YFr(ty + 1, 1, i1, tx) : T(0), (j == N) ? YFr(ty, 1, i1, tx) : T(0));
          o[j] = fma(tb.D0[i1], eJ[j], fma(tb.DN[i1], fJ[j], seed));
        }
        T p0[N1];  // the x-sums' pivots u(0, j) (FP32)
#pragma unroll
        for (int j = 0; j < N1; ++j) p0[j] = kPivot ? Uv(0, j) : T(0);
#pragma unroll
        for (int i = 0; i < N1; ++i) {
#pragma unroll
          for (int j = 0; j < N1; ++j)
            o[j] = fma(KWv((i1 * N1 + i) * N1 + j), kPivot ? Uv(i, j) - p0[j] : Uv(i, j), o[j]);
        }
        T cp[N1];  // the row (i1, .), less its first value (FP32)
#pragma unroll
        for (int i = 0; i < N1; ++i) c[i] = U(i1, i);
#pragma unroll
        for (int i = 0; i < N1; ++i) cp[i] = kPivot ? c[i] - c[0] : c[i];
        const T gj = YFr(ty + 1, 0, i1, tx), hj = YFr(ty, 0, i1, tx);
#pragma unroll
        for (int j = 0; j < N1; ++j) {
          T v = o[j];
#pragma unroll
          for (int i = 0; i < N1; ++i) v = fma(KWv((j * N1 + i) * N1 + i1), cp[i], v);
          v = fma(tb.D0[j], gj, v);
          o[j] = fma(tb.DN[j], hj, v);
        }
#pragma unroll
        for (int j = 0; j < N1; ++j) {
          const int k = i1 * N1 + j;
          const size_t gk = (size_t)k * noe + e;
          if (BASE == APPLY_RESID) {
            const T rv = __ldg(a.b + gk) - o[j];
            a.out[gk] = rv;
            acc = fma(rv, rv, acc);
          } else {
            a.out[gk] = o[j];
            if (BASE == APPLY_CG) pnew[gk] = c[j];
            if (kDot) acc = fma(c[j], o[j], acc);
          }
        }
      }
    } else {
      T o[NN];
#pragma unroll
      for (int j = 0; j < N1; ++j) {  // rows
        const T ej = XFr(ty, 0, j, tx), fj = XFr(ty, 0, j, tx + 1);
        T r[N1];
#pragma unroll
        for (int i = 0; i < N1; ++i) r[i] = U(i, j);
        if (kPivot) {
          const T r0 = r[0];
#pragma unroll
          for (int i = 0; i < N1; ++i) r[i] = r[i] - r0;
        }
#pragma unroll
        for (int i1 = 0; i1 < N1; ++i1) {
          T s = T(0);
#pragma unroll
          for (int i = 0; i < N1; ++i) s = fma(tb.K[i1 * N1 + i], r[i], s);
          o[i1 * N1 + j] = fma(tb.w[j], s, fma(tb.D0[i1], ej, tb.DN[i1] * fj));
        }
      }
#pragma unroll
      for (int j = 0; j < N1; ++j) {  // columns
        const T gj = YFr(ty + 1, 0, j, tx), hj = YFr(ty, 0, j, tx);
        T c[N1];
#pragma unroll
        for (int i = 0; i < N1; ++i) c[i] = U(j, i);
        if (kPivot) {
          const T c0 = c[0];
#pragma unroll
          for (int i = 0; i < N1; ++i) c[i] = c[i] - c0;
        }
#pragma unroll
        for (int i2 = 0; i2 < N1; ++i2) {
          T s = T(0);
#pragma unroll
          for (int i = 0; i < N1; ++i) s = fma(tb.K[i2 * N1 + i], c[i], s);
          T v = fma(tb.w[j], s, o[j * N1 + i2]);
          v = fma(tb.D0[i2], gj, v);
          o[j * N1 + i2] = fma(tb.DN[i2], hj, v);
        }
      }
#pragma unroll
      for (int j = 0; j < N1; ++j) {  // consistency + penalty at the face nodes
        o[0 * N1 + j] += XFr(ty, 1, j, tx);
        o[N * N1 + j] -= XFr(ty, 1, j, tx + 1);
        o[j * N1 + 0] += YFr(ty + 1, 1, j, tx);
        o[j * N1 + N] -= YFr(ty, 1, j, tx);
      }
#pragma unroll
      for (int k = 0; k < NN; ++k) {
        const size_t gk = (size_t)k * noe + e;
        if (BASE == APPLY_RESID) {
          const T rv = __ldg(a.b + gk) - o[k];
          a.out[gk] = rv;
          acc = fma(rv, rv, acc);
        } else {
          a.out[gk] = o[k];
          if (kDot) {
            const T pk = kRegs ? ureg[kRegs ? k : 0] : us[k * TE + t];
            if (BASE == APPLY_CG) pnew[gk] = pk;
            acc = fma(pk, o[k], acc);
          }
        }
      }
    }
  }

  if (BASE != APPLY_PLAIN) {
    const T bt = block_sum<T, TE>(acc, red_sh);
    T total;
    if (grid_sum_last<T, TE>(bt, a.red, bid, nblocks, red_sh, &total) && t == 0)
      apply_finish<T, BASE>(a.st, total, par);
  }
}

template <typename T, int P, int TX, int TY, int MODE>
__global__ void __launch_bounds__(TX* TY)
    k_sipg_apply(const __grid_constant__ ApplyArgs<T> a, const __grid_constant__ Tab<T, P> tb) {
  apply_tile<T, P, TX, TY, MODE>(a, tb, blockIdx.x, blockIdx.y, blockIdx.y * gridDim.x + blockIdx.x,
                                 gridDim.x * gridDim.y);
}

// Many operators of the same degree in one launch: block g works on tile
// g - tile_start[i] of instance i, where tile_start[i] <= g < tile_start[i+1]
// (the instances' tiles concatenated; each instance reduces into its own
// scratch and state, and a converged instance's blocks return at once).
template <typename T, int P, int TX, int TY, int MODE>
__global__ void __launch_bounds__(TX* TY)
    k_sipg_apply_batched(const ApplyArgs<T>* __restrict__ insts, const int* __restrict__ tile_start, int ninst,
                         const __grid_constant__ Tab<T, P> tb) {
  const int g = blockIdx.x;
  int lo = 0, hi = ninst - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(tile_start + mid) <= g) lo = mid;
    else hi = mid - 1;
  }
  const ApplyArgs<T> a = insts[lo];
  const int lt = g - __ldg(tile_start + lo);
  const int tiles_x = (a.dim + TX - 1) / TX, tiles_y = (a.dim + TY - 1) / TY;
  apply_tile<T, P, TX, TY, MODE>(a, tb, lt % tiles_x, lt / tiles_x, lt, tiles_x * tiles_y);
}

template <typename T, int P, int TX, int TY>
cudaError_t launch_apply_tile(int mode, const ApplyArgs<T>& a, const Tab<T, P>& tb, cudaStream_t s) {
  using S = ApplySmem<T, P, TX, TY>;
  const int rows = a.nrows > 0 ? a.nrows : a.dim;
  const dim3 grid((a.dim + TX - 1) / TX, (rows + TY - 1) / TY), block(TX, TY);
  const size_t smem = S::bytes;
  // the dynamic shared memory opt-in, for all three modes (outside any capture)
  cudaError_t err = cudaFuncSetAttribute(k_sipg_apply<T, P, TX, TY, APPLY_PLAIN>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_sipg_apply<T, P, TX, TY, APPLY_CG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_sipg_apply<T, P, TX, TY, APPLY_RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_sipg_apply<T, P, TX, TY, APPLY_DOT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
  if constexpr (sizeof(T) == 8) {
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(k_sipg_apply<T, P, TX, TY, APPLY_RESID_PIVOT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(k_sipg_apply<T, P, TX, TY, APPLY_DOT_PIVOT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  } else {
    mode = apply_base_mode(mode);  // the FP32 sums are always pivoted
  }
  if (err != cudaSuccess) return err;
  switch (mode) {
    case APPLY_PREPARE:
      return cudaSuccess;
    case APPLY_PLAIN:
      k_sipg_apply<T, P, TX, TY, APPLY_PLAIN><<<grid, block, smem, s>>>(a, tb);
      break;
    case APPLY_CG:
      k_sipg_apply<T, P, TX, TY, APPLY_CG><<<grid, block, smem, s>>>(a, tb);
      break;
    case APPLY_RESID:
      k_sipg_apply<T, P, TX, TY, APPLY_RESID><<<grid, block, smem, s>>>(a, tb);
      break;
    case APPLY_DOT:
      k_sipg_apply<T, P, TX, TY, APPLY_DOT><<<grid, block, smem, s>>>(a, tb);
      break;
    case APPLY_RESID_PIVOT:
      if constexpr (sizeof(T) == 8) k_sipg_apply<T, P, TX, TY, APPLY_RESID_PIVOT><<<grid, block, smem, s>>>(a, tb);
      break;
    case APPLY_DOT_PIVOT:
      if constexpr (sizeof(T) == 8) k_sipg_apply<T, P, TX, TY, APPLY_DOT_PIVOT><<<grid, block, smem, s>>>(a, tb);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  count_launch();
  return cudaGetLastError();
}

// Tile shapes compiled for each degree: TX = 32 (one warp per element row),
// TY = 2, 4 or 8 rows; shapes whose shared memory exceeds 227 KB are skipped.
template <typename T, int P>
cudaError_t launch_apply_p(const TileCfg& cfg, int mode, const ApplyArgs<T>& a, const HostTables& h, cudaStream_t s) {
  const Tab<T, P> tb = make_tab<T, P>(h);
  constexpr size_t kMax = 227 * 1024;
  constexpr bool fits8 = ApplySmem<T, P, 32, 8>::bytes <= kMax;
  if (cfg.tx != 32 || cfg.tpe != 1) return cudaErrorInvalidValue;
  switch (cfg.ty) {
    case 2:
      return launch_apply_tile<T, P, 32, 2>(mode, a, tb, s);
    case 4:
      return launch_apply_tile<T, P, 32, 4>(mode, a, tb, s);
    case 8:
      if (!fits8) return cudaErrorInvalidConfiguration;
      return launch_apply_tile<T, P, 32, (fits8 ? 8 : 4)>(mode, a, tb, s);
  }
  return cudaErrorInvalidValue;
}

template <typename T, int P, int TX, int TY>
cudaError_t launch_apply_batched_tile(int mode, const ApplyArgs<T>* insts, const int* tile_start, int ninst,
                                      int total_tiles, const Tab<T, P>& tb, cudaStream_t s) {
  const size_t smem = ApplySmem<T, P, TX, TY>::bytes;
  cudaError_t err = cudaFuncSetAttribute(k_sipg_apply_batched<T, P, TX, TY, APPLY_PLAIN>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_sipg_apply_batched<T, P, TX, TY, APPLY_CG>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_sipg_apply_batched<T, P, TX, TY, APPLY_RESID>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_sipg_apply_batched<T, P, TX, TY, APPLY_DOT>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if constexpr (sizeof(T) == 8) {
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(k_sipg_apply_batched<T, P, TX, TY, APPLY_RESID_PIVOT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(k_sipg_apply_batched<T, P, TX, TY, APPLY_DOT_PIVOT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  } else {
    mode = apply_base_mode(mode);
  }
  if (err != cudaSuccess || mode == APPLY_PREPARE || total_tiles == 0) return err;
  const dim3 grid(total_tiles), block(TX, TY);
  switch (mode) {
    case APPLY_PLAIN:
      k_sipg_apply_batched<T, P, TX, TY, APPLY_PLAIN><<<grid, block, smem, s>>>(insts, tile_start, ninst, tb);
      break;
    case APPLY_CG:
      k_sipg_apply_batched<T, P, TX, TY, APPLY_CG><<<grid, block, smem, s>>>(insts, tile_start, ninst, tb);
      break;
    case APPLY_RESID:
      k_sipg_apply_batched<T, P, TX, TY, APPLY_RESID><<<grid, block, smem, s>>>(insts, tile_start, ninst, tb);
      break;
    case APPLY_DOT:
      k_sipg_apply_batched<T, P, TX, TY, APPLY_DOT><<<grid, block, smem, s>>>(insts, tile_start, ninst, tb);
      break;
    case APPLY_RESID_PIVOT:
      if constexpr (sizeof(T) == 8)
        k_sipg_apply_batched<T, P, TX, TY, APPLY_RESID_PIVOT><<<grid, block, smem, s>>>(insts, tile_start, ninst, tb);
      break;
    case APPLY_DOT_PIVOT:
      if constexpr (sizeof(T) == 8)
        k_sipg_apply_batched<T, P, TX, TY, APPLY_DOT_PIVOT><<<grid, block, smem, s>>>(insts, tile_start, ninst, tb);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  count_launch();
  return cudaGetLastError();
}

template <typename T, int P>
cudaError_t launch_apply_batched_p(const TileCfg& cfg, int mode, const ApplyArgs<T>* insts, const int* tile_start,
                                   int ninst, int total_tiles, const HostTables& h, cudaStream_t s) {
  const Tab<T, P> tb = make_tab<T, P>(h);
  constexpr size_t kMax = 227 * 1024;
  constexpr bool fits8 = ApplySmem<T, P, 32, 8>::bytes <= kMax;
  // batched solves keep 32-element rows: their tiles are laid out by
  // tile_start for that width
  if (cfg.tx != 32) return cudaErrorInvalidValue;
  switch (cfg.ty) {
    case 2:
      return launch_apply_batched_tile<T, P, 32, 2>(mode, insts, tile_start, ninst, total_tiles, tb, s);
    case 4:
      return launch_apply_batched_tile<T, P, 32, 4>(mode, insts, tile_start, ninst, total_tiles, tb, s);
    case 8:
      if (!fits8) return cudaErrorInvalidConfiguration;
      return launch_apply_batched_tile<T, P, 32, (fits8 ? 8 : 4)>(mode, insts, tile_start, ninst, total_tiles, tb,
                                                                  s);
  }
  return cudaErrorInvalidValue;
}

template <typename T>
inline size_t apply_smem_bytes(int p, int ty) {
  size_t n1 = p + 1, te = 32 * ty;
  return (n1 * n1 * te + ty * 2 * n1 * 33 + (ty + 1) * 2 * n1 * 32) * sizeof(T);
}

}  // namespace sipg
