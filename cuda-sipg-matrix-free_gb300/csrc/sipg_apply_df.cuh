// sipg_apply_df.cuh -- the fused SIPG apply on double-float vectors with
// compensated arithmetic: every value and every operation on the FP32 pipes,
// about 48 significant bits throughout.
//
// A vector of n values is 2 n floats, the hi plane then the lo plane (value =
// hi + lo, |lo| <= ulp(hi) / 2).  Same tiling, phases and face-centric
// formulation as k_sipg_apply (sipg_apply.cuh); every table coefficient is
// split into hi + lo floats and every product and sum is a double-float
// operation (sipg_df.cuh).  Why: GB300 runs FP64 at ~1/50 of its FP32 rate,
// and the SIPG operator's condition number (~p^4 / h^2: 2e7 for 512 x 512
// elements at p = 6) is as large as 1 / eps_32, so a CG whose vectors are
// rounded to FP32 cannot converge -- the rounding noise of a smooth direction,
// amplified by A, is as large as the step it takes.  Pairs carry 2^-48
// relative noise instead, and this kernel keeps the matvec that accurate at
// FP32-pipe cost (about ten FP32 instructions per multiply-add).
//
// Modes: APPLY_PLAIN (y = A u), APPLY_CG (p = r + beta p_old as pairs, Ap,
// p.Ap reduced from double-float products, alpha = rr / pAp) and APPLY_DOT (Ap
// and alpha for a direction p formed beforehand, k_cg_direction_pairs: the
// apply then reads one vector, which at this kernel's occupancy -- two CTAs
// per SM, bound by shared memory -- halves its exposed load latency).  The CG scalars
// are FP64 (ApplyArgs::stp): a CG whose alpha, beta and dots carry 24 bits
// smears the low end of this operator's spectrum (relative rounding 6e-8
// times kappa ~ 1) and needs about three times the iterations.
#pragma once

#include "sipg_apply.cuh"
#include "sipg_df.cuh"

namespace sipg {

// The phase-2 form per degree: up to p = 4 the weighted stiffness KW[(a *
// N1 + i) * N1 + b] = w_b K[a][i] (n^3 three-float coefficients, 1.5 KB at
// p = 4) saves the two weight multiplications per output; from p = 5 on the
// table read with a per-row index overflows the constant cache and K with
// the weights applied afterwards is faster (measured: 68.7 against 59.8
// GDoF/s at p = 4, 800^2; 28.7 against 35.8 at p = 6, 512^2).
template <int P>
struct DfKwForm {
  static constexpr bool value = P <= 4;
};

template <int P>
struct TabDF {
  static constexpr int N1 = P + 1;
  cf w[N1], D0[N1], DN[N1], K[N1 * N1];
  cf KW[DfKwForm<P>::value ? N1 * N1 * N1 : 1];
};

// a double as three floats, h + m + l (exact to ~2^-72 relative)
inline cf split_cf(double v) {
  cf c;
  c.h = (float)v;
  const double r1 = v - (double)c.h;
  c.m = (float)r1;
  c.l = (float)(r1 - (double)c.m);
  return c;
}

template <int P>
inline TabDF<P> make_tab_df(const HostTables& h) {
  TabDF<P> t;
  const int n = P + 1;
  for (int i = 0; i < n; ++i) {
    t.w[i] = split_cf(h.w[i]);
    t.D0[i] = split_cf(h.D[i * n + 0]);
    t.DN[i] = split_cf(h.D[i * n + P]);
  }
  for (int i = 0; i < n * n; ++i) t.K[i] = split_cf(h.K[i]);
  // w_b K[a][i] to 72 bits: the product of two doubles, rounded once more
  // than either factor (2^-53 relative, far below the pairs' 2^-48)
  if (DfKwForm<P>::value)
    for (int a = 0; a < n; ++a)
      for (int i = 0; i < n; ++i)
        for (int b = 0; b < n; ++b) t.KW[(a * n + i) * n + b] = split_cf(h.w[b] * h.K[a * n + i]);
  return t;
}

template <int P, int TX, int TY>
struct ApplyDfSmem {
  static constexpr int N1 = P + 1, NN = N1 * N1, TE = TX * TY;
  static constexpr int US = 2 * NN * TE;             // nodal values: hi plane, lo plane
  static constexpr int XF = TY * 4 * N1 * (TX + 1);  // x faces [TY][4][N1][TX+1]: (u0h|Jh, u0l|Jl, d0h|Qh, d0l|Ql)
  static constexpr int YF = (TY + 1) * 4 * N1 * TX;  // y faces [TY+1][4][N1][TX]
  static constexpr size_t bytes = (size_t)(US + XF + YF) * sizeof(float);
};

// hi + lo renormalised so that hi = fl(hi + lo) (Dekker's FastTwoSum; |hi| >= |lo|)
__device__ __forceinline__ df df_norm(df v) {
  const float s = __fadd_rn(v.hi, v.lo);
  return df{s, __fsub_rn(v.lo, __fsub_rn(s, v.hi))};
}

// TPE threads per element (1 or 2; threadIdx.z = s): with 2, s = 0 takes the
// x faces, s = 1 the y faces, and the two split the element's nodal loads and
// output columns -- twice the resident warps for the same shared memory.
template <int P, int TX, int TY, int TPE, int MODE>
__device__ __forceinline__ void apply_tile_df(const ApplyArgs<float>& a, const TabDF<P>& tb, int bx, int by, int bid,
                                              int nblocks) {
  constexpr int N = P, N1 = P + 1, NN = N1 * N1, TE = TX * TY, NT = TE * TPE;
  static_assert(TPE == 1 || TPE == 2, "one or two threads per element");
  static_assert(TPE == 2 || TE >= TX + TY, "halo threads");
  using S = ApplyDfSmem<P, TX, TY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red_sh[32];
  float* __restrict__ us = reinterpret_cast<float*>(smem_raw);
  float* __restrict__ xf = us + S::US;
  float* __restrict__ yf = xf + S::XF;

  constexpr bool kReduce = (MODE == APPLY_CG || MODE == APPLY_DOT);  // p.Ap -> alpha
  if (kReduce) {
    if (*(volatile int*)&a.stp->done) return;
  }
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
  const int s = (TPE == 2) ? (int)threadIdx.z : 0;
  const int lt = s * TE + t;  // linear thread id
  const bool xs = (TPE == 1) || s == 0, ys = (TPE == 1) || s == 1;  // this thread's face directions
  // halo roles: A (the row above / below, x index ha), B (the column right /
  // left, row hb)
  const bool haloA = (TPE == 1) ? (t < TX) : (s == 0 && t < TX);
  const bool haloB = (TPE == 1) ? (t >= TX && t < TX + TY) : (s == 1 && t < TY);
  const int hb = (TPE == 1) ? t - TX : t;
  const int dim = a.dim;
  const int x0 = bx * TX, y0 = by * TY;
  const int gx = x0 + tx, gy = y0 + ty;
  const bool act = (gx < dim) && (gy < dim);
  const size_t noe = (size_t)dim * dim;
  const size_t lo_off = (size_t)NN * noe;  // the lo plane
  const size_t e = (size_t)gy * dim + gx;

  bool first = true;
  float beta_h = 0.f, beta_l = 0.f;  // beta (FP64) as a double-float coefficient
  int par = 0;
  if (MODE == APPLY_CG) {
    first = a.stp->first != 0;
    const double beta = a.stp->beta;
    beta_h = (float)beta;
    beta_l = (float)(beta - (double)beta_h);
    par = a.stp->parity;
  }
  const float* __restrict__ pold = par ? a.pbuf1 : a.pbuf0;
  float* __restrict__ pnew = par ? a.pbuf0 : a.pbuf1;
  // the input value of node k of element ee (CG: the new direction)
  auto ld = [&](int k, size_t ee) -> df {
    const size_t i = (size_t)k * noe + ee;
    const df r{__ldg(a.in + i), __ldg(a.in + lo_off + i)};
    if (MODE == APPLY_CG && !first) {
      const df po{__ldg(pold + i), __ldg(pold + lo_off + i)};
      return df_norm(df_mac2(r, beta_h, beta_l, po));
    }
    return r;
  };
  auto U = [&](int i1, int i2) -> df {
    const int k = (i1 * N1 + i2) * TE + t;
    return df{us[k], us[NN * TE + k]};
  };
  auto Uv = [&](int i1, int i2) -> df {
    const int k = (i1 * N1 + i2) * TE + t;
    return df{((volatile float*)us)[k], ((volatile float*)us)[NN * TE + k]};
  };
  auto XFr = [&](int row, int comp, int j, int fx) -> float& { return xf[((row * 4 + comp) * N1 + j) * (TX + 1) + fx]; };
  auto YFr = [&](int frow, int comp, int j, int col) -> float& { return yf[((frow * 4 + comp) * N1 + j) * TX + col]; };
  auto XF2 = [&](int row, int c0, int j, int fx) -> df { return df{XFr(row, c0, j, fx), XFr(row, c0 + 1, j, fx)}; };
  auto YF2 = [&](int frow, int c0, int j, int col) -> df { return df{YFr(frow, c0, j, col), YFr(frow, c0 + 1, j, col)}; };
  // J = kappa w (u0 - uN), Q = w (kappa (d0 + dN) + nu (u0 - uN)), kappa = 1/2 or 1
  auto combine = [&](int j, bool interior, df u0, df d0, df uN, df dN, df& J, df& Q) {
    const float kap = interior ? 0.5f : 1.f;
    const df jmp = df_add(u0, df_neg(uN));
    const df wj = df_mulc(tb.w[j], jmp);
    J = df{wj.hi * kap, wj.lo * kap};  // exact: kappa is a power of two
    df s = df_add(d0, dN);
    s = df{s.hi * kap, s.lo * kap};
    s = df_macc(s, cf{a.nu, a.nu_lo, a.nu_lo2}, jmp);  // the penalty, per operator
    Q = df_mulc(tb.w[j], s);
  };
  auto put = [&](float& h, float& l, df v) {
    h = v.hi;
    l = v.lo;
  };

  // ---- phase 0: nodal values of the tile's elements ------------------------
  // (loads only: CG mode writes the new direction in phase 2)
#pragma unroll(ApplyColumnForm<float, P>::load_unroll)
  for (int k = s; k < NN; k += TPE) {
    const df v = act ? ld(k, e) : df_zero();
    us[k * TE + t] = v.hi;
    us[NN * TE + k * TE + t] = v.lo;
  }
  __syncthreads();

  // ---- phase 1a: 0-side traces and derivatives -----------------------------
  if (act && xs) {
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      df d = df_zero();
#pragma unroll
      for (int i = 0; i < N1; ++i) d = df_macc(d, tb.D0[i], U(i, j));
      put(XFr(ty, 0, j, tx), XFr(ty, 1, j, tx), U(0, j));
      put(XFr(ty, 2, j, tx), XFr(ty, 3, j, tx), d);
    }
  }
  if (act && ys) {
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      df d = df_zero();
#pragma unroll
      for (int i = 0; i < N1; ++i) d = df_macc(d, tb.D0[i], U(j, i));
      put(YFr(ty + 1, 0, j, tx), YFr(ty + 1, 1, j, tx), U(j, 0));
      put(YFr(ty + 1, 2, j, tx), YFr(ty + 1, 3, j, tx), d);
    }
  }
  if (haloA) {  // halo above: its DOWN face
    const int hx = x0 + t;
    if (y0 > 0 && hx < dim) {
      const size_t he = (size_t)(y0 - 1) * dim + hx;
#pragma unroll 1
      for (int j = 0; j < N1; ++j) {
        df d = df_zero(), u0 = df_zero();
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const df v = ld(j * N1 + i, he);
          if (i == 0) u0 = v;
          d = df_macc(d, tb.D0[i], v);
        }
        put(YFr(0, 0, j, t), YFr(0, 1, j, t), u0);
        put(YFr(0, 2, j, t), YFr(0, 3, j, t), d);
      }
    }
  }
  if (haloB) {  // halo right: its LEFT face
    const int r = hb, hy = y0 + r, hx = x0 + TX;
    if (hx < dim && hy < dim) {
      const size_t he = (size_t)hy * dim + hx;
#pragma unroll 1
      for (int j = 0; j < N1; ++j) {
        df d = df_zero(), u0 = df_zero();
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const df v = ld(i * N1 + j, he);
          if (i == 0) u0 = v;
          d = df_macc(d, tb.D0[i], v);
        }
        put(XFr(r, 0, j, TX), XFr(r, 1, j, TX), u0);
        put(XFr(r, 2, j, TX), XFr(r, 3, j, TX), d);
      }
    }
  }
  __syncthreads();

  // ---- phase 1b: N-side combines (J, Q) ------------------------------------
  if (act && xs) {
    const bool rint = gx < dim - 1;
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      df dN = df_zero();
#pragma unroll
      for (int i = 0; i < N1; ++i) dN = df_macc(dN, tb.DN[i], U(i, j));
      const df u0 = rint ? XF2(ty, 0, j, tx + 1) : df_zero();
      const df d0 = rint ? XF2(ty, 2, j, tx + 1) : df_zero();
      df J, Q;
      combine(j, rint, u0, d0, U(N, j), dN, J, Q);
      put(XFr(ty, 0, j, tx + 1), XFr(ty, 1, j, tx + 1), J);
      put(XFr(ty, 2, j, tx + 1), XFr(ty, 3, j, tx + 1), Q);
    }
    if (gx == 0) {
#pragma unroll
      for (int j = 0; j < N1; ++j) {
        df J, Q;
        combine(j, false, XF2(ty, 0, j, tx), XF2(ty, 2, j, tx), df_zero(), df_zero(), J, Q);
        put(XFr(ty, 0, j, tx), XFr(ty, 1, j, tx), J);
        put(XFr(ty, 2, j, tx), XFr(ty, 3, j, tx), Q);
      }
    }
  }
  if (act && ys) {
    const bool uint_ = gy > 0;
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      df dN = df_zero();
#pragma unroll
      for (int i = 0; i < N1; ++i) dN = df_macc(dN, tb.DN[i], U(j, i));
      const df u0 = uint_ ? YF2(ty, 0, j, tx) : df_zero();
      const df d0 = uint_ ? YF2(ty, 2, j, tx) : df_zero();
      df J, Q;
      combine(j, uint_, u0, d0, U(j, N), dN, J, Q);
      put(YFr(ty, 0, j, tx), YFr(ty, 1, j, tx), J);
      put(YFr(ty, 2, j, tx), YFr(ty, 3, j, tx), Q);
    }
    if (gy == dim - 1) {
#pragma unroll
      for (int j = 0; j < N1; ++j) {
        df J, Q;
        combine(j, false, YF2(ty + 1, 0, j, tx), YF2(ty + 1, 2, j, tx), df_zero(), df_zero(), J, Q);
        put(YFr(ty + 1, 0, j, tx), YFr(ty + 1, 1, j, tx), J);
        put(YFr(ty + 1, 2, j, tx), YFr(ty + 1, 3, j, tx), Q);
      }
    }
  }
  if (haloA) {  // halo below: N-side of y face TY
    const int hx = x0 + t, hy = y0 + TY;
    if (hy < dim && hx < dim) {
      const size_t he = (size_t)hy * dim + hx;
#pragma unroll 1
      for (int j = 0; j < N1; ++j) {
        df dN = df_zero(), uN = df_zero();
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const df v = ld(j * N1 + i, he);
          if (i == N) uN = v;
          dN = df_macc(dN, tb.DN[i], v);
        }
        df J, Q;
        combine(j, true, YF2(TY, 0, j, t), YF2(TY, 2, j, t), uN, dN, J, Q);
        put(YFr(TY, 0, j, t), YFr(TY, 1, j, t), J);
        put(YFr(TY, 2, j, t), YFr(TY, 3, j, t), Q);
      }
    }
  }
  if (haloB) {  // halo left: N-side of x face 0
    const int r = hb, hy = y0 + r;
    if (x0 > 0 && hy < dim) {
      const size_t he = (size_t)hy * dim + (x0 - 1);
#pragma unroll 1
      for (int j = 0; j < N1; ++j) {
        df dN = df_zero(), uN = df_zero();
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const df v = ld(i * N1 + j, he);
          if (i == N) uN = v;
          dN = df_macc(dN, tb.DN[i], v);
        }
        df J, Q;
        combine(j, true, XF2(r, 0, j, 0), XF2(r, 2, j, 0), uN, dN, J, Q);
        put(XFr(r, 0, j, 0), XFr(r, 1, j, 0), J);
        put(XFr(r, 2, j, 0), XFr(r, 3, j, 0), Q);
      }
    }
  }
  __syncthreads();

  // ---- phase 2: outputs, one column at a time -------------------------------
  df dot = df_zero();
  if (act) {
#pragma unroll 1
    for (int i1 = s; i1 < N1; i1 += TPE) {
      constexpr bool kKw = DfKwForm<P>::value;
      const bool xf = (i1 == 0) || (i1 == N);
      // the node's face corrections (+-Q) as the seed of its chain: no
      // separate additions except at the corners
      auto seed_of = [&](int j) -> df {
        df seed = df_zero();
        if (i1 == 0) seed = XF2(ty, 2, j, tx);
        if (i1 == N) seed = df_neg(XF2(ty, 2, j, tx + 1));
        if (j == 0) seed = xf ? df_add(seed, YF2(ty + 1, 2, i1, tx)) : YF2(ty + 1, 2, i1, tx);
        if (j == N) seed = xf ? df_add(seed, df_neg(YF2(ty, 2, i1, tx))) : df_neg(YF2(ty, 2, i1, tx));
        return seed;
      };
      const cf d0i = tb.D0[i1], dni = tb.DN[i1], wi = tb.w[i1];
      df o[N1];
      if (kKw) {
        // KW form: seed, x-face lifting, sum_i w_j K(i1,i) u(i,j), then (below)
        // sum_i w_i1 K(j,i) u(i1,i) and the y-face lifting
#pragma unroll
        for (int j = 0; j < N1; ++j)
          o[j] = df_macc(df_macc(seed_of(j), dni, XF2(ty, 0, j, tx + 1)), d0i, XF2(ty, 0, j, tx));
#pragma unroll
        for (int i = 0; i < N1; ++i) {
#pragma unroll
          for (int j = 0; j < N1; ++j) o[j] = df_macc(o[j], tb.KW[kKw ? (i1 * N1 + i) * N1 + j : 0], Uv(i, j));
        }
      } else {
#pragma unroll
        for (int j = 0; j < N1; ++j) o[j] = df_zero();
#pragma unroll
        for (int i = 0; i < N1; ++i) {
          const cf kc = tb.K[i1 * N1 + i];
#pragma unroll
          for (int j = 0; j < N1; ++j) o[j] = df_macc(o[j], kc, Uv(i, j));
        }
      }
      df c[N1];
#pragma unroll
      for (int i = 0; i < N1; ++i) c[i] = U(i1, i);
      const df gJ = YF2(ty + 1, 0, i1, tx);
      const df hJ = YF2(ty, 0, i1, tx);
#pragma unroll
      for (int j = 0; j < N1; ++j) {
        df v;
        if (kKw) {
          v = o[j];
#pragma unroll
          for (int i = 0; i < N1; ++i) v = df_macc(v, tb.KW[kKw ? (j * N1 + i) * N1 + i1 : 0], c[i]);
        } else {
          // K form: w_j (K u)_j on the seed, the x-face lifting, w_i1 (K u)_i1
          df s = df_zero();
#pragma unroll
          for (int i = 0; i < N1; ++i) s = df_macc(s, tb.K[j * N1 + i], c[i]);
          v = df_macc(seed_of(j), tb.w[j], o[j]);
          v = df_macc(v, d0i, XF2(ty, 0, j, tx));
          v = df_macc(v, dni, XF2(ty, 0, j, tx + 1));
          v = df_macc(v, wi, s);
        }
        v = df_macc(v, tb.D0[j], gJ);
        v = df_macc(v, tb.DN[j], hJ);
        v = df_norm(v);
        const size_t oi = (size_t)(i1 * N1 + j) * noe + e;
        a.out[oi] = v.hi;
        a.out[lo_off + oi] = v.lo;
        if (MODE == APPLY_CG) {
          pnew[oi] = c[j].hi;
          pnew[lo_off + oi] = c[j].lo;
        }
        if (kReduce) dot = df_mac2(dot, c[j].hi, c[j].lo, v);
      }
    }
  }

  if (kReduce) {
    const double bt = block_sum<double, NT>((double)dot.hi + (double)dot.lo, red_sh);
    double total;
    if (grid_sum_last<double, NT>(bt, a.red, bid, nblocks, red_sh, &total) && lt == 0) {
      CgState<double>* st = a.stp;
      const double pAp = total;
      const double alpha = st->rr / pAp;
      st->pAp = pAp;
      st->alpha = alpha;
      if (MODE == APPLY_CG) st->parity = 1 - par;
      if (!(pAp > 0.0) || !isfinite(alpha)) {
        st->status = (int)SIPG_ERR_BREAKDOWN;
        st->done = 1;
      }
    }
  }
}

template <int P, int TX, int TY, int TPE, int MODE>
__global__ void __launch_bounds__(TX* TY* TPE)
    k_sipg_apply_df(const __grid_constant__ ApplyArgs<float> a, const __grid_constant__ TabDF<P> tb) {
  apply_tile_df<P, TX, TY, TPE, MODE>(a, tb, blockIdx.x, blockIdx.y, blockIdx.y * gridDim.x + blockIdx.x,
                                      gridDim.x * gridDim.y);
}

template <int P, int TX, int TY, int TPE, int MODE>
__global__ void __launch_bounds__(TX* TY* TPE)
    k_sipg_apply_df_batched(const ApplyArgs<float>* __restrict__ insts, const int* __restrict__ tile_start, int ninst,
                            const __grid_constant__ TabDF<P> tb) {
  const int g = blockIdx.x;
  int lo = 0, hi = ninst - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(tile_start + mid) <= g) lo = mid;
    else hi = mid - 1;
  }
  const ApplyArgs<float> a = insts[lo];
  const int lt = g - __ldg(tile_start + lo);
  const int tiles_x = (a.dim + TX - 1) / TX, tiles_y = (a.dim + TY - 1) / TY;
  apply_tile_df<P, TX, TY, TPE, MODE>(a, tb, lt % tiles_x, lt / tiles_x, lt, tiles_x * tiles_y);
}

// Launch (single operator when insts == nullptr, else batched over `ninst`
// operators of degree P; each carries its own penalty split into three floats).
template <int P, int TY, int TPE>
cudaError_t launch_apply_df_tile(int mode, const ApplyArgs<float>& a, const ApplyArgs<float>* insts,
                                 const int* tile_start, int ninst, int total_tiles, const TabDF<P>& tb,
                                 cudaStream_t s) {
  constexpr int TX = 32;
  const size_t smem = ApplyDfSmem<P, TX, TY>::bytes;
  cudaError_t err = cudaSuccess;
  const void* fns[6] = {(const void*)k_sipg_apply_df<P, TX, TY, TPE, APPLY_PLAIN>,
                        (const void*)k_sipg_apply_df<P, TX, TY, TPE, APPLY_CG>,
                        (const void*)k_sipg_apply_df<P, TX, TY, TPE, APPLY_DOT>,
                        (const void*)k_sipg_apply_df_batched<P, TX, TY, TPE, APPLY_PLAIN>,
                        (const void*)k_sipg_apply_df_batched<P, TX, TY, TPE, APPLY_CG>,
                        (const void*)k_sipg_apply_df_batched<P, TX, TY, TPE, APPLY_DOT>};
  for (const void* f : fns) {
    err = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
  }
  if (mode == APPLY_PREPARE) return cudaSuccess;
  const dim3 block(TX, TY, TPE);
  if (!insts) {
    const dim3 grid((a.dim + TX - 1) / TX, (a.dim + TY - 1) / TY);
    if (mode == APPLY_PLAIN) k_sipg_apply_df<P, TX, TY, TPE, APPLY_PLAIN><<<grid, block, smem, s>>>(a, tb);
    else if (mode == APPLY_CG) k_sipg_apply_df<P, TX, TY, TPE, APPLY_CG><<<grid, block, smem, s>>>(a, tb);
    else if (mode == APPLY_DOT) k_sipg_apply_df<P, TX, TY, TPE, APPLY_DOT><<<grid, block, smem, s>>>(a, tb);
    else return cudaErrorInvalidValue;
  } else {
    if (total_tiles == 0) return cudaSuccess;
    if (mode == APPLY_PLAIN)
      k_sipg_apply_df_batched<P, TX, TY, TPE, APPLY_PLAIN><<<total_tiles, block, smem, s>>>(insts, tile_start, ninst,
                                                                                             tb);
    else if (mode == APPLY_CG)
      k_sipg_apply_df_batched<P, TX, TY, TPE, APPLY_CG><<<total_tiles, block, smem, s>>>(insts, tile_start, ninst, tb);
    else if (mode == APPLY_DOT)
      k_sipg_apply_df_batched<P, TX, TY, TPE, APPLY_DOT><<<total_tiles, block, smem, s>>>(insts, tile_start, ninst,
                                                                                           tb);
    else return cudaErrorInvalidValue;
  }
  count_launch();
  return cudaGetLastError();
}

// Compiled shapes: rows TY in {2, 4, 8} with one thread per element, and TY in
// {2, 4} with two (TY = 8 x 2 would be 512 threads of ~100 registers).
template <int P>
cudaError_t launch_apply_df_p(const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const ApplyArgs<float>* insts,
                              const int* tile_start, int ninst, int total_tiles, const HostTables& h, cudaStream_t s) {
  const TabDF<P> tb = make_tab_df<P>(h);
  constexpr size_t kMax = 227 * 1024;
  constexpr bool fits8 = ApplyDfSmem<P, 32, 8>::bytes <= kMax;
  if (cfg.tpe == 2) {
    switch (cfg.ty) {
      case 2:
        return launch_apply_df_tile<P, 2, 2>(mode, a, insts, tile_start, ninst, total_tiles, tb, s);
      case 4:
        return launch_apply_df_tile<P, 4, 2>(mode, a, insts, tile_start, ninst, total_tiles, tb, s);
    }
    return cudaErrorInvalidConfiguration;
  }
  if (cfg.tpe != 1) return cudaErrorInvalidConfiguration;
  switch (cfg.ty) {
    case 2:
      return launch_apply_df_tile<P, 2, 1>(mode, a, insts, tile_start, ninst, total_tiles, tb, s);
    case 4:
      return launch_apply_df_tile<P, 4, 1>(mode, a, insts, tile_start, ninst, total_tiles, tb, s);
    case 8:
      if (!fits8) return cudaErrorInvalidConfiguration;
      return launch_apply_df_tile<P, (fits8 ? 8 : 4), 1>(mode, a, insts, tile_start, ninst, total_tiles, tb, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace sipg
