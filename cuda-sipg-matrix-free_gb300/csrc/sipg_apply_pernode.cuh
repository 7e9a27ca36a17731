// sipg_apply_pernode.cuh -- the FP64 apply for small meshes: one thread per
// output node.
//
// GB300 issues FP64 at a small fraction of its FP32 rate: a warp instruction of
// 32 DFMAs occupies a sub-partition's FP64 unit for tens of cycles.  The
// element-per-thread apply (sipg_apply.cuh) gives every thread the whole
// (p+1)^2-output chain of one element, so a mesh with few elements -- 256 at
// 16 x 16 -- runs a few warps, each through ~1000 dependent-issue DFMAs, on a
// handful of SMs: tens of microseconds per apply, whatever the tile shape.
// Here a CTA holds EX x EY elements and gives each output node its own thread:
// the same operations spread over (p+1)^2 times more warps, on more SMs.
//
// Each output is formed by exactly the operations, in exactly the order, of
// the element-per-thread kernel's column form (the FP64 form): one chain
// from the face nodes' +-Q and the x-face lifting through the weighted volume
// sums sum_i w_j K(i1,i) u(i,j) and sum_i w_i1 K(j,i) u(i1,i) to the y-face
// lifting.  Face
// values (J, Q) come from the same one-sided traces and derivatives combined
// by the same expression.  So the result is bit-identical to every other
// FP64 tile shape; only the CG reductions (p.Ap, r.r) group their partial
// sums differently.
//
// A CTA works through tiles blockIdx.x, blockIdx.x + gridDim.x, ... with the
// grid at most the resident CTAs, so a mesh of any size has at most a few
// thousand reduction partials.  Phases per tile (static shared memory, a few
// KB):
//   0  the tables, and the nodal blocks of the EX x EY elements and of the
//      2 (EX + EY) halo elements around them (from L2: small meshes live
//      there), with p = r + beta p_old formed on the fly in the CG mode;
//   1  one thread per face node: trace and normal derivative of each side,
//      combined into J and Q (both sides present inside the mesh, one side on
//      the domain boundary);
//   2  one thread per output node, then the epilogue (store, direction store
//      in the CG mode, deterministic grid reduction in the CG / DOT /
//      residual modes).
#pragma once

#include <algorithm>
#include <atomic>

#include "sipg_apply.cuh"

namespace sipg {

template <int P, int SHAPE>
struct PernodeShape {
  static constexpr int N1 = P + 1, NN = N1 * N1;
  static constexpr int EX = pernode_ex(P, SHAPE), EY = pernode_ey(P), NE = EX * EY;
  static constexpr int NT = (NE * NN + 31) / 32 * 32;  // threads: whole warps, the tail idle in phase 2
  static constexpr int SX = EX + 2, SY = EY + 2;       // element slots, halo ring included
  static constexpr int NX = EY * (EX + 1) * N1;        // x-face nodes: [EY][EX+1][N1]
  static constexpr int NY = EX * (EY + 1) * N1;        // y-face nodes: [EY+1][EX][N1]
};

// The CTA's shared memory: the nodal blocks of its tile and halo ring, the
// face values, and the tables.
template <typename T, int P, int SHAPE>
struct PernodeSmem {
  using S = PernodeShape<P, SHAPE>;
  T us[S::SX * S::SY * S::NN];  // slot (sy, sx) = element (y0 - 1 + sy, x0 - 1 + sx), values [i1 * N1 + i2]
  T xj[S::NX], xq[S::NX], yj[S::NY], yq[S::NY];
  T tw[S::N1], twh[S::N1], td0[S::N1], tdn[S::N1], tkw[S::NN * S::N1];
};

// The tables into shared memory (indexed per thread below: a constant-bank
// read whose address differs across the warp would serialise).  The caller
// synchronises before their first use.
template <typename T, int P, int SHAPE>
__device__ __forceinline__ void pernode_tables(PernodeSmem<T, P, SHAPE>& sm, const Tab<T, P>& tb) {
  using S = PernodeShape<P, SHAPE>;
  const int t = threadIdx.x;
  for (int k = t; k < S::NN * S::N1; k += S::NT) sm.tkw[k] = tb.KW[k];
  if (t < S::N1) {
    sm.tw[t] = tb.w[t];
    sm.twh[t] = tb.WH[t];
    sm.td0[t] = tb.D0[t];
    sm.tdn[t] = tb.DN[t];
  }
}

// One tile (origin x0, y0): phases 0-2, returning this thread's share of the
// reduction (p.Ap in the CG / DOT modes, r.r in the residual mode).
// kCoherent: read a.in and pold through L2 only -- for a caller that runs
// while other CTAs of the same grid write them (the persistent CG).
template <typename T, int P, int SHAPE, int MODE, bool kCoherent>
__device__ __forceinline__ T pernode_tile(const ApplyArgs<T>& a, PernodeSmem<T, P, SHAPE>& sm, int x0, int y0,
                                          bool first, T beta, const T* __restrict__ pold, T* __restrict__ pnew) {
  using S = PernodeShape<P, SHAPE>;
  constexpr int N = P, N1 = S::N1, NN = S::NN, EX = S::EX, NE = S::NE, NT = S::NT;
  constexpr int SX = S::SX, SY = S::SY, NX = S::NX, NY = S::NY, NSLOT = SX * SY;
  constexpr bool kDot = (MODE == APPLY_CG || MODE == APPLY_DOT);
  T* __restrict__ us = sm.us;
  T* __restrict__ xj = sm.xj;
  T* __restrict__ xq = sm.xq;
  T* __restrict__ yj = sm.yj;
  T* __restrict__ yq = sm.yq;
  const T* __restrict__ tw = sm.tw;
  const T* __restrict__ twh = sm.twh;
  const T* __restrict__ td0 = sm.td0;
  const T* __restrict__ tdn = sm.tdn;
  const T* __restrict__ tkw = sm.tkw;
  const int t = threadIdx.x;
  const int dim = a.dim;
  const size_t noe = (size_t)dim * dim;
  const T nu = a.nu;
  auto ldin = [&](const T* p) -> T { return kCoherent ? __ldcg(p) : __ldg(p); };
  T acc = T(0);
  // ---- phase 0: nodal blocks ------------------------------------------------
  for (int idx = t; idx < NSLOT * NN; idx += NT) {
    const int k = idx / NSLOT, sl = idx - k * NSLOT;
    const int sy = sl / SX, sx = sl - sy * SX;
    const int gx = x0 - 1 + sx, gy = y0 - 1 + sy;
    const bool corner = (sx == 0 || sx == SX - 1) && (sy == 0 || sy == SY - 1);
    T v = T(0);
    if (!corner && gx >= 0 && gx < dim && gy >= 0 && gy < dim) {
      const size_t gk = (size_t)k * noe + (size_t)gy * dim + gx;
      v = ldin(a.in + gk);
      if (MODE == APPLY_CG && !first) v = fma(beta, ldin(pold + gk), v);
    }
    us[sl * NN + k] = v;
  }
  __syncthreads();

  // ---- phase 1: J and Q of every face node of the tile -----------------------
  for (int f = t; f < NX + NY; f += NT) {
    T u0 = T(0), d0 = T(0), uN = T(0), dN = T(0);
    bool zv, nv;  // 0-side / N-side element inside the mesh
    int j;
    if (f < NX) {
      // x face fx of tile row ey: the left element (slot fx) is its N-side
      // (i1 = P), the right element (slot fx + 1) its 0-side (i1 = 0)
      j = f % N1;
      const int r = f / N1, fx = r % (EX + 1), ey = r / (EX + 1);
      const int gy = y0 + ey, gxl = x0 + fx - 1;
      nv = gy < dim && gxl >= 0 && gxl < dim;
      zv = gy < dim && gxl + 1 < dim;
      const T* L = us + ((ey + 1) * SX + fx) * NN;
      const T* R = L + NN;
      if (zv) {
        u0 = R[j];
#pragma unroll
        for (int i = 0; i < N1; ++i) d0 = fma(td0[i], R[i * N1 + j], d0);
      }
      if (nv) {
        uN = L[N * N1 + j];
#pragma unroll
        for (int i = 0; i < N1; ++i) dN = fma(tdn[i], L[i * N1 + j], dN);
      }
    } else {
      // y face fy of tile column ex: the upper element (slot row fy) is its
      // 0-side (i2 = 0), the lower element (slot row fy + 1) its N-side (i2 = P)
      const int g = f - NX;
      j = g % N1;
      const int r = g / N1, ex = r % EX, fy = r / EX;
      const int gx = x0 + ex, gyu = y0 + fy - 1;
      zv = gx < dim && gyu >= 0 && gyu < dim;
      nv = gx < dim && gyu + 1 < dim;
      const T* Up = us + (fy * SX + ex + 1) * NN;
      const T* Dn = Up + SX * NN;
      if (zv) {
        u0 = Up[j * N1];
#pragma unroll
        for (int i = 0; i < N1; ++i) d0 = fma(td0[i], Up[j * N1 + i], d0);
      }
      if (nv) {
        uN = Dn[j * N1 + N];
#pragma unroll
        for (int i = 0; i < N1; ++i) dN = fma(tdn[i], Dn[j * N1 + i], dN);
      }
    }
    T J, Q;
    face_combine<T>(tw[j], twh[j], nu, zv && nv, u0, d0, uN, dN, J, Q);
    if (f < NX) {
      xj[f] = J;
      xq[f] = Q;
    } else {
      yj[f - NX] = J;
      yq[f - NX] = Q;
    }
  }
  __syncthreads();

  // ---- phase 2: one output node per thread ------------------------------------
  if (t < NE * NN) {
    const int le = t % NE, k = t / NE;  // element fastest: neighbouring threads store neighbouring elements
    const int ex = le % EX, ey = le / EX;
    const int i1 = k / N1, j = k - i1 * N1;
    const int gx = x0 + ex, gy = y0 + ey;
    if (gx < dim && gy < dim) {
      const T* E = us + ((ey + 1) * SX + ex + 1) * NN;
      const int fl = (ey * (EX + 1) + ex) * N1;  // left x face; the right one is fl + N1
      const int fd = ((ey + 1) * EX + ex) * N1;  // down y face; the up one is fd - EX * N1
      const int fu = fd - EX * N1;
      const bool xf = (i1 == 0) || (i1 == N);
      const T seed = face_seed<T, N>(i1, j, xf ? xq[fl + j] : T(0), xf ? xq[fl + N1 + j] : T(0),
                                     (j == 0) ? yq[fd + i1] : T(0), (j == N) ? yq[fu + i1] : T(0));
      T v = fma(td0[i1], xj[fl + j], fma(tdn[i1], xj[fl + N1 + j], seed));
#pragma unroll
      for (int i = 0; i < N1; ++i) v = fma(tkw[(i1 * N1 + i) * N1 + j], E[i * N1 + j], v);
#pragma unroll
      for (int i = 0; i < N1; ++i) v = fma(tkw[(j * N1 + i) * N1 + i1], E[i1 * N1 + i], v);
      v = fma(td0[j], yj[fd + i1], v);
      v = fma(tdn[j], yj[fu + i1], v);
      const size_t gk = (size_t)k * noe + (size_t)gy * dim + gx;
      if (MODE == APPLY_RESID) {
        const T rv = __ldg(a.b + gk) - v;
        a.out[gk] = rv;
        acc = fma(rv, rv, acc);
      } else {
        a.out[gk] = v;
        const T c = E[k];
        if (MODE == APPLY_CG) pnew[gk] = c;
        if (kDot) acc = fma(c, v, acc);
      }
    }
  }
  __syncthreads();  // the next tile overwrites the shared memory
  return acc;
}

template <typename T, int P, int SHAPE, int MODE>
__global__ void __launch_bounds__(PernodeShape<P, SHAPE>::NT)
    k_sipg_apply_pernode(const __grid_constant__ ApplyArgs<T> a, const __grid_constant__ Tab<T, P> tb) {
  using S = PernodeShape<P, SHAPE>;
  constexpr int EX = S::EX, EY = S::EY, NT = S::NT;
  __shared__ PernodeSmem<T, P, SHAPE> sm;
  __shared__ T red_sh[32];

  constexpr bool kDot = (MODE == APPLY_CG || MODE == APPLY_DOT);
  if (kDot) {
    if (*(volatile int*)&a.st->done) return;  // converged: the launch is a no-op
  }
  const int t = threadIdx.x;
  const int dim = a.dim;
  const int rows = a.nrows > 0 ? a.nrows : dim;  // a band of element rows from a.row0
  const int tiles_x = (dim + EX - 1) / EX, ntiles = tiles_x * ((rows + EY - 1) / EY);

  bool first = true;
  T beta = T(0);
  int par = 0;
  if (MODE == APPLY_CG) {
    first = a.st->first != 0;
    beta = a.st->beta;
    par = a.st->parity;
  }
  const T* __restrict__ pold = par ? a.pbuf1 : a.pbuf0;
  T* __restrict__ pnew = par ? a.pbuf0 : a.pbuf1;
  pernode_tables<T, P, SHAPE>(sm, tb);
  T acc = T(0);
  // the CTA's tiles: blockIdx.x, + gridDim.x, ... (the grid is at most the
  // resident CTAs, so the reduction has few partials on any mesh)
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int x0 = (tile % tiles_x) * EX, y0 = a.row0 + (tile / tiles_x) * EY;
    acc += pernode_tile<T, P, SHAPE, MODE, false>(a, sm, x0, y0, first, beta, pold, pnew);
  }

  if (MODE != APPLY_PLAIN) {
    const T bt = block_sum<T, NT>(acc, red_sh);
    T total;
    if (grid_sum_last<T, NT>(bt, a.red, (int)blockIdx.x, (int)gridDim.x, red_sh, &total) && t == 0)
      apply_finish<T, MODE>(a.st, total, par);
  }
}

// Resident CTAs of a per-node kernel on the current device (occupancy x SMs),
// computed once per kernel.
template <typename K>
int pernode_resident_blocks(K kernel, int threads) {
  static std::atomic<int> cached{0};
  int v = cached.load(std::memory_order_relaxed);
  if (v > 0) return v;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return 152;  // one CTA per SM of a GB300
  }
  v = sms * per_sm;
  cached.store(v, std::memory_order_relaxed);
  return v;
}

template <typename T, int P, int SHAPE>
cudaError_t launch_apply_pernode_shape(int mode, const ApplyArgs<T>& a, const Tab<T, P>& tb, cudaStream_t s) {
  using S = PernodeShape<P, SHAPE>;
  if (mode == APPLY_PREPARE) return cudaSuccess;  // static shared memory: no attribute to set
  const int rows = a.nrows > 0 ? a.nrows : a.dim;
  const long long ntiles = (long long)((a.dim + S::EX - 1) / S::EX) * ((rows + S::EY - 1) / S::EY);
  // at most the resident CTAs, and in a reducing mode at most one partial per
  // scratch entry
  auto grid_for = [&](auto kernel, bool reduces) {
    long long g = std::min<long long>(ntiles, pernode_resident_blocks(kernel, S::NT));
    if (reduces) g = std::min<long long>(g, a.red.capacity);
    return (int)std::max<long long>(g, 1);
  };
  const dim3 block(S::NT);
  switch (mode) {
    case APPLY_PLAIN: {
      auto k = k_sipg_apply_pernode<T, P, SHAPE, APPLY_PLAIN>;
      k<<<grid_for(k, false), block, 0, s>>>(a, tb);
      break;
    }
    case APPLY_CG: {
      auto k = k_sipg_apply_pernode<T, P, SHAPE, APPLY_CG>;
      k<<<grid_for(k, true), block, 0, s>>>(a, tb);
      break;
    }
    case APPLY_RESID: {
      auto k = k_sipg_apply_pernode<T, P, SHAPE, APPLY_RESID>;
      k<<<grid_for(k, true), block, 0, s>>>(a, tb);
      break;
    }
    case APPLY_DOT: {
      auto k = k_sipg_apply_pernode<T, P, SHAPE, APPLY_DOT>;
      k<<<grid_for(k, true), block, 0, s>>>(a, tb);
      break;
    }
    default:
      return cudaErrorInvalidValue;
  }
  count_launch();
  return cudaGetLastError();
}

// The per-node tile named by cfg (tpe = (p+1)^2; tx x ty one of the two
// compiled shapes).
template <typename T, int P>
cudaError_t launch_apply_pernode(const TileCfg& cfg, int mode, const ApplyArgs<T>& a, const HostTables& h,
                                 cudaStream_t s) {
  if (cfg.ty != pernode_ey(P)) return cudaErrorInvalidConfiguration;
  const Tab<T, P> tb = make_tab<T, P>(h);
  if (cfg.tx == pernode_ex(P, 0)) return launch_apply_pernode_shape<T, P, 0>(mode, a, tb, s);
  if (cfg.tx == pernode_ex(P, 1)) return launch_apply_pernode_shape<T, P, 1>(mode, a, tb, s);
  return cudaErrorInvalidConfiguration;
}

}  // namespace sipg
