// twolevel.cu -- the two-level preconditioner of the mixed-precision inner
// solve (no counterpart in the reference):
//
//   z = B^-1 r + P V(P^T r)
//
// B^-1: exact element block-Jacobi.  The diagonal block of an element
//   depends only on which of its four faces lie on the domain boundary, so a
//   mesh has at most nine distinct blocks (one for dim = 1, four for dim = 2);
//   they are probed from the FP64 operator on a mesh of min(dim, 3) elements
//   per side (checkerboard colouring: face neighbours never share a probe) and
//   inverted on the host.
// P: the continuous bilinear (Q1) functions on the (dim + 1)^2 element
//   vertices, sampled at each element's LGL nodes; P^T r sums each vertex's
//   hat function against r over the (up to four) elements around it.
// V: one symmetric multigrid V-cycle on the Q1 vertex grid for the coarse
//   operator A_0 = P^T A P (probed from the FP64 operator with nine colours
//   of vertices -- its stencil is 9-point), Galerkin levels A_{l+1} =
//   P_l^T A_l P_l down to at most kTlCoarsestCells cells per side (built on
//   the host; a level of m cells goes to ceil(m/2), odd m with one coarse
//   cell of a single fine cell at its end), two damped-Jacobi sweeps before
//   and after each coarse correction, the coarsest level by its dense
//   inverse.
//
// The block part removes the degree's share of the condition number, the
// coarse part the mesh size's: CG iterations stay flat in dim (measured with
// a CPU restatement, FP64, pen p^2, 16^2..64^2: p = 2: 24, 4: 41-44, 6:
// 59-62, 8: 76-79, against 119-376 for plain CG at p = 4, 6).  That is what
// lets the inner solve run in FP32: unpreconditioned, kappa ~ 2e7 at 512^2,
// p = 6 and FP32 CG (kappa eps_32 ~ 1) needs ~2,000 iterations to reduce its
// residual 100-fold.
//
// The kernels are templates on the value type: the inner solve runs the
// float ones; the set-up probes with the double ones.
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <vector>

#include "sipg_cg.cuh"
#include "sipg_twolevel.cuh"

using namespace sipg;

namespace sipg {

constexpr int kTlElemThreads = 64;  // element kernels: one thread per element
constexpr int kTlVecThreads = 256;  // vertex kernels: one thread per vertex
constexpr int kTlCoarsestCells = 8; // coarsen while a level has more cells per side
constexpr int kTlTypes = 16;        // element types: bit 0 LEFT, 1 RIGHT, 2 DOWN, 3 UP face on the boundary

// Element type of element (row, col): which faces are on the domain boundary
// (row 0 is the top row, so its UP face is).
__host__ __device__ inline int tl_elem_type(int row, int col, int dim) {
  return (col == 0 ? 1 : 0) | (col == dim - 1 ? 2 : 0) | (row == dim - 1 ? 4 : 0) | (row == 0 ? 8 : 0);
}

// 1-D interpolation weight of fine vertex i (of a level with m cells) from
// coarse vertex J: the coarse vertices sit at the even fine vertices and at
// m; an odd fine vertex other than m is the midpoint of its two neighbours.
template <typename T>
__host__ __device__ inline T tl_w(int i, int J, int m) {
  if (i % 2 == 0 || i == m) return ((i + 1) / 2 == J) ? T(1) : T(0);
  return (J == (i - 1) / 2 || J == (i + 1) / 2) ? T(0.5) : T(0);
}

// The element's bilinear hat functions at its LGL nodes: l[a][i] = (1 -+ x_i) / 2.
template <typename T, int P>
struct TlHat {
  T l[2][P + 1];
};

__device__ __forceinline__ bool tl_done(const int* done) { return done && *(volatile const int*)done; }

template <typename T>
__device__ __forceinline__ T tl_stencil(const TlLev<T>& L, const T* __restrict__ x, int vx, int vy) {
  const int n1 = L.m + 1, nv = n1 * n1, v = vy * n1 + vx;
  T s = T(0);
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx) {
      const int ux = vx + dx, uy = vy + dy;
      if (ux < 0 || uy < 0 || ux > L.m || uy > L.m) continue;
      s = fma(L.S[((dy + 1) * 3 + (dx + 1)) * nv + v], x[uy * n1 + ux], s);
    }
  return s;
}

// ---- the DG <-> Q1 transfers (one thread per element, 64 per block) ----

// corner sums cp[(a * 2 + b) * noe + e] = sum_{i1,i2} l_a(x_i1) l_b(x_i2) r(i1,i2,e)
template <typename T, int P>
__device__ __forceinline__ void tl_restrict_elem_body(const T* __restrict__ r, T* __restrict__ cp, size_t noe,
                                                      const TlHat<T, P>& h, int bid, int nb) {
  constexpr int N1 = P + 1;
  for (size_t e = (size_t)bid * blockDim.x + threadIdx.x; e < noe; e += (size_t)nb * blockDim.x) {
    T c00 = T(0), c01 = T(0), c10 = T(0), c11 = T(0);
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      T s0 = T(0), s1 = T(0);
#pragma unroll
      for (int i2 = 0; i2 < N1; ++i2) {
        const T v = __ldg(r + (size_t)(i1 * N1 + i2) * noe + e);
        s0 = fma(h.l[0][i2], v, s0);
        s1 = fma(h.l[1][i2], v, s1);
      }
      c00 = fma(h.l[0][i1], s0, c00);
      c01 = fma(h.l[0][i1], s1, c01);
      c10 = fma(h.l[1][i1], s0, c10);
      c11 = fma(h.l[1][i1], s1, c11);
    }
    cp[0 * noe + e] = c00;
    cp[1 * noe + e] = c01;
    cp[2 * noe + e] = c10;
    cp[3 * noe + e] = c11;
  }
}

template <typename T, int P>
__global__ void __launch_bounds__(kTlElemThreads)
    k_tl_restrict_elem(const T* __restrict__ r, T* __restrict__ cp, size_t noe, const __grid_constant__ TlHat<T, P> h,
                       const int* done) {
  if (tl_done(done)) return;
  tl_restrict_elem_body<T, P>(r, cp, noe, h, blockIdx.x, gridDim.x);
}

// The inner PCG update fused with the restriction of the new residual, one
// thread per element: x += alpha p, r -= alpha Ap (p: pb1 if the state's
// parity is 1, else pb0), r.r and the stop test, and the corner sums cp of
// the new r that the next z = M r starts from.
template <int P>
__device__ __forceinline__ void tl_update_restrict_body(float* __restrict__ x, const float* __restrict__ pb0,
                                                        const float* __restrict__ pb1, float* __restrict__ r,
                                                        const float* __restrict__ Ap, float* __restrict__ cp, size_t noe,
                                                        CgState<float>* st, const ReduceScratch& red,
                                                        const TlHat<float, P>& h, int bid, int nb) {
  constexpr int N1 = P + 1;
  __shared__ float sh[32];
  if (*(volatile int*)&st->done) return;
  const float alpha = st->alpha;
  const float* __restrict__ p = st->parity ? pb1 : pb0;
  float acc = 0.f;
  for (size_t e = (size_t)bid * blockDim.x + threadIdx.x; e < noe; e += (size_t)nb * blockDim.x) {
    float c00 = 0.f, c01 = 0.f, c10 = 0.f, c11 = 0.f;
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1) {
      // a row of nodes: every load first, so that they are in flight together
      float xv[N1], pv[N1], rv[N1], av[N1];
#pragma unroll
      for (int i2 = 0; i2 < N1; ++i2) {
        const size_t g = (size_t)(i1 * N1 + i2) * noe + e;
        xv[i2] = x[g];
        pv[i2] = p[g];
        rv[i2] = r[g];
        av[i2] = Ap[g];
      }
      float s0 = 0.f, s1 = 0.f;
#pragma unroll
      for (int i2 = 0; i2 < N1; ++i2) {
        const size_t g = (size_t)(i1 * N1 + i2) * noe + e;
        x[g] = fmaf(alpha, pv[i2], xv[i2]);
        const float ri = fmaf(-alpha, av[i2], rv[i2]);
        r[g] = ri;
        acc = fmaf(ri, ri, acc);
        s0 = fmaf(h.l[0][i2], ri, s0);
        s1 = fmaf(h.l[1][i2], ri, s1);
      }
      c00 = fmaf(h.l[0][i1], s0, c00);
      c01 = fmaf(h.l[0][i1], s1, c01);
      c10 = fmaf(h.l[1][i1], s0, c10);
      c11 = fmaf(h.l[1][i1], s1, c11);
    }
    cp[0 * noe + e] = c00;
    cp[1 * noe + e] = c01;
    cp[2 * noe + e] = c10;
    cp[3 * noe + e] = c11;
  }
  const float bt = block_sum<float, kTlElemThreads>(acc, sh);
  float total;
  if (grid_sum_last<float, kTlElemThreads>(bt, red, bid, nb, sh, &total) && threadIdx.x == 0)
    pcg_update_bookkeep<float>(st, total);
}

template <int P>
__global__ void __launch_bounds__(kTlElemThreads)
    k_tl_update_restrict(float* __restrict__ x, const float* __restrict__ pb0, const float* __restrict__ pb1,
                         float* __restrict__ r, const float* __restrict__ Ap, float* __restrict__ cp, size_t noe,
                         CgState<float>* st, ReduceScratch red, const __grid_constant__ TlHat<float, P> h) {
  tl_update_restrict_body<P>(x, pb0, pb1, r, Ap, cp, noe, st, red, h, blockIdx.x, gridDim.x);
}

// b0 at vertex (vx, vy): the corner sums of the elements around it, in a fixed order
template <typename T>
__device__ __forceinline__ T tl_corner_sum(const T* __restrict__ cp, int dim, int vx, int vy) {
  const size_t noe = (size_t)dim * dim;
  T acc = T(0);
#pragma unroll
  for (int R = vy - 1; R <= vy; ++R) {  // element rows counted bottom-up
    if (R < 0 || R >= dim) continue;
#pragma unroll
    for (int col = vx - 1; col <= vx; ++col) {
      if (col < 0 || col >= dim) continue;
      const size_t e = (size_t)(dim - 1 - R) * dim + col;
      const int a = vx - col, b = vy - R;
      acc += __ldg(cp + (size_t)(a * 2 + b) * noe + e);
    }
  }
  return acc;
}

// b0 = the vertex sums of the corner sums (used by the set-up's probing)
template <typename T>
__global__ void __launch_bounds__(kTlVecThreads)
    k_tl_restrict_vert(const T* __restrict__ cp, T* __restrict__ b0, int dim) {
  const int n1 = dim + 1, v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n1 * n1) b0[v] = tl_corner_sum(cp, dim, v % n1, v / n1);
}

// out = P xv: the Q1 function of vertex values xv at every element's nodes
template <typename T, int P>
__global__ void __launch_bounds__(kTlElemThreads)
    k_tl_prolong(const T* __restrict__ xv, T* __restrict__ out, int dim, const __grid_constant__ TlHat<T, P> h) {
  constexpr int N1 = P + 1;
  const size_t noe = (size_t)dim * dim;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < noe; e += (size_t)gridDim.x * blockDim.x) {
    const int row = (int)(e / dim), col = (int)(e % dim), R = dim - 1 - row;
    const T x00 = xv[R * (dim + 1) + col], x10 = xv[R * (dim + 1) + col + 1];
    const T x01 = xv[(R + 1) * (dim + 1) + col], x11 = xv[(R + 1) * (dim + 1) + col + 1];
#pragma unroll
    for (int i1 = 0; i1 < N1; ++i1)
#pragma unroll
      for (int i2 = 0; i2 < N1; ++i2)
        out[(size_t)(i1 * N1 + i2) * noe + e] =
            h.l[0][i1] * (h.l[0][i2] * x00 + h.l[1][i2] * x01) + h.l[1][i1] * (h.l[0][i2] * x10 + h.l[1][i2] * x11);
  }
}

// ---- the V-cycle on the vertex grid ----
//
// Per level: b the right-hand side, x the pre-smoothed iterate, y the
// V-cycle result.  The vertex kernels are latency bound (a level-0 grid of
// (dim + 1)^2 vertices is a few MB), so each level takes one fused kernel on
// the way down and one on the way up, each block working on a square tile of
// vertices through shared-memory windows that hold zero outside the level.

constexpr int kTlDown = 16;          // coarse vertices per side of a down tile
constexpr int kTlUp = 32;            // fine vertices per side of an up tile
constexpr int kTlTileThreads = 256;  // threads of the tile kernels
constexpr int kTlTailCells = 32;     // levels of at most this many cells per side run in one block
constexpr int kTlTailThreads = 1024;

// The vertex kernels wait on memory, not arithmetic: each pass of a tile
// kernel first loads what every one of its thread's steps needs (stencil
// rows, weights, right-hand sides) and only then computes, so that all of a
// thread's loads are in flight together.
template <int N>
__host__ __device__ constexpr int tl_steps() {
  return (N + kTlTileThreads - 1) / kTlTileThreads;
}

// A vertex's stencil row (S[k] = entry k of its 9-point row), damping and
// right-hand side.
template <typename T>
struct TlRow {
  T S[9];
  T wd, b;
};

template <typename T>
__device__ __forceinline__ void tl_load_row(const TlLev<T>& L, int v, int nv, bool ok, bool with_b, TlRow<T>& r) {
#pragma unroll
  for (int k = 0; k < 9; ++k) r.S[k] = ok ? __ldg(L.S + (size_t)k * nv + v) : T(0);
  r.wd = ok ? __ldg(L.wd + v) : T(0);
  r.b = (ok && with_b) ? __ldg(L.b + v) : T(0);
}

// The row applied to the 3 x 3 patch of window w around the vertex (w points
// at the patch's corner [0][0], row stride W).
template <typename T, int W>
__device__ __forceinline__ T tl_row_apply(const TlRow<T>& r, const T* w) {
  T s = T(0);
#pragma unroll
  for (int dy = 0; dy < 3; ++dy)
#pragma unroll
    for (int dx = 0; dx < 3; ++dx) s = fma(r.S[dy * 3 + dx], w[dy * W + dx], s);
  return s;
}

// One down step for the 16 x 16 tile (tx, ty) of coarse vertices: on the
// fine level F (with cp: b from the element corner sums, level 0)
//   x1 = wd b,   x = x1 + wd (b - A x1)   (two damped-Jacobi sweeps from zero),
// then C.b = P^T (b - A x).  The tile's fine footprint is [2 cx0 - 1,
// 2 cx0 + 31]^2; x is needed one vertex beyond it, b and x1 two.  The block
// writes x (and, from cp, b) at the fine vertices [2 cx0, 2 cx0 + 32)^2 it
// owns; every fine vertex has exactly one owner.
template <typename T>
__device__ __forceinline__ void tl_down_body(const TlLev<T>& F, const TlLev<T>& C, const T* __restrict__ cp, int dim,
                                             int tx, int ty) {
  constexpr int W3 = 2 * kTlDown + 5, W2 = W3 - 2, W1 = W3 - 4;  // 37, 35, 33
  __shared__ T sb[W3][W3], sx1[W3][W3], sx[W2][W2], sr[W1][W1];
  const int m = F.m, n1 = m + 1, nv = n1 * n1, t = threadIdx.x;
  const int cx0 = tx * kTlDown, cy0 = ty * kTlDown;
  const int ox = 2 * cx0 - 3, oy = 2 * cy0 - 3;  // fine vertex of window entry [0][0] of sb
  auto owned = [&](int ix, int iy) {
    return ix >= 2 * cx0 && ix < 2 * cx0 + 2 * kTlDown && iy >= 2 * cy0 && iy < 2 * cy0 + 2 * kTlDown;
  };
  auto inside = [&](int ix, int iy) { return ix >= 0 && iy >= 0 && ix <= m && iy <= m; };
  {  // b and x1 on the W3 window
    constexpr int NS = tl_steps<W3 * W3>();
    T b[NS], w[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W3, lx = i - ly * W3, ix = ox + lx, iy = oy + ly;
      const bool ok = i < W3 * W3 && inside(ix, iy);
      const int v = ok ? iy * n1 + ix : 0;
      b[k] = ok ? (cp ? tl_corner_sum(cp, dim, ix, iy) : __ldg(F.b + v)) : T(0);
      w[k] = ok ? __ldg(F.wd + v) : T(0);
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W3, lx = i - ly * W3;
      if (i >= W3 * W3) break;
      sb[ly][lx] = b[k];
      sx1[ly][lx] = w[k] * b[k];
      if (cp && inside(ox + lx, oy + ly) && owned(ox + lx, oy + ly)) F.b[(oy + ly) * n1 + ox + lx] = b[k];
    }
  }
  __syncthreads();
  {  // x on the W2 window
    constexpr int NS = tl_steps<W2 * W2>();
    TlRow<T> r[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W2, lx = i - ly * W2, ix = ox + 1 + lx, iy = oy + 1 + ly;
      const bool ok = i < W2 * W2 && inside(ix, iy);
      tl_load_row(F, ok ? iy * n1 + ix : 0, nv, ok, false, r[k]);
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W2, lx = i - ly * W2, ix = ox + 1 + lx, iy = oy + 1 + ly;
      if (i >= W2 * W2) break;
      // outside the level the row is zero and so is x
      const T x = fma(r[k].wd, sb[ly + 1][lx + 1] - tl_row_apply<T, W3>(r[k], &sx1[ly][lx]), sx1[ly + 1][lx + 1]);
      sx[ly][lx] = x;
      if (inside(ix, iy) && owned(ix, iy)) F.x[iy * n1 + ix] = x;
    }
  }
  __syncthreads();
  {  // the residual on the footprint (W1 window)
    constexpr int NS = tl_steps<W1 * W1>();
    TlRow<T> r[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W1, lx = i - ly * W1, ix = ox + 2 + lx, iy = oy + 2 + ly;
      const bool ok = i < W1 * W1 && inside(ix, iy);
      tl_load_row(F, ok ? iy * n1 + ix : 0, nv, ok, false, r[k]);
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W1, lx = i - ly * W1, ix = ox + 2 + lx, iy = oy + 2 + ly;
      if (i >= W1 * W1) break;
      sr[ly][lx] = inside(ix, iy) ? sb[ly + 2][lx + 2] - tl_row_apply<T, W2>(r[k], &sx[ly][lx]) : T(0);
    }
  }
  __syncthreads();
  const int J = cx0 + t % kTlDown, I = cy0 + t / kTlDown;
  if (J > C.m || I > C.m) return;
  T acc = T(0);
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy) {
    const int iy = 2 * I + dy;
    if (iy < 0 || iy > m) continue;
    const T wy = tl_w<T>(iy, I, m);
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx) {
      const int ix = 2 * J + dx;
      if (ix < 0 || ix > m) continue;
      acc = fma(wy * tl_w<T>(ix, J, m), sr[iy - oy - 2][ix - ox - 2], acc);
    }
  }
  C.b[I * (C.m + 1) + J] = acc;
}

// The prolongation of the coarse result at fine vertex (ux, uy): the coarse
// vertices it lies between, (jx0, jx1) x (jy0, jy1), and its weights.
struct TlProlong {
  int jx0, jx1, jy0, jy1;
  bool px, py;  // on a coarse vertex line in x, in y
};
__device__ __forceinline__ TlProlong tl_prolong_at(int ux, int uy, int m) {
  TlProlong q;
  q.px = (ux % 2 == 0) || (ux == m);
  q.py = (uy % 2 == 0) || (uy == m);
  q.jx0 = q.px ? (ux + 1) / 2 : (ux - 1) / 2;
  q.jx1 = q.px ? q.jx0 : (ux + 1) / 2;
  q.jy0 = q.py ? (uy + 1) / 2 : (uy - 1) / 2;
  q.jy1 = q.py ? q.jy0 : (uy + 1) / 2;
  return q;
}
// c = [c00 c01; c10 c11] (c_ab at (jy_a, jx_b)) combined with the weights
template <typename T>
__device__ __forceinline__ T tl_prolong_value(const TlProlong& q, T c00, T c01, T c10, T c11) {
  if (q.px && q.py) return c00;
  if (q.px) return T(0.5) * (c00 + c10);
  if (q.py) return T(0.5) * (c00 + c01);
  return T(0.25) * ((c00 + c01) + (c10 + c11));
}

// The pre-smoothed iterate plus the prolonged coarse result at fine vertex (ux, uy).
template <typename T>
__device__ __forceinline__ T tl_corrected(const TlLev<T>& F, const TlLev<T>& C, int ux, int uy) {
  const int cn1 = C.m + 1;
  const TlProlong q = tl_prolong_at(ux, uy, F.m);
  return F.x[uy * (F.m + 1) + ux] + tl_prolong_value(q, C.y[q.jy0 * cn1 + q.jx0], C.y[q.jy0 * cn1 + q.jx1],
                                                      C.y[q.jy1 * cn1 + q.jx0], C.y[q.jy1 * cn1 + q.jx1]);
}

// One up step for the 32 x 32 tile (tx, ty) of fine vertices: with
// xc = x + P C.y, two damped-Jacobi sweeps
//   y1 = xc + wd (b - A xc),   F.y = y1 + wd (b - A y1).
template <typename T>
__device__ __forceinline__ void tl_up_body(const TlLev<T>& F, const TlLev<T>& C, int tx, int ty) {
  constexpr int W2 = kTlUp + 4, W1 = kTlUp + 2;  // 36, 34
  __shared__ T sxc[W2][W2], sy[W1][W1];
  const int m = F.m, n1 = m + 1, nv = n1 * n1, cn1 = C.m + 1, t = threadIdx.x;
  const int fx0 = tx * kTlUp, fy0 = ty * kTlUp;
  const int ox = fx0 - 2, oy = fy0 - 2;  // fine vertex of window entry [0][0] of sxc
  auto inside = [&](int ix, int iy) { return ix >= 0 && iy >= 0 && ix <= m && iy <= m; };
  {  // xc on the W2 window
    constexpr int NS = tl_steps<W2 * W2>();
    T xv[NS], c[NS][4];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W2, lx = i - ly * W2, ix = ox + lx, iy = oy + ly;
      const bool ok = i < W2 * W2 && inside(ix, iy);
      const TlProlong q = tl_prolong_at(ok ? ix : 0, ok ? iy : 0, m);
      xv[k] = ok ? __ldg(F.x + iy * n1 + ix) : T(0);
      c[k][0] = ok ? __ldg(C.y + q.jy0 * cn1 + q.jx0) : T(0);
      c[k][1] = ok ? __ldg(C.y + q.jy0 * cn1 + q.jx1) : T(0);
      c[k][2] = ok ? __ldg(C.y + q.jy1 * cn1 + q.jx0) : T(0);
      c[k][3] = ok ? __ldg(C.y + q.jy1 * cn1 + q.jx1) : T(0);
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W2, lx = i - ly * W2, ix = ox + lx, iy = oy + ly;
      if (i >= W2 * W2) break;
      const bool ok = inside(ix, iy);
      const TlProlong q = tl_prolong_at(ok ? ix : 0, ok ? iy : 0, m);
      sxc[ly][lx] = ok ? xv[k] + tl_prolong_value(q, c[k][0], c[k][1], c[k][2], c[k][3]) : T(0);
    }
  }
  __syncthreads();
  {  // y1 on the W1 window
    constexpr int NS = tl_steps<W1 * W1>();
    TlRow<T> r[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W1, lx = i - ly * W1, ix = ox + 1 + lx, iy = oy + 1 + ly;
      const bool ok = i < W1 * W1 && inside(ix, iy);
      tl_load_row(F, ok ? iy * n1 + ix : 0, nv, ok, true, r[k]);
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / W1, lx = i - ly * W1;
      if (i >= W1 * W1) break;
      // outside the level the row, b and xc are zero and so is y1
      sy[ly][lx] = fma(r[k].wd, r[k].b - tl_row_apply<T, W2>(r[k], &sxc[ly][lx]), sxc[ly + 1][lx + 1]);
    }
  }
  __syncthreads();
  {  // y on the tile
    constexpr int NS = tl_steps<kTlUp * kTlUp>();
    TlRow<T> r[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / kTlUp, lx = i - ly * kTlUp, ix = fx0 + lx, iy = fy0 + ly;
      const bool ok = i < kTlUp * kTlUp && inside(ix, iy);
      tl_load_row(F, ok ? iy * n1 + ix : 0, nv, ok, true, r[k]);
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const int i = k * kTlTileThreads + t, ly = i / kTlUp, lx = i - ly * kTlUp, ix = fx0 + lx, iy = fy0 + ly;
      if (i >= kTlUp * kTlUp || !inside(ix, iy)) continue;
      F.y[iy * n1 + ix] = fma(r[k].wd, r[k].b - tl_row_apply<T, W1>(r[k], &sy[ly][lx]), sy[ly + 1][lx + 1]);
    }
  }
}

// The coarse end of the V-cycle in one block: from level l0 (at most
// kTlTailCells cells per side; its b given, or from the corner sums cp when
// l0 = 0) down to the coarsest level, its dense solve, and back up to l0's
// result y.  Every phase is one pass over a level's vertices followed by a
// block barrier; x1 and the residual live in y on the way down, the
// corrected iterate and the first post-sweep in y and x on the way up.
template <typename T, typename LevAt>
__device__ __forceinline__ void tl_tail_body(LevAt lev, int l0, int nl, const T* __restrict__ ainv,
                                             const T* __restrict__ cp, int dim) {
  const int tid = threadIdx.x, nt = blockDim.x;
  if (l0 == 0 && cp) {
    const TlLev<T> F = lev(0);
    const int n1 = F.m + 1;
    for (int v = tid; v < n1 * n1; v += nt) F.b[v] = tl_corner_sum(cp, dim, v % n1, v / n1);
    __syncthreads();
  }
  for (int l = l0; l + 1 < nl; ++l) {
    const TlLev<T> F = lev(l), C = lev(l + 1);
    const int m = F.m, n1 = m + 1, nv = n1 * n1;
    for (int v = tid; v < nv; v += nt) F.y[v] = F.wd[v] * F.b[v];  // x1
    __syncthreads();
    for (int v = tid; v < nv; v += nt) F.x[v] = fma(F.wd[v], F.b[v] - tl_stencil(F, F.y, v % n1, v / n1), F.y[v]);
    __syncthreads();
    for (int v = tid; v < nv; v += nt) F.y[v] = F.b[v] - tl_stencil(F, F.x, v % n1, v / n1);  // residual
    __syncthreads();
    const int cn1 = C.m + 1;
    for (int v = tid; v < cn1 * cn1; v += nt) {
      const int J = v % cn1, I = v / cn1;
      T acc = T(0);
      for (int iy = 2 * I - 1; iy <= 2 * I + 1; ++iy) {
        if (iy < 0 || iy > m) continue;
        const T wy = tl_w<T>(iy, I, m);
        for (int ix = 2 * J - 1; ix <= 2 * J + 1; ++ix) {
          if (ix < 0 || ix > m) continue;
          acc = fma(wy * tl_w<T>(ix, J, m), F.y[iy * n1 + ix], acc);
        }
      }
      C.b[v] = acc;
    }
    __syncthreads();
  }
  {
    const TlLev<T> L = lev(nl - 1);
    const int nv = (L.m + 1) * (L.m + 1);
    for (int v = tid; v < nv; v += nt) {
      T acc = T(0);
      for (int u = 0; u < nv; ++u) acc = fma(ainv[v * nv + u], L.b[u], acc);
      L.y[v] = acc;
    }
    __syncthreads();
  }
  for (int l = nl - 2; l >= l0; --l) {
    const TlLev<T> F = lev(l), C = lev(l + 1);
    const int n1 = F.m + 1, nv = n1 * n1;
    for (int v = tid; v < nv; v += nt) F.y[v] = tl_corrected(F, C, v % n1, v / n1);  // xc
    __syncthreads();
    for (int v = tid; v < nv; v += nt) F.x[v] = fma(F.wd[v], F.b[v] - tl_stencil(F, F.y, v % n1, v / n1), F.y[v]);
    __syncthreads();
    for (int v = tid; v < nv; v += nt) F.y[v] = fma(F.wd[v], F.b[v] - tl_stencil(F, F.x, v % n1, v / n1), F.x[v]);
    __syncthreads();
  }
}

// The first level of the one-block tail.
__host__ __device__ inline int tl_tail_level(const int* m, int nl) {
  int l = 0;
  while (l + 1 < nl && m[l] > kTlTailCells) ++l;
  return l;
}

__host__ __device__ inline int tl_tiles(int verts, int tile) { return (verts + tile - 1) / tile; }

template <typename T>
__global__ void __launch_bounds__(kTlTileThreads)
    k_tl_down(TlLev<T> F, TlLev<T> C, const T* __restrict__ cp, int dim, const int* done) {
  if (tl_done(done)) return;
  const int t = tl_tiles(C.m + 1, kTlDown);
  tl_down_body<T>(F, C, cp, dim, blockIdx.x % t, blockIdx.x / t);
}
template <typename T>
__global__ void __launch_bounds__(kTlTileThreads) k_tl_up(TlLev<T> F, TlLev<T> C, const int* done) {
  if (tl_done(done)) return;
  const int t = tl_tiles(F.m + 1, kTlUp);
  tl_up_body<T>(F, C, blockIdx.x % t, blockIdx.x / t);
}
// The levels of one preconditioner (kernel parameter).
template <typename T>
struct TlLevels {
  TlLev<T> lev[kTlMaxLevels];
};

template <typename T>
__global__ void __launch_bounds__(kTlTailThreads)
    k_tl_tail(const __grid_constant__ TlLevels<T> L, int l0, int nl, const T* __restrict__ ainv,
              const T* __restrict__ cp, int dim, const int* done) {
  if (tl_done(done)) return;
  tl_tail_body<T>([&](int l) { return L.lev[l]; }, l0, nl, ainv, cp, dim);
}

// The Q1 function of the element's corner values at node (i1, i2).
template <typename T, int P>
__device__ __forceinline__ T tl_q1(const TlHat<T, P>& h, int i1, int i2, T x00, T x01, T x10, T x11) {
  return h.l[0][i1] * (h.l[0][i2] * x00 + h.l[1][i2] * x01) + h.l[1][i1] * (h.l[0][i2] * x10 + h.l[1][i2] * x11);
}

// Floats of one factor of an element type's table (V_x, V_y or D^-1, n1^2
// values), padded to a 16-byte multiple so that each is read as float4s.
__host__ __device__ constexpr int tl_fdm_stride(int n1) { return (n1 * n1 + 3) & ~3; }

// z = B^-1 r + P x0 (x0: the level-0 V-cycle result), B^-1 by fast
// diagonalisation.  With R[i1][i2] the element's residual (node i1 N1 + i2)
// and its type's factors V_x, V_y, D^-1 (fdm: [V_x | V_y | D^-1] per type),
//   B^-1 r = V_x (D^-1 o U) V_y^T,   U = V_x^T R V_y,
// four 1-D transforms of N1^3 multiply-adds each, with the transform's 1-D
// factor in registers (read as float4s) and the element's nodal block in a
// column of shared memory between transforms: the first transform reads r
// straight from global memory and the last writes z there, so each of the
// two middle passes costs one shared-memory read and write per node.
// MODE 1: also r.z = sum D^-1 o U o U + r.(P x0) and the PCG bookkeeping of
// the inner state (first: rr = r.z; else beta = r.z / rr, rr = r.z), reduced
// over the nb blocks of this instance.
template <typename T, int P, int MODE>
__device__ __forceinline__ void tl_finish_body(const T* __restrict__ r, T* __restrict__ z, const T* __restrict__ x0,
                                               const T* __restrict__ fdm, int dim, const TlHat<T, P>& h,
                                               CgState<T>* st, const ReduceScratch& red, int bid, int nb) {
  static_assert(sizeof(T) == 4, "the element-block factors are FP32");
  constexpr int N1 = P + 1, NN = N1 * N1, FS = tl_fdm_stride(N1);
  __shared__ T col[NN][kTlElemThreads];
  __shared__ T sh[32];
  const int t = threadIdx.x;
  const size_t noe = (size_t)dim * dim;
  T acc = T(0);
  T f[FS];
  auto load_factor = [&](const T* __restrict__ src) {
    const float4* __restrict__ s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
    for (int q = 0; q < FS / 4; ++q) {
      const float4 v = __ldg(s4 + q);
      f[4 * q] = v.x;
      f[4 * q + 1] = v.y;
      f[4 * q + 2] = v.z;
      f[4 * q + 3] = v.w;
    }
  };
  const size_t tiles = (noe + kTlElemThreads - 1) / kTlElemThreads;
  for (size_t tile = bid; tile < tiles; tile += nb) {
    const size_t e = tile * kTlElemThreads + t;
    if (e >= noe) continue;
    const int row = (int)(e / dim), cl = (int)(e % dim), R = dim - 1 - row;
    const T* __restrict__ F = fdm + (size_t)tl_elem_type(row, cl, dim) * 3 * FS;
    const T x00 = x0[R * (dim + 1) + cl], x10 = x0[R * (dim + 1) + cl + 1];
    const T x01 = x0[(R + 1) * (dim + 1) + cl], x11 = x0[(R + 1) * (dim + 1) + cl + 1];
    load_factor(F);  // V_x
    // U1 = V_x^T R (along i1), R read column by column from global memory
#pragma unroll
    for (int i2 = 0; i2 < N1; ++i2) {
      T c[N1];
#pragma unroll
      for (int i1 = 0; i1 < N1; ++i1) c[i1] = __ldg(r + (size_t)(i1 * N1 + i2) * noe + e);
      if (MODE == 1) {
#pragma unroll
        for (int i1 = 0; i1 < N1; ++i1) acc = fma(c[i1], tl_q1<T, P>(h, i1, i2, x00, x01, x10, x11), acc);
      }
#pragma unroll
      for (int a = 0; a < N1; ++a) {
        T s = T(0);
#pragma unroll
        for (int i1 = 0; i1 < N1; ++i1) s = fma(f[i1 * N1 + a], c[i1], s);
        col[a * N1 + i2][t] = s;
      }
    }
    load_factor(F + FS);  // V_y
    // D^-1 o (U1 V_y), then its product with V_y^T (along i2)
#pragma unroll 1
    for (int a = 0; a < N1; ++a) {
      T c[N1], u[N1];
#pragma unroll
      for (int i2 = 0; i2 < N1; ++i2) c[i2] = col[a * N1 + i2][t];
#pragma unroll
      for (int b = 0; b < N1; ++b) {
        T s = T(0);
#pragma unroll
        for (int i2 = 0; i2 < N1; ++i2) s = fma(f[i2 * N1 + b], c[i2], s);
        const T dv = __ldg(F + 2 * FS + a * N1 + b);
        if (MODE == 1) acc = fma(s * s, dv, acc);
        u[b] = s * dv;
      }
#pragma unroll
      for (int i2 = 0; i2 < N1; ++i2) {
        T s = T(0);
#pragma unroll
        for (int b = 0; b < N1; ++b) s = fma(f[i2 * N1 + b], u[b], s);
        col[a * N1 + i2][t] = s;
      }
    }
    load_factor(F);  // V_x
    // z = V_x (...) + P x0 (along i1)
#pragma unroll 1
    for (int i2 = 0; i2 < N1; ++i2) {
      T c[N1];
#pragma unroll
      for (int a = 0; a < N1; ++a) c[a] = col[a * N1 + i2][t];
#pragma unroll
      for (int i1 = 0; i1 < N1; ++i1) {
        T s = tl_q1<T, P>(h, i1, i2, x00, x01, x10, x11);
#pragma unroll
        for (int a = 0; a < N1; ++a) s = fma(f[i1 * N1 + a], c[a], s);
        z[(size_t)(i1 * N1 + i2) * noe + e] = s;
      }
    }
  }
  if (MODE == 1) {
    const T bt = block_sum<T, kTlElemThreads>(acc, sh);
    T total;
    if (grid_sum_last<T, kTlElemThreads>(bt, red, bid, nb, sh, &total) && t == 0) {
      if (!st->first) st->beta = total / st->rr;
      st->rr = total;
      if (!(total > T(0)) || !isfinite(total)) {
        st->status = (int)SIPG_ERR_BREAKDOWN;
        st->done = 1;
      }
    }
  }
}

template <typename T, int P, int MODE>
__global__ void __launch_bounds__(kTlElemThreads)
    k_tl_finish(const T* __restrict__ r, T* __restrict__ z, const T* __restrict__ x0, const T* __restrict__ fdm,
                int dim, const __grid_constant__ TlHat<T, P> h, CgState<T>* st, ReduceScratch red) {
  if (MODE == 1 && *(volatile int*)&st->done) return;
  tl_finish_body<T, P, MODE>(r, z, x0, fdm, dim, h, st, red, blockIdx.x, gridDim.x);
}

// ---- many instances (instance = blockIdx.y; element kernels per degree group) ----

__device__ __forceinline__ bool tlb_skip(const TlInst& v) { return *(volatile const int*)&v.st->done != 0; }

template <int P>
__global__ void __launch_bounds__(kTlElemThreads)
    k_tlb_restrict_elem(const TlInst* __restrict__ insts, int first, const __grid_constant__ TlHat<float, P> h) {
  const TlInst& v = insts[first + blockIdx.y];
  if ((int)blockIdx.x >= v.nblk || tlb_skip(v)) return;
  tl_restrict_elem_body<float, P>(v.r, v.cp, (size_t)v.dim * v.dim, h, blockIdx.x, v.nblk);
}
// level l -> l + 1 of every instance that has level l + 1 (grid.x: the largest tile count)
__global__ void __launch_bounds__(kTlTileThreads) k_tlb_down(const TlInst* __restrict__ insts, int l) {
  const TlInst& v = insts[blockIdx.y];
  if (l >= v.tail0 || tlb_skip(v)) return;
  const int t = tl_tiles(v.lev[l + 1].m + 1, kTlDown);
  if ((int)blockIdx.x >= t * t) return;
  tl_down_body<float>(v.lev[l], v.lev[l + 1], l == 0 ? v.cp : nullptr, v.dim, blockIdx.x % t, blockIdx.x / t);
}
__global__ void __launch_bounds__(kTlTailThreads) k_tlb_tail(const TlInst* __restrict__ insts) {
  const TlInst& v = insts[blockIdx.y];
  if (tlb_skip(v)) return;
  tl_tail_body<float>([&](int l) { return v.lev[l]; }, v.tail0, v.nl, v.ainv, v.cp, v.dim);
}
__global__ void __launch_bounds__(kTlTileThreads) k_tlb_up(const TlInst* __restrict__ insts, int l) {
  const TlInst& v = insts[blockIdx.y];
  if (l >= v.tail0 || tlb_skip(v)) return;
  const int t = tl_tiles(v.lev[l].m + 1, kTlUp);
  if ((int)blockIdx.x >= t * t) return;
  tl_up_body<float>(v.lev[l], v.lev[l + 1], blockIdx.x % t, blockIdx.x / t);
}
template <int P>
__global__ void __launch_bounds__(kTlElemThreads)
    k_tlb_finish(const TlInst* __restrict__ insts, int first, const __grid_constant__ TlHat<float, P> h) {
  const TlInst& v = insts[first + blockIdx.y];
  if ((int)blockIdx.x >= v.nblk || tlb_skip(v)) return;
  tl_finish_body<float, P, 1>(v.r, v.z, v.lev[0].y, v.fdm, v.dim, h, v.st, v.red, blockIdx.x, v.nblk);
}

// ---- host side ----

int tl_grid(size_t n, int threads, int cap) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + threads - 1) / threads, (size_t)cap));
}

template <typename T, int P>
TlHat<T, P> tl_hat(const HostTables& h) {
  TlHat<T, P> t;
  for (int i = 0; i <= P; ++i) {
    t.l[0][i] = (T)(0.5 * (1.0 - h.nodes[i]));
    t.l[1][i] = (T)(0.5 * (1.0 + h.nodes[i]));
  }
  return t;
}

#define SIPG_TL_DISPATCH(FN, T, p, ...)  \
  switch (p) {                             \
    case 1: FN<T, 1>(__VA_ARGS__); break;  \
    case 2: FN<T, 2>(__VA_ARGS__); break;  \
    case 3: FN<T, 3>(__VA_ARGS__); break;  \
    case 4: FN<T, 4>(__VA_ARGS__); break;  \
    case 5: FN<T, 5>(__VA_ARGS__); break;  \
    case 6: FN<T, 6>(__VA_ARGS__); break;  \
    case 7: FN<T, 7>(__VA_ARGS__); break;  \
    case 8: FN<T, 8>(__VA_ARGS__); break;  \
  }

template <typename T, int P>
void tl_launch_restrict_elem(const HostTables& h, const T* r, T* cp, size_t noe, const int* done, cudaStream_t s) {
  k_tl_restrict_elem<T, P><<<tl_grid(noe, kTlElemThreads, 152 * 32), kTlElemThreads, 0, s>>>(r, cp, noe,
                                                                                             tl_hat<T, P>(h), done);
}
template <typename T, int P>
void tl_launch_update_restrict(const HostTables& h, float* x, const float* pb0, const float* pb1, float* r,
                               const float* Ap, float* cp, size_t noe, CgState<float>* st, ReduceScratch red,
                               cudaStream_t s) {
  k_tl_update_restrict<P><<<tl_grid(noe, kTlElemThreads, red.capacity), kTlElemThreads, 0, s>>>(
      x, pb0, pb1, r, Ap, cp, noe, st, red, tl_hat<float, P>(h));
}
template <typename T, int P>
void tl_launch_prolong(const HostTables& h, const T* xv, T* out, int dim, cudaStream_t s) {
  k_tl_prolong<T, P><<<tl_grid((size_t)dim * dim, kTlElemThreads, 152 * 32), kTlElemThreads, 0, s>>>(
      xv, out, dim, tl_hat<T, P>(h));
}
template <typename T, int P>
void tl_launch_finish(const HostTables& h, int mode, const T* r, T* z, const T* x0, const T* fdm, int dim,
                      CgState<T>* st, ReduceScratch red, cudaStream_t s) {
  const size_t noe = (size_t)dim * dim;
  if (mode == 1)
    k_tl_finish<T, P, 1><<<tl_grid(noe, kTlElemThreads, red.capacity), kTlElemThreads, 0, s>>>(
        r, z, x0, fdm, dim, tl_hat<T, P>(h), st, red);
  else
    k_tl_finish<T, P, 0><<<tl_grid(noe, kTlElemThreads, 152 * 32), kTlElemThreads, 0, s>>>(r, z, x0, fdm, dim,
                                                                                           tl_hat<T, P>(h), st, red);
}

// Gauss-Jordan inverse with partial pivoting (n <= 81); false if singular.
bool tl_invert(std::vector<double>& a, int n) {
  std::vector<double> inv((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[(size_t)i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[(size_t)r * n + c]) > std::fabs(a[(size_t)piv * n + c])) piv = r;
    if (!(std::fabs(a[(size_t)piv * n + c]) > 0.0)) return false;
    if (piv != c)
      for (int k = 0; k < n; ++k) {
        std::swap(a[(size_t)piv * n + k], a[(size_t)c * n + k]);
        std::swap(inv[(size_t)piv * n + k], inv[(size_t)c * n + k]);
      }
    const double d = 1.0 / a[(size_t)c * n + c];
    for (int k = 0; k < n; ++k) {
      a[(size_t)c * n + k] *= d;
      inv[(size_t)c * n + k] *= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[(size_t)r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        a[(size_t)r * n + k] -= f * a[(size_t)c * n + k];
        inv[(size_t)r * n + k] -= f * inv[(size_t)c * n + k];
      }
    }
  }
  a.swap(inv);
  return true;
}

// Symmetric eigen-decomposition a = Q diag(lam) Q^T by cyclic Jacobi
// rotations (n <= 9; a is overwritten).
void tl_jacobi_eig(std::vector<double>& a, int n, std::vector<double>& lam, std::vector<double>& Q) {
  Q.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += a[(size_t)i * n + j] * a[(size_t)i * n + j];
        if (i != j) off += a[(size_t)i * n + j] * a[(size_t)i * n + j];
      }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[(size_t)p * n + q];
        if (apq == 0.0) continue;
        // the rotation in the (p, q) plane that zeroes a_pq: cot 2 theta = (a_qq - a_pp) / (2 a_pq)
        const double th = (a[(size_t)q * n + q] - a[(size_t)p * n + p]) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
          const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - sn * akq;
          a[(size_t)k * n + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - sn * aqk;
          a[(size_t)q * n + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double qkp = Q[(size_t)k * n + p], qkq = Q[(size_t)k * n + q];
          Q[(size_t)k * n + p] = c * qkp - sn * qkq;
          Q[(size_t)k * n + q] = sn * qkp + c * qkq;
        }
      }
  }
  lam.resize(n);
  for (int i = 0; i < n; ++i) lam[i] = a[(size_t)i * n + i];
}

// Generalised eigenvalues of an element block at most this fraction of the
// largest in magnitude count as zero (a singular block, as the single element
// of a 1 x 1 mesh at p = 1 and penalty 1 is): their modes are left out.
constexpr double kTlNullRel = 1e-12;

// Fast diagonalisation of one element block B (nn x nn, node k = i1 n1 +
// i2, i1 along x): the SIPG element block is separable,
//   B = L_x (x) W + W (x) L_y,   W = diag(w),
// L_x the 1-D operator along x with its own face terms (which of the LEFT /
// RIGHT faces are on the boundary), L_y along y.  With L V = W V Lambda and
// V^T W V = I in each direction, B^-1 = (V_x (x) V_y) D^-1 (V_x (x) V_y)^T,
// D = Lambda_x (x) I + I (x) Lambda_y.  out = [V_x | V_y | D^-1], each
// tl_fdm_stride(n1) floats (V[i][a] at i n1 + a, D^-1[a][b] at a n1 + b;
// zero for a null mode).  False if B is not of this form (to 1e-9) or is zero.
bool tl_fdm(const std::vector<double>& B, const double* w, int n1, float* out) {
  const int nn = n1 * n1;
  auto b = [&](int i1, int i2, int j1, int j2) { return B[(size_t)(i1 * n1 + i2) * nn + (j1 * n1 + j2)]; };
  std::vector<double> Lx((size_t)n1 * n1), Ly((size_t)n1 * n1);
  // off-diagonals from the first row / column of nodes; the split of the
  // diagonal is free up to L_x + c W, L_y - c W: take L_y[0][0] = 0
  for (int i = 0; i < n1; ++i)
    for (int j = 0; j < n1; ++j) {
      if (i != j) {
        Lx[(size_t)i * n1 + j] = b(i, 0, j, 0) / w[0];
        Ly[(size_t)i * n1 + j] = b(0, i, 0, j) / w[0];
      }
    }
  for (int i = 0; i < n1; ++i) Lx[(size_t)i * n1 + i] = b(i, 0, i, 0) / w[0];
  for (int j = 0; j < n1; ++j) Ly[(size_t)j * n1 + j] = (b(0, j, 0, j) - Lx[0] * w[j]) / w[0];
  double err = 0.0, mx = 0.0;
  for (int i1 = 0; i1 < n1; ++i1)
    for (int i2 = 0; i2 < n1; ++i2)
      for (int j1 = 0; j1 < n1; ++j1)
        for (int j2 = 0; j2 < n1; ++j2) {
          const double m = (i2 == j2 ? Lx[(size_t)i1 * n1 + j1] * w[i2] : 0.0) +
                           (i1 == j1 ? w[i1] * Ly[(size_t)i2 * n1 + j2] : 0.0);
          err = std::max(err, std::fabs(m - b(i1, i2, j1, j2)));
          mx = std::max(mx, std::fabs(b(i1, i2, j1, j2)));
        }
  if (!(err <= 1e-9 * mx)) return false;
  std::vector<double> V[2], lam[2];
  for (int d = 0; d < 2; ++d) {
    const std::vector<double>& L = d ? Ly : Lx;
    std::vector<double> C((size_t)n1 * n1), Q;
    for (int i = 0; i < n1; ++i)
      for (int j = 0; j < n1; ++j)
        C[(size_t)i * n1 + j] = 0.5 * (L[(size_t)i * n1 + j] + L[(size_t)j * n1 + i]) / std::sqrt(w[i] * w[j]);
    tl_jacobi_eig(C, n1, lam[d], Q);
    V[d].resize((size_t)n1 * n1);
    for (int i = 0; i < n1; ++i)
      for (int a = 0; a < n1; ++a) V[d][(size_t)i * n1 + a] = Q[(size_t)i * n1 + a] / std::sqrt(w[i]);
  }
  const int fs = tl_fdm_stride(n1);
  for (int i = 0; i < nn; ++i) {
    out[i] = (float)V[0][i];
    out[fs + i] = (float)V[1][i];
  }
  double dmax = 0.0;
  for (int a = 0; a < n1; ++a)
    for (int c = 0; c < n1; ++c) dmax = std::max(dmax, std::fabs(lam[0][a] + lam[1][c]));
  for (int a = 0; a < n1; ++a)
    for (int c = 0; c < n1; ++c) {
      const double dsum = lam[0][a] + lam[1][c];
      out[2 * fs + a * n1 + c] = std::fabs(dsum) <= kTlNullRel * dmax ? 0.0f : (float)(1.0 / dsum);
    }
  return dmax > 0.0;
}

// A fixed pool of host worker threads for the set-up's row loops (created on
// first use, kept for the process): a loop is cut into one chunk per worker
// and the caller waits for its own chunks.  Several callers (the solve
// server's preparation threads) may share the pool; chunks never wait on
// other chunks.
class HostPool {
 public:
  static HostPool& get() {
    static HostPool pool;
    return pool;
  }
  int size() const { return (int)workers_.size(); }
  // runs every task and returns when all have run
  void run(std::vector<std::function<void()>>& tasks) {
    std::mutex done_mu;
    std::condition_variable done_cv;
    size_t left = tasks.size();
    {
      std::lock_guard<std::mutex> lock(mu_);
      for (std::function<void()>& t : tasks)
        queue_.push_back([&t, &done_mu, &done_cv, &left] {
          t();
          std::lock_guard<std::mutex> l(done_mu);
          if (--left == 0) done_cv.notify_all();
        });
    }
    cv_.notify_all();
    std::unique_lock<std::mutex> lock(done_mu);
    done_cv.wait(lock, [&] { return left == 0; });
  }

 private:
  HostPool() {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    for (unsigned k = 0; k < hw; ++k)
      workers_.emplace_back([this] {
        for (;;) {
          std::function<void()> task;
          {
            std::unique_lock<std::mutex> lock(mu_);
            cv_.wait(lock, [&] { return stop_ || !queue_.empty(); });
            if (stop_ && queue_.empty()) return;
            task = std::move(queue_.front());
            queue_.pop_front();
          }
          task();
        }
      });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lock(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (std::thread& t : workers_) t.join();
  }
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::function<void()>> queue_;
  std::vector<std::thread> workers_;
  bool stop_ = false;
};

// Runs f(lo, hi) over [0, n) split across the host pool when n is large (the
// set-up of a large mesh's hierarchy is host work proportional to its
// vertices); each row range is written by one chunk, so results do not
// depend on the split.
template <typename F>
void host_rows(int n, F f) {
  HostPool& pool = HostPool::get();
  const int nt = (n >= 128 && pool.size() > 1) ? std::min(pool.size(), n / 32) : 1;
  if (nt <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::function<void()>> tasks;
  for (int t = 0; t < nt; ++t) {
    const int lo = (int)((long long)n * t / nt), hi = (int)((long long)n * (t + 1) / nt);
    tasks.emplace_back([=, &f] { f(lo, hi); });
  }
  pool.run(tasks);
}

// Host 9-point stencil of one level: S[k * nv + v].
struct HostLevel {
  int m = 0;
  std::vector<double> S;
  double omega = 0;
};

void host_stencil_apply(const HostLevel& L, const std::vector<double>& x, std::vector<double>& y) {
  const int n1 = L.m + 1, nv = n1 * n1;
  y.assign(nv, 0.0);
  host_rows(n1, [&](int lo, int hi) {
    for (int vy = lo; vy < hi; ++vy)
      for (int vx = 0; vx <= L.m; ++vx) {
        const int v = vy * n1 + vx;
        double s = 0.0;
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            const int ux = vx + dx, uy = vy + dy;
            if (ux < 0 || uy < 0 || ux > L.m || uy > L.m) continue;
            s += L.S[(size_t)((dy + 1) * 3 + (dx + 1)) * nv + v] * x[uy * n1 + ux];
          }
        y[v] = s;
      }
  });
}

// The coarse vertices whose interpolation weight at fine vertex g is not
// zero (one or two): the coarse vertices sit at the even fine vertices and
// at m, an odd fine vertex other than m lies between two.
inline int tl_parents(int g, int m, int* out) {
  if (g % 2 == 0 || g == m) {
    out[0] = (g + 1) / 2;
    return 1;
  }
  out[0] = (g - 1) / 2;
  out[1] = (g + 1) / 2;
  return 2;
}

// the next level's stencil, C = P^T A P, entry by entry: for coarse vertex
// v, every fine vertex f under it (weight P(f, v)), every neighbour g of f
// (A(f, g)) and every coarse vertex u over g (P(g, u)) -- at most nine
// neighbours u, all within one coarse cell of v
HostLevel host_galerkin(const HostLevel& F) {
  HostLevel C;
  C.m = (F.m + 1) / 2;
  const int cn1 = C.m + 1, cnv = cn1 * cn1, fn1 = F.m + 1, fnv = fn1 * fn1, m = F.m;
  C.S.assign((size_t)9 * cnv, 0.0);
  host_rows(cn1, [&](int lo, int hi) {
    for (int I = lo; I < hi; ++I)
      for (int J = 0; J <= C.m; ++J) {
        double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int fy = std::max(0, 2 * I - 1); fy <= std::min(m, 2 * I + 1); ++fy) {
          const double wy = tl_w<double>(fy, I, m);
          if (wy == 0.0) continue;
          for (int fx = std::max(0, 2 * J - 1); fx <= std::min(m, 2 * J + 1); ++fx) {
            const double wx = tl_w<double>(fx, J, m);
            if (wx == 0.0) continue;
            const int f = fy * fn1 + fx;
            for (int dy = -1; dy <= 1; ++dy)
              for (int dx = -1; dx <= 1; ++dx) {
                const int gx = fx + dx, gy = fy + dy;
                if (gx < 0 || gy < 0 || gx > m || gy > m) continue;
                const double a = F.S[(size_t)((dy + 1) * 3 + (dx + 1)) * fnv + f];
                if (a == 0.0) continue;
                int py[2], px[2];
                const int ny = tl_parents(gy, m, py), nx = tl_parents(gx, m, px);
                for (int iy = 0; iy < ny; ++iy)
                  for (int ix = 0; ix < nx; ++ix)
                    acc[(py[iy] - I + 1) * 3 + (px[ix] - J + 1)] +=
                        wx * wy * a * tl_w<double>(gy, py[iy], m) * tl_w<double>(gx, px[ix], m);
              }
          }
        }
        for (int k = 0; k < 9; ++k) C.S[(size_t)k * cnv + I * cn1 + J] = acc[k];
      }
  });
  return C;
}

// omega = 1.52 / lambda_max(D^-1 A) (power iteration from a fixed vector)
double host_omega(const HostLevel& L) {
  const int n1 = L.m + 1, nv = n1 * n1;
  std::vector<double> x(nv), y, nrm_row(n1), nx_row(n1);
  for (int v = 0; v < nv; ++v) x[v] = std::sin(0.7 * v + 0.3) + 0.5;
  double lam = 1.0;
  for (int it = 0; it < 40; ++it) {
    host_stencil_apply(L, x, y);
    // per-row partial sums, then the rows in order: the same result for any split
    host_rows(n1, [&](int lo, int hi) {
      for (int vy = lo; vy < hi; ++vy) {
        double a = 0.0, b = 0.0;
        for (int v = vy * n1; v < (vy + 1) * n1; ++v) {
          y[v] /= L.S[(size_t)4 * nv + v];
          a += y[v] * y[v];
          b += x[v] * x[v];
        }
        nrm_row[vy] = a;
        nx_row[vy] = b;
      }
    });
    double nrm = 0.0, nx = 0.0;
    for (int vy = 0; vy < n1; ++vy) {
      nrm += nrm_row[vy];
      nx += nx_row[vy];
    }
    lam = std::sqrt(nrm / nx);
    const double s = 1.0 / std::sqrt(nrm);
    host_rows(n1, [&](int lo, int hi) {
      for (int v = lo * n1; v < hi * n1; ++v) x[v] = y[v] * s;
    });
  }
  return 1.6 / (1.05 * lam);
}

}  // namespace sipg

namespace {

// Everything the preconditioner keeps on the device for one operator.
struct TwoLevel {
  int dim = 0, p = 0;
  float* fdm = nullptr;   // [16][3][tl_fdm_stride] element block factors [V_x | V_y | D^-1]
  float* cp = nullptr;    // [4][noe] corner sums
  float* ainv = nullptr;  // coarsest level's dense inverse
  std::vector<TlLev<float>> lev;
  int tail0 = 0;          // first level of the one-block tail
  std::vector<void*> allocs;
  ~TwoLevel() {
    for (void* a : allocs) cudaFree(a);
  }
};

void twolevel_free(void* p) { delete static_cast<TwoLevel*>(p); }

template <typename T>
sipg_status dalloc(TwoLevel& tl, T** out, size_t count) {
  void* p = nullptr;
  SIPG_CUDA_TRY(cudaMalloc(&p, sizeof(T) * std::max<size_t>(count, 1)));
  tl.allocs.push_back(p);
  *out = static_cast<T*>(p);
  return SIPG_OK;
}

// Element block inverses by fast diagonalisation: probe the diagonal blocks
// with the FP64 operator on a mesh of min(dim, 3) elements per side, one
// checkerboard colour and node at a time, and factor each (tl_fdm).
// The element-block factors depend on the degree, the penalty and (below 3
// elements per side) the mesh, not on the mesh size: each set is probed once
// per process and kept.
std::mutex g_fdm_mutex;
std::map<std::tuple<int, double, int>, std::vector<float>> g_fdm_cache;

sipg_status build_blocks_probe(sipg_op* op, std::vector<float>& table, cudaStream_t ss);

sipg_status build_blocks(sipg_op* op, std::vector<float>& table, cudaStream_t ss) {
  const auto key = std::make_tuple(op->p, op->pen, std::min(op->dim, 3));
  {
    std::lock_guard<std::mutex> lock(g_fdm_mutex);
    auto it = g_fdm_cache.find(key);
    if (it != g_fdm_cache.end()) {
      table = it->second;
      return SIPG_OK;
    }
  }
  const sipg_status st = build_blocks_probe(op, table, ss);
  if (st == SIPG_OK) {
    std::lock_guard<std::mutex> lock(g_fdm_mutex);
    g_fdm_cache[key] = table;
  }
  return st;
}

sipg_status build_blocks_probe(sipg_op* op, std::vector<float>& table, cudaStream_t ss) {
  const int p = op->p, n1 = p + 1, nn = n1 * n1, dm = std::min(op->dim, 3), noe = dm * dm;
  sipg_op* small = nullptr;
  sipg_status st = sipg_op_create(dm, p, op->pen, &small);
  if (st != SIPG_OK) return st;
  const size_t n = (size_t)nn * noe;
  double *dx = nullptr, *dy = nullptr;
  std::vector<double> hx(n), hy(n);
  std::vector<std::vector<double>> blk(kTlTypes);
  cudaError_t e = cudaMallocAsync(&dx, n * sizeof(double), ss);
  if (e == cudaSuccess) e = cudaMallocAsync(&dy, n * sizeof(double), ss);
  for (int color = 0; color < 2 && e == cudaSuccess && st == SIPG_OK; ++color)
    for (int k = 0; k < nn && e == cudaSuccess && st == SIPG_OK; ++k) {
      std::fill(hx.begin(), hx.end(), 0.0);
      for (int el = 0; el < noe; ++el)
        if (((el / dm) + (el % dm)) % 2 == color) hx[(size_t)k * noe + el] = 1.0;
      e = cudaMemcpyAsync(dx, hx.data(), n * sizeof(double), cudaMemcpyHostToDevice, ss);
      if (e != cudaSuccess) break;
      st = sipg_apply_f64(small, dx, dy, ss);
      if (st != SIPG_OK) break;
      e = cudaMemcpyAsync(hy.data(), dy, n * sizeof(double), cudaMemcpyDeviceToHost, ss);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ss);
      if (e != cudaSuccess) break;
      for (int el = 0; el < noe; ++el) {
        if (((el / dm) + (el % dm)) % 2 != color) continue;
        std::vector<double>& B = blk[tl_elem_type(el / dm, el % dm, dm)];
        if (B.empty()) B.assign((size_t)nn * nn, 0.0);
        for (int j = 0; j < nn; ++j) B[(size_t)j * nn + k] = hy[(size_t)j * noe + el];
      }
    }
  if (dx) cudaFreeAsync(dx, ss);
  if (dy) cudaFreeAsync(dy, ss);
  sipg_op_destroy(small);
  if (st != SIPG_OK) return st;
  SIPG_CUDA_TRY(e);
  const int fs = tl_fdm_stride(n1);
  table.assign((size_t)kTlTypes * 3 * fs, 0.0f);
  for (int t = 0; t < kTlTypes; ++t) {
    if (blk[t].empty()) continue;
    if (!tl_fdm(blk[t], op->tab.w, n1, table.data() + (size_t)t * 3 * fs)) {
      set_error("two-level preconditioner: an element block is not of the form W (x) L_x + L_y (x) W");
      return SIPG_ERR_INVALID;
    }
  }
  return SIPG_OK;
}

// The level-0 vertex operator P^T A P, probed with the FP64 operator and nine
// colours of vertices.
sipg_status build_level0_probe(sipg_op* op, HostLevel& L0, cudaStream_t ss) {
  const int dim = op->dim, p = op->p, n1 = dim + 1, nv = n1 * n1;
  const size_t noe = (size_t)dim * dim, n = (size_t)op->ndof;
  L0.m = dim;
  L0.S.assign((size_t)9 * nv, 0.0);
  double *xv = nullptr, *xd = nullptr, *yd = nullptr, *cp = nullptr, *yv = nullptr;
  cudaError_t e = cudaMallocAsync(&xv, nv * sizeof(double), ss);
  if (e == cudaSuccess) e = cudaMallocAsync(&yv, nv * sizeof(double), ss);
  if (e == cudaSuccess) e = cudaMallocAsync(&xd, n * sizeof(double), ss);
  if (e == cudaSuccess) e = cudaMallocAsync(&yd, n * sizeof(double), ss);
  if (e == cudaSuccess) e = cudaMallocAsync(&cp, 4 * noe * sizeof(double), ss);
  std::vector<double> hx(nv);
  std::vector<std::vector<double>> hys(9, std::vector<double>(nv));
  sipg_status st = SIPG_OK;
  for (int c = 0; c < 9 && e == cudaSuccess && st == SIPG_OK; ++c) {
    const int cx = c % 3, cy = c / 3;
    for (int v = 0; v < nv; ++v) hx[v] = ((v % n1) % 3 == cx && (v / n1) % 3 == cy) ? 1.0 : 0.0;
    e = cudaMemcpyAsync(xv, hx.data(), nv * sizeof(double), cudaMemcpyHostToDevice, ss);
    if (e != cudaSuccess) break;
    SIPG_TL_DISPATCH(tl_launch_prolong, double, p, op->tab, xv, xd, dim, ss)
    count_launch();
    st = sipg_apply_f64(op, xd, yd, ss);
    if (st != SIPG_OK) break;
    SIPG_TL_DISPATCH(tl_launch_restrict_elem, double, p, op->tab, yd, cp, noe, (const int*)nullptr, ss)
    k_tl_restrict_vert<double><<<tl_grid(nv, kTlVecThreads, 1 << 30), kTlVecThreads, 0, ss>>>(cp, yv, dim);
    count_launch(2);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hys[c].data(), yv, nv * sizeof(double), cudaMemcpyDeviceToHost, ss);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ss);
    if (e != cudaSuccess) break;
  }
  if (e == cudaSuccess && st == SIPG_OK)  // entry (v, u) is probe colour(u)'s result at v
    host_rows(n1, [&](int lo, int hi) {
      for (int vy = lo; vy < hi; ++vy)
        for (int vx = 0; vx <= dim; ++vx)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const int ux = vx + dx, uy = vy + dy;
              if (ux < 0 || uy < 0 || ux > dim || uy > dim) continue;
              L0.S[(size_t)((dy + 1) * 3 + (dx + 1)) * nv + vy * n1 + vx] =
                  hys[(uy % 3) * 3 + ux % 3][vy * n1 + vx];
            }
    });
  for (double* q : {xv, yv, xd, yd, cp})
    if (q) cudaFreeAsync(q, ss);
  if (st != SIPG_OK) return st;
  SIPG_CUDA_TRY(e);
  return SIPG_OK;
}

// Meshes larger than this get their level-0 operator stamped from one of
// this many elements per side.
constexpr int kTlStampMesh = 6;

// Vertex v (0..m) of a large level as the vertex of the kTlStampMesh level
// whose row has the same entries: the two vertices at each end as they are,
// every other one as the middle vertex.
int tl_stamp_class(int v, int m) {
  if (v <= 2) return v;
  if (v >= m - 2) return kTlStampMesh - (m - v);
  return kTlStampMesh / 2;
}

// The level-0 vertex operator of op.  Its rows are a(phi_v, phi_u) for the
// bilinear vertex functions, which are continuous, so every jump term of the
// SIPG form vanishes between them and only the vertices on the boundary see
// the Nitsche terms; in 2-D the element and face terms do not depend on the
// element size.  So every row of a mesh with more than kTlStampMesh elements
// per side equals a row of the kTlStampMesh mesh (its two end vertices per
// axis, or its middle one) and is copied from it: nine probes of a 6 x 6 mesh
// instead of nine applies on the full mesh.
// The probed kTlStampMesh level per degree and penalty (the rows every larger
// mesh copies), probed once per process.
std::mutex g_stamp_mutex;
std::map<std::pair<int, double>, HostLevel> g_stamp_cache;

sipg_status build_level0(sipg_op* op, HostLevel& L0, cudaStream_t ss) {
  const int dim = op->dim;
  if (dim <= kTlStampMesh) return build_level0_probe(op, L0, ss);
  const auto key = std::make_pair(op->p, op->pen);
  HostLevel Ls;
  bool have = false;
  {
    std::lock_guard<std::mutex> lock(g_stamp_mutex);
    auto it = g_stamp_cache.find(key);
    if (it != g_stamp_cache.end()) {
      Ls = it->second;
      have = true;
    }
  }
  if (!have) {
    sipg_op* small = nullptr;
    sipg_status st = sipg_op_create(kTlStampMesh, op->p, op->pen, &small);
    if (st != SIPG_OK) return st;
    st = build_level0_probe(small, Ls, ss);
    sipg_op_destroy(small);
    if (st != SIPG_OK) return st;
    std::lock_guard<std::mutex> lock(g_stamp_mutex);
    g_stamp_cache[key] = Ls;
  }
  const int n1 = dim + 1, nv = n1 * n1, ns = kTlStampMesh + 1, nvs = ns * ns;
  L0.m = dim;
  L0.S.assign((size_t)9 * nv, 0.0);
  host_rows(n1, [&](int lo, int hi) {
    for (int vy = lo; vy < hi; ++vy) {
      const int cy = tl_stamp_class(vy, dim);
      for (int vx = 0; vx <= dim; ++vx) {
        const int c = cy * ns + tl_stamp_class(vx, dim);
        for (int k = 0; k < 9; ++k) L0.S[(size_t)k * nv + vy * n1 + vx] = Ls.S[(size_t)k * nvs + c];
      }
    }
  });
  return SIPG_OK;
}

// The set-up runs on a stream of its own with stream-ordered temporaries and
// waits only for that stream: an operator built while other streams of the
// process have work in flight (a serving lane's round) does not wait for it.
sipg_status build_on(sipg_op* op, TwoLevel& tl, cudaStream_t ss);

sipg_status build(sipg_op* op, TwoLevel& tl) {
  cudaStream_t ss = nullptr;
  SIPG_CUDA_TRY(cudaStreamCreateWithFlags(&ss, cudaStreamNonBlocking));
  const sipg_status st = build_on(op, tl, ss);
  const cudaError_t e = cudaStreamSynchronize(ss);  // host staging below outlives every copy
  cudaStreamDestroy(ss);
  if (st != SIPG_OK) return st;
  SIPG_CUDA_TRY(e);
  return SIPG_OK;
}

sipg_status build_on(sipg_op* op, TwoLevel& tl, cudaStream_t ss) {
  tl.dim = op->dim;
  tl.p = op->p;
  // everything on the host first: the element factors, the vertex levels,
  // the coarsest level's inverse
  std::vector<float> table;
  sipg_status st = build_blocks(op, table, ss);
  if (st != SIPG_OK) return st;
  std::vector<HostLevel> H(1);
  st = build_level0(op, H[0], ss);
  if (st != SIPG_OK) return st;
  while (H.back().m > kTlCoarsestCells) {
    if ((int)H.size() >= kTlMaxLevels) {
      set_error("two-level preconditioner: mesh too large for the vertex-grid hierarchy");
      return SIPG_ERR_UNSUPPORTED;
    }
    H.back().omega = host_omega(H.back());
    H.push_back(host_galerkin(H.back()));
  }
  const HostLevel& Lc = H.back();
  const int cn1 = Lc.m + 1, cnv = cn1 * cn1;
  std::vector<double> A((size_t)cnv * cnv, 0.0);
  for (int v = 0; v < cnv; ++v)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int ux = v % cn1 + dx, uy = v / cn1 + dy;
        if (ux < 0 || uy < 0 || ux > Lc.m || uy > Lc.m) continue;
        A[(size_t)v * cnv + uy * cn1 + ux] = Lc.S[(size_t)((dy + 1) * 3 + (dx + 1)) * cnv + v];
      }
  if (!tl_invert(A, cnv)) {
    set_error("two-level preconditioner: singular coarsest operator");
    return SIPG_ERR_INVALID;
  }
  std::vector<float> af(A.begin(), A.end());
  std::vector<std::vector<float>> hs(H.size()), hw(H.size());
  for (size_t l = 0; l < H.size(); ++l) {
    const HostLevel& L = H[l];
    const int nv = (L.m + 1) * (L.m + 1);
    hs[l].resize((size_t)9 * nv);
    hw[l].resize(nv);
    for (size_t i = 0; i < hs[l].size(); ++i) hs[l][i] = (float)L.S[i];
    for (int v = 0; v < nv; ++v) hw[l][v] = (float)(L.omega / L.S[(size_t)4 * nv + v]);
  }
  // one device allocation, carved in 256-byte aligned pieces
  size_t total = 0;
  auto piece = [&](size_t floats) {
    const size_t at = total;
    total += (floats * sizeof(float) + 255) & ~size_t(255);
    return at;
  };
  const size_t o_fdm = piece(table.size()), o_cp = piece(4 * (size_t)op->noe), o_ainv = piece(af.size());
  std::vector<size_t> o_lev(H.size());
  for (size_t l = 0; l < H.size(); ++l) {
    const size_t nv = (size_t)(H[l].m + 1) * (H[l].m + 1);
    o_lev[l] = piece(9 * nv);
    piece(nv);
    piece(nv);
    piece(nv);
    piece(nv);
  }
  char* base = nullptr;
  st = dalloc(tl, &base, total);
  if (st != SIPG_OK) return st;
  auto at = [&](size_t off) { return reinterpret_cast<float*>(base + off); };
  tl.fdm = at(o_fdm);
  tl.cp = at(o_cp);
  tl.ainv = at(o_ainv);
  SIPG_CUDA_TRY(cudaMemcpyAsync(tl.fdm, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice, ss));
  SIPG_CUDA_TRY(cudaMemcpyAsync(tl.ainv, af.data(), af.size() * sizeof(float), cudaMemcpyHostToDevice, ss));
  for (size_t l = 0; l < H.size(); ++l) {
    const size_t nv = (size_t)(H[l].m + 1) * (H[l].m + 1);
    const size_t step = (nv * sizeof(float) + 255) & ~size_t(255);
    TlLev<float> d{};
    d.m = H[l].m;
    float* S = at(o_lev[l]);
    float* wd = at(o_lev[l] + ((9 * nv * sizeof(float) + 255) & ~size_t(255)));
    d.S = S;
    d.wd = wd;
    d.b = reinterpret_cast<float*>(reinterpret_cast<char*>(wd) + step);
    d.x = reinterpret_cast<float*>(reinterpret_cast<char*>(wd) + 2 * step);
    d.y = reinterpret_cast<float*>(reinterpret_cast<char*>(wd) + 3 * step);
    SIPG_CUDA_TRY(cudaMemcpyAsync(S, hs[l].data(), hs[l].size() * sizeof(float), cudaMemcpyHostToDevice, ss));
    SIPG_CUDA_TRY(cudaMemcpyAsync(wd, hw[l].data(), hw[l].size() * sizeof(float), cudaMemcpyHostToDevice, ss));
    tl.lev.push_back(d);
  }
  std::vector<int> ms;
  for (const TlLev<float>& L : tl.lev) ms.push_back(L.m);
  tl.tail0 = tl_tail_level(ms.data(), (int)ms.size());
  SIPG_CUDA_TRY(cudaStreamSynchronize(ss));  // the host staging above ends here
  return SIPG_OK;
}

}  // namespace

namespace sipg {

// The operator's two-level preconditioner, built on first use (synchronous;
// not during stream capture).
sipg_status twolevel_get(sipg_op* op, void** out) {
  std::lock_guard<std::mutex> lk(op->mu);
  if (!op->tl) {
    SIPG_CUDA_TRY(cudaSetDevice(op->device));
    TwoLevel* tl = new (std::nothrow) TwoLevel;
    if (!tl) return SIPG_ERR_NOMEM;
    const sipg_status st = build(op, *tl);
    if (st != SIPG_OK) {
      delete tl;
      return st;
    }
    op->tl = tl;
    op->tl_free = twolevel_free;
  }
  *out = op->tl;
  return SIPG_OK;
}

// Enqueues z = M r on s (FP32).  With st (the inner PCG state): every kernel
// is skipped once st->done, and the last one sets r.z and beta in st.
sipg_status twolevel_enqueue(const sipg_op* op, const void* handle, const float* r, float* z, CgState<float>* st,
                             const ReduceScratch& red, cudaStream_t s, bool cp_ready) {
  const TwoLevel& tl = *static_cast<const TwoLevel*>(handle);
  const int* done = st ? &st->done : nullptr;
  const int dim = tl.dim, nl = (int)tl.lev.size();
  const size_t noe = (size_t)dim * dim;
  if (!cp_ready) {
    SIPG_TL_DISPATCH(tl_launch_restrict_elem, float, tl.p, op->tab, r, tl.cp, noe, done, s)
    count_launch();
  }
  const int l0 = tl.tail0;
  for (int l = 0; l < l0; ++l) {
    const int t = tl_tiles(tl.lev[l + 1].m + 1, kTlDown);
    k_tl_down<float><<<t * t, kTlTileThreads, 0, s>>>(tl.lev[l], tl.lev[l + 1], l == 0 ? tl.cp : nullptr, dim, done);
    count_launch();
  }
  TlLevels<float> levels{};
  for (int l = 0; l < nl; ++l) levels.lev[l] = tl.lev[l];
  k_tl_tail<float><<<1, kTlTailThreads, 0, s>>>(levels, l0, nl, tl.ainv, tl.cp, dim, done);
  count_launch();
  for (int l = l0 - 1; l >= 0; --l) {
    const int t = tl_tiles(tl.lev[l].m + 1, kTlUp);
    k_tl_up<float><<<t * t, kTlTileThreads, 0, s>>>(tl.lev[l], tl.lev[l + 1], done);
    count_launch();
  }
  SIPG_TL_DISPATCH(tl_launch_finish, float, tl.p, op->tab, st ? 1 : 0, r, z, tl.lev[0].y, tl.fdm, dim, st, red, s)
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  return SIPG_OK;
}

// Enqueues the restriction of r into the preconditioner's corner sums (what a
// twolevel_enqueue with cp_ready expects).
sipg_status twolevel_enqueue_restrict(const sipg_op* op, const void* handle, const float* r, cudaStream_t s) {
  const TwoLevel& tl = *static_cast<const TwoLevel*>(handle);
  const size_t noe = (size_t)tl.dim * tl.dim;
  SIPG_TL_DISPATCH(tl_launch_restrict_elem, float, tl.p, op->tab, r, tl.cp, noe, nullptr, s)
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  return SIPG_OK;
}

// Enqueues the inner PCG update x += alpha p, r -= alpha Ap with r.r, the stop
// test and the restriction of the new r (the next z = M r then runs with
// cp_ready).
sipg_status twolevel_enqueue_update(const sipg_op* op, const void* handle, float* x, const float* pb0,
                                    const float* pb1, float* r, const float* Ap, CgState<float>* st,
                                    const ReduceScratch& red, cudaStream_t s) {
  const TwoLevel& tl = *static_cast<const TwoLevel*>(handle);
  const size_t noe = (size_t)tl.dim * tl.dim;
  SIPG_TL_DISPATCH(tl_launch_update_restrict, float, tl.p, op->tab, x, pb0, pb1, r, Ap, tl.cp, noe, st, red, s)
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  return SIPG_OK;
}


// ---- many instances ----

namespace {
size_t round16(size_t n) { return (n + 3) & ~size_t(3); }  // floats, to a 16-byte multiple
}  // namespace

size_t twolevel_scratch_floats_for(int dim) {
  size_t n = round16(4 * (size_t)dim * dim);
  for (int m = dim;; m = (m + 1) / 2) {
    n += 3 * round16((size_t)(m + 1) * (m + 1));
    if (m <= kTlCoarsestCells) break;
  }
  return n;
}

size_t twolevel_scratch_floats(const void* handle) {
  const TwoLevel& tl = *static_cast<const TwoLevel*>(handle);
  size_t n = round16(4 * (size_t)tl.dim * tl.dim);
  for (const TlLev<float>& L : tl.lev) n += 3 * round16((size_t)(L.m + 1) * (L.m + 1));
  return n;
}

TlInst twolevel_inst(const void* handle, float* scratch, const float* r, float* z, CgState<float>* st,
                     const ReduceScratch& red) {
  const TwoLevel& tl = *static_cast<const TwoLevel*>(handle);
  TlInst v{};
  v.r = r;
  v.z = z;
  v.fdm = tl.fdm;
  v.ainv = tl.ainv;
  v.st = st;
  v.red = red;
  v.dim = tl.dim;
  v.p = tl.p;
  v.nl = (int)tl.lev.size();
  v.tail0 = tl.tail0;
  v.nblk = tl_grid((size_t)tl.dim * tl.dim, kTlElemThreads, red.capacity);
  float* q = scratch;
  v.cp = q;
  q += round16(4 * (size_t)tl.dim * tl.dim);
  for (int l = 0; l < v.nl; ++l) {
    const size_t nv = round16((size_t)(tl.lev[l].m + 1) * (tl.lev[l].m + 1));
    v.lev[l] = tl.lev[l];  // m, S, wd shared with the op
    v.lev[l].b = q;
    v.lev[l].x = q + nv;
    v.lev[l].y = q + 2 * nv;
    q += 3 * nv;
  }
  return v;
}

TlPlan twolevel_plan(const TlInst* h, const HostTables* const* tabs, int n) {
  TlPlan plan;
  plan.n = n;
  for (int i = 0; i < n; ++i) {
    plan.maxl = std::max(plan.maxl, h[i].nl);
    plan.nblk_max = std::max(plan.nblk_max, h[i].nblk);
    plan.max_tail0 = std::max(plan.max_tail0, h[i].tail0);
    if ((int)plan.side_max.size() < h[i].nl) plan.side_max.resize(h[i].nl, 0);
    for (int l = 0; l < h[i].nl; ++l) plan.side_max[l] = std::max(plan.side_max[l], h[i].lev[l].m + 1);
    if (plan.groups.empty() || plan.groups.back().p != h[i].p) plan.groups.push_back({h[i].p, i, 0, 0, tabs[i]});
    TlPlan::Group& g = plan.groups.back();
    g.count += 1;
    g.nblk_max = std::max(g.nblk_max, h[i].nblk);
  }
  return plan;
}

template <int P>
void tlb_elem_launch(int which, const TlInst* d, const TlPlan::Group& g, cudaStream_t s) {
  const dim3 grid(g.nblk_max, g.count);
  if (which == 0)
    k_tlb_restrict_elem<P><<<grid, kTlElemThreads, 0, s>>>(d, g.first, tl_hat<float, P>(*g.tab));
  else
    k_tlb_finish<P><<<grid, kTlElemThreads, 0, s>>>(d, g.first, tl_hat<float, P>(*g.tab));
}

// One batched element kernel (0: restriction, 1: finish) for every degree
// group of the plan.
void tlb_elem_all(int which, const TlInst* d, const TlPlan& plan, cudaStream_t s) {
  for (const TlPlan::Group& g : plan.groups) {
    switch (g.p) {
      case 1: tlb_elem_launch<1>(which, d, g, s); break;
      case 2: tlb_elem_launch<2>(which, d, g, s); break;
      case 3: tlb_elem_launch<3>(which, d, g, s); break;
      case 4: tlb_elem_launch<4>(which, d, g, s); break;
      case 5: tlb_elem_launch<5>(which, d, g, s); break;
      case 6: tlb_elem_launch<6>(which, d, g, s); break;
      case 7: tlb_elem_launch<7>(which, d, g, s); break;
      case 8: tlb_elem_launch<8>(which, d, g, s); break;
    }
  }
  count_launch(plan.groups.size());
}

sipg_status twolevel_enqueue_batched(const TlInst* d, const TlPlan& plan, cudaStream_t s) {
  if (plan.n == 0) return SIPG_OK;
  const int n = plan.n;
  tlb_elem_all(0, d, plan, s);
  auto tiles = [&](int l, int tile) {
    const int t = tl_tiles(plan.side_max[l], tile);
    return dim3(t * t, n);
  };
  for (int l = 0; l < plan.max_tail0; ++l) {
    k_tlb_down<<<tiles(l + 1, kTlDown), kTlTileThreads, 0, s>>>(d, l);
    count_launch();
  }
  k_tlb_tail<<<dim3(1, n), kTlTailThreads, 0, s>>>(d);
  count_launch();
  for (int l = plan.max_tail0 - 1; l >= 0; --l) {
    k_tlb_up<<<tiles(l, kTlUp), kTlTileThreads, 0, s>>>(d, l);
    count_launch();
  }
  tlb_elem_all(1, d, plan, s);
  SIPG_CUDA_TRY(cudaGetLastError());
  return SIPG_OK;
}

}  // namespace sipg

extern "C" sipg_status sipg_apply_twolevel_f32(sipg_op* op, const float* d_r, float* d_z, void* stream) {
  if (!op || !d_r || !d_z || d_r == d_z) {
    set_error("sipg_apply_twolevel_f32: null or aliased vectors");
    return SIPG_ERR_INVALID;
  }
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  void* tl = nullptr;
  sipg_status st = twolevel_get(op, &tl);
  if (st != SIPG_OK) return st;
  return twolevel_enqueue(op, tl, d_r, d_z, nullptr, ReduceScratch{}, (cudaStream_t)stream, false);
}
