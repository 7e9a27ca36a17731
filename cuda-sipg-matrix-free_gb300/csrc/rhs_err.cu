// rhs_err.cu -- the steps either side of the solve, on the device:
//   k_rhs:       the right-hand side of sipg_sem_2d<T>::compute_rhs
//                (sipg_sem_2d.hpp:232-305): quadrature of f, plus the Nitsche
//                terms of the Dirichlet data on the four boundary strips;
//   k_err_norms: sipg_sem_2d<T>::err_norms (sipg_sem_2d.hpp:311-370): max
//                nodal error and LGL-quadrature L2 / broken-H1 errors.
// One thread per element; element corner coordinates are the reference's
// accumulated sums (build_square_mesh.hpp:250-288), computed on the host and
// passed in as one x per column and one y per row.
#include <cmath>
#include <cstring>
#include <vector>

#include "sipg_internal.cuh"

namespace sipg {

struct ProblemArgs {
  int sol;
  sipg_modes modes;
};

// u, f, du/dx, du/dy of the test problems (analytical_solutions.hpp:7-94 for
// A..E, with the reference's PI literal).
__device__ void eval_problem(const ProblemArgs& pa, double x, double y, double* u, double* f, double* dx, double* dy) {
  const double PI = 3.14159265359;
  switch (pa.sol) {
    case SIPG_SOL_A: {
      const double ex = exp(x - y);
      *u = x * y * (y - 1) * (x - 1) * ex;
      *f = -2 * x * (y - 1) * (y - 2 * x + x * y + 2) * ex;
      *dx = (x * x + x - 1) * (y - 1) * y * ex;
      *dy = -1 * (y * y - 3 * y + 1) * (x - 1) * x * ex;
      break;
    }
    case SIPG_SOL_B: {
      const double e3 = exp(3 * x), s = sin(2 * PI * y);
      *u = x * (1 - x) * e3 * s;
      *f = -s * e3 * ((4 - 3 * x - 9 * x * x) - 4 * PI * PI * (x - x * x));
      *dx = (3 * (1 - x) * x - x + (1 - x)) * e3 * s;
      *dy = 2 * PI * (1 - x) * x * e3 * cos(2 * PI * y);
      break;
    }
    case SIPG_SOL_C:
      *u = y * (1 - y) * x * x * x;
      *f = 2 * x * x * x - 6 * x * y * (1 - y);
      *dx = y * (1 - y) * x * x * 3;
      *dy = (1 - 2 * y) * x * x * x;
      break;
    case SIPG_SOL_D:
      *u = x * x * y * y;
      *f = -2 * y * y - 2 * x * x;
      *dx = 2 * x * y * y;
      *dy = 2 * y * x * x;
      break;
    case SIPG_SOL_E:
      *u = cos(8 * PI * x) + cos(8 * PI * y);
      *f = 64 * PI * PI * cos(8 * PI * x) + 64 * PI * PI * cos(8 * PI * y);
      *dx = -8 * PI * sin(8 * PI * x);
      *dy = -8 * PI * sin(8 * PI * y);
      break;
    case SIPG_SOL_SINSIN: {
      const double tp = 2 * M_PI;
      const double sx = sin(tp * x), sy = sin(tp * y);
      *u = sx * sy;
      *f = 2 * tp * tp * sx * sy;
      *dx = tp * cos(tp * x) * sy;
      *dy = tp * sx * cos(tp * y);
      break;
    }
    case SIPG_SOL_MODES: {
      double su = 0, sf = 0, sx = 0, sy = 0;
      for (int q = 0; q < pa.modes.nmodes; ++q) {
        const double kx = pa.modes.k[q] * M_PI, ly = pa.modes.l[q] * M_PI;
        const double A = pa.modes.amp[q], lam = kx * kx + ly * ly;
        const double s1 = sin(kx * x), s2 = sin(ly * y);
        sf += A * s1 * s2;
        su += A / lam * s1 * s2;
        sx += A / lam * kx * cos(kx * x) * s2;
        sy += A / lam * ly * s1 * cos(ly * y);
      }
      *u = su;
      *f = sf;
      *dx = sx;
      *dy = sy;
      break;
    }
    default:
      *u = *f = *dx = *dy = 0;
  }
}

__device__ __forceinline__ double prob_u(const ProblemArgs& pa, double x, double y) {
  double u, f, dx, dy;
  eval_problem(pa, x, y, &u, &f, &dx, &dy);
  return u;
}

struct RhsTables {
  double nodes[SIPG_MAX_N];    // (xi*.5 + .5)/dim
  double weights[SIPG_MAX_N];  // raw LGL weights
  double w[SIPG_MAX_N];        // weights * .5 / dim
  double D[SIPG_MAX_N * SIPG_MAX_N];
};

__global__ void k_rhs(double* __restrict__ b, int p, int dim, double pen, const __grid_constant__ ProblemArgs pa,
                      const __grid_constant__ RhsTables tb, const double* __restrict__ xcol,
                      const double* __restrict__ yrow) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int noe = dim * dim;
  if (e >= noe) return;
  const int n = p + 1, N = p;
  const int row = e / dim, col = e % dim;
  const double xe = xcol[col], ye = yrow[row];
  const size_t NOE = (size_t)noe;
  auto B = [&](int i1, int i2) -> double& { return b[((size_t)i1 * n + i2) * NOE + e]; };
  for (int i1 = 0; i1 <= N; ++i1)
    for (int i2 = 0; i2 <= N; ++i2) {
      double u, f, dx, dy;
      eval_problem(pa, xe + tb.nodes[i1], ye + tb.nodes[i2], &u, &f, &dx, &dy);
      B(i1, i2) = tb.w[i1] * tb.w[i2] * f;
    }
  // Boundary strips, in the reference's order: by strip position xx, then per
  // face node i the penalty terms (DOWN, UP, LEFT, RIGHT), then per normal node
  // j the consistency terms.  An element is touched at most at two xx values.
  const bool isD = row == dim - 1, isU = row == 0, isL = col == 0, isR = col == dim - 1;
  if (!(isD || isU || isL || isR)) return;
  int xs[2], nx = 0;
  auto add_x = [&](int v) {
    for (int q = 0; q < nx; ++q)
      if (xs[q] == v) return;
    xs[nx++] = v;
  };
  if (isD) add_x(col);
  if (isU) add_x(col);
  if (isL) add_x(row);
  if (isR) add_x(row);
  if (nx == 2 && xs[1] < xs[0]) {
    const int tmp = xs[0];
    xs[0] = xs[1];
    xs[1] = tmp;
  }
  for (int q = 0; q < nx; ++q) {
    const int xx = xs[q];
    const bool D = isD && col == xx, U = isU && col == xx, L = isL && row == xx, R = isR && row == xx;
    for (int i = 0; i <= N; ++i) {
      const double gD = D ? prob_u(pa, xe + tb.nodes[i], ye + tb.nodes[0]) : 0.0;
      const double gU = U ? prob_u(pa, xe + tb.nodes[i], ye + tb.nodes[N]) : 0.0;
      const double gL = L ? prob_u(pa, xe + tb.nodes[0], ye + tb.nodes[i]) : 0.0;
      const double gR = R ? prob_u(pa, xe + tb.nodes[N], ye + tb.nodes[i]) : 0.0;
      if (D) B(i, 0) += pen * tb.weights[i] * gD;
      if (U) B(i, N) += pen * tb.weights[i] * gU;
      if (L) B(0, i) += pen * tb.weights[i] * gL;
      if (R) B(N, i) += pen * tb.weights[i] * gR;
      for (int j = 0; j <= N; ++j) {
        if (D) B(i, j) -= -1 * tb.weights[i] * tb.D[j * n + 0] * gD;
        if (U) B(i, j) -= tb.weights[i] * tb.D[j * n + N] * gU;
        if (L) B(j, i) -= -1 * tb.weights[i] * tb.D[j * n + 0] * gL;
        if (R) B(j, i) -= tb.weights[i] * tb.D[j * n + N] * gR;
      }
    }
  }
}

constexpr int kErrThreads = 128;

__global__ void __launch_bounds__(kErrThreads)
    k_err_norms(const double* __restrict__ u, int p, int dim, const __grid_constant__ ProblemArgs pa,
                const __grid_constant__ RhsTables tb, const double* __restrict__ xcol,
                const double* __restrict__ yrow, double* __restrict__ partial /* [grid][4] */) {
  __shared__ double sh[4][kErrThreads / 32];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int noe = dim * dim;
  double l2 = 0, dxs = 0, dys = 0, mx = -1;
  if (e < noe) {
    const int n = p + 1, N = p;
    const int row = e / dim, col = e % dim;
    const double xe = xcol[col], ye = yrow[row];
    const size_t NOE = (size_t)noe;
    auto Uv = [&](int i1, int i2) -> double { return u[((size_t)i1 * n + i2) * NOE + e]; };
    for (int pp = 0; pp <= N; ++pp)
      for (int q = 0; q <= N; ++q) {
        double dx_u = 0, dy_u = 0;
        const double w2 = tb.w[pp] * tb.w[q];
        for (int i = 0; i <= N; ++i) {
          dx_u += Uv(i, q) * 2 * dim * tb.D[i * n + pp];
          dy_u += Uv(pp, i) * 2 * dim * tb.D[i * n + q];
        }
        double ue, fe, dxe, dye;
        eval_problem(pa, xe + tb.nodes[pp], ye + tb.nodes[q], &ue, &fe, &dxe, &dye);
        const double err = fabs(Uv(pp, q) - ue);
        mx = fmax(mx, err);
        l2 += w2 * err * err;
        dxs += w2 * (dx_u - dxe) * (dx_u - dxe);
        dys += w2 * (dy_u - dye) * (dy_u - dye);
      }
  }
  for (int o = 16; o > 0; o >>= 1) {
    l2 += __shfl_xor_sync(0xffffffffu, l2, o);
    dxs += __shfl_xor_sync(0xffffffffu, dxs, o);
    dys += __shfl_xor_sync(0xffffffffu, dys, o);
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][w] = l2;
    sh[1][w] = dxs;
    sh[2][w] = dys;
    sh[3][w] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, bsum = 0, c = 0, m = -1;
    for (int k = 0; k < kErrThreads / 32; ++k) {
      a += sh[0][k];
      bsum += sh[1][k];
      c += sh[2][k];
      m = fmax(m, sh[3][k]);
    }
    partial[4 * blockIdx.x + 0] = a;
    partial[4 * blockIdx.x + 1] = bsum;
    partial[4 * blockIdx.x + 2] = c;
    partial[4 * blockIdx.x + 3] = m;
  }
}

static RhsTables make_rhs_tables(const HostTables& h, int dim) {
  RhsTables t;
  const int n = h.p + 1;
  for (int i = 0; i < n; ++i) {
    t.nodes[i] = (h.nodes[i] * .5 + .5) / dim;
    t.weights[i] = h.w[i];
    t.w[i] = h.w[i] * .5 / dim;
  }
  for (int i = 0; i < n * n; ++i) t.D[i] = h.D[i];
  return t;
}

// One x per column and one y per row, accumulated as square_mesh does.
static void mesh_axes(int dim, std::vector<double>& xcol, std::vector<double>& yrow) {
  xcol.resize(dim);
  yrow.resize(dim);
  const double delta = 1. / (double)dim;
  double xx = 0;
  for (int j = 0; j < dim; ++j) {
    xcol[j] = xx;
    xx += delta;
  }
  double yy = 1;
  for (int i = 0; i < dim; ++i) {
    yy -= delta;
    yrow[i] = yy;
  }
}

// The same axes on the device (one thread per axis, the same additions in
// the same order: bit-identical to mesh_axes).
__global__ void k_mesh_axes(double* __restrict__ xcol, double* __restrict__ yrow, int dim) {
  const double delta = 1. / (double)dim;
  if (threadIdx.x == 0) {
    double xx = 0;
    for (int j = 0; j < dim; ++j) {
      xcol[j] = xx;
      xx += delta;
    }
  } else if (threadIdx.x == 1) {
    double yy = 1;
    for (int i = 0; i < dim; ++i) {
      yy -= delta;
      yrow[i] = yy;
    }
  }
}

// Stream-ordered throughout (no host synchronisation): a right-hand side
// queued behind other work on s, or beside other streams' work, waits for
// nothing.
sipg_status rhs_f64(const sipg_op* op, int sol, const sipg_modes* modes, double* d_b, cudaStream_t s) {
  double* d_axes = nullptr;
  SIPG_CUDA_TRY(cudaMallocAsync((void**)&d_axes, sizeof(double) * 2 * op->dim, s));
  k_mesh_axes<<<1, 2, 0, s>>>(d_axes, d_axes + op->dim, op->dim);
  count_launch();
  ProblemArgs pa;
  pa.sol = sol;
  std::memset(&pa.modes, 0, sizeof(pa.modes));
  if (modes) pa.modes = *modes;
  const RhsTables tb = make_rhs_tables(op->tab, op->dim);
  const int threads = 128, blocks = (int)((op->noe + threads - 1) / threads);
  k_rhs<<<blocks, threads, 0, s>>>(d_b, op->p, op->dim, op->pen, pa, tb, d_axes, d_axes + op->dim);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  SIPG_CUDA_TRY(cudaFreeAsync(d_axes, s));
  return SIPG_OK;
}

sipg_status err_norms_f64(const sipg_op* op, int sol, const sipg_modes* modes, const double* d_u, double* err,
                          cudaStream_t s) {
  std::vector<double> xc, yr;
  mesh_axes(op->dim, xc, yr);
  const int blocks = (int)((op->noe + kErrThreads - 1) / kErrThreads);
  double* d_buf = nullptr;
  SIPG_CUDA_TRY(cudaMallocAsync((void**)&d_buf, sizeof(double) * (2 * op->dim + 4 * (size_t)blocks), s));
  SIPG_CUDA_TRY(cudaMemcpyAsync(d_buf, xc.data(), sizeof(double) * op->dim, cudaMemcpyHostToDevice, s));
  SIPG_CUDA_TRY(cudaMemcpyAsync(d_buf + op->dim, yr.data(), sizeof(double) * op->dim, cudaMemcpyHostToDevice, s));
  ProblemArgs pa;
  pa.sol = sol;
  std::memset(&pa.modes, 0, sizeof(pa.modes));
  if (modes) pa.modes = *modes;
  const RhsTables tb = make_rhs_tables(op->tab, op->dim);
  double* d_part = d_buf + 2 * op->dim;
  k_err_norms<<<blocks, kErrThreads, 0, s>>>(d_u, op->p, op->dim, pa, tb, d_buf, d_buf + op->dim, d_part);
  count_launch();
  SIPG_CUDA_TRY(cudaGetLastError());
  std::vector<double> part(4 * (size_t)blocks);
  SIPG_CUDA_TRY(cudaMemcpyAsync(part.data(), d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s));
  SIPG_CUDA_TRY(cudaStreamSynchronize(s));
  SIPG_CUDA_TRY(cudaFreeAsync(d_buf, s));
  double l2 = 0, dx = 0, dy = 0, mx = -1;
  for (int k = 0; k < blocks; ++k) {
    l2 += part[4 * k + 0];
    dx += part[4 * k + 1];
    dy += part[4 * k + 2];
    mx = std::fmax(mx, part[4 * k + 3]);
  }
  err[0] = std::sqrt(l2);
  err[1] = std::sqrt(l2 + dx + dy);
  err[2] = mx;
  return SIPG_OK;
}

}  // namespace sipg
