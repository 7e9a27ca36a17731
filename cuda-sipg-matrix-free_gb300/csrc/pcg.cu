// pcg.cu -- the reference's block-Jacobi preconditioned CG (its
// USE_PRECONDITIONER path), on the device.
//
// The preconditioner (laplacian_operator.hpp:95-186, mode_matrix.hpp:474-522):
// the diagonal block of an interior element -- element Laplacian, the four
// faces' consistency terms with the interior factor 1/2, the penalty on the
// face nodes -- is inverted once on the host (LU with partial pivoting and
// substitution, the computation of LAPACK's dgetrf + dgetri that the reference
// calls), and the inverse is kept only on the "cross" pattern of the
// stored-operator kernel: for output node (i1,i2) the entries at (i1,i2), at
// (i1,j) and at (j,i2), 2p+1 per row.  z = M r applies those rows element by
// element (the reference runs volume_mvm<T,1>, mode_matrix_kernels.hpp:7-65).
// As in the reference the same rows serve every element, boundary ones
// included, and the penalty is truncated to an integer first (the
// preconditioner's constructor takes `int _pen`, laplacian_operator.hpp:116).
//
// The iteration (conjugate_gradient_gpu.hpp:116-213) as four kernels,
// captured K at a time in a CUDA graph with every scalar on the device:
//   k_sipg_apply<APPLY_DOT>: Ap, p.Ap, alpha = (r.z) / p.Ap
//   k_pcg_update:            x += alpha p, r -= alpha Ap, r.r (the stop test)
//   k_cross_apply<P, 1>:     z = M r, r.z, beta = (r.z)_new / (r.z)_old
//   k_cg_direction:          p = z + beta p
#include <cmath>
#include <new>
#include <vector>

#include "sipg_cg.cuh"

using namespace sipg;

namespace sipg {
cudaError_t launch_apply_f64(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>& a, const HostTables& h,
                             cudaStream_t s);

namespace {

// The preconditioner rows of degree p at rows[((i1*n + i2)*(2p+1)) + r]:
// r = 0 the diagonal, then (i1, j) for j != i2, then (j, i2) for j != i1.
int build_prec_rows(const HostTables& t, double pen_in, std::vector<double>& rows) {
  const int N = t.p, n = N + 1, nn = n * n, R = 2 * N + 1;
  const double pen = (double)(int)pen_in;
  const double* w = t.w;
  const double* D = t.D;  // D[mode * n + node]
  std::vector<double> a((size_t)nn * nn, 0.0);
  auto at = [&](int i1, int i2, int j1, int j2) -> double& {
    return a[(size_t)nn * (n * i2 + i1) + (n * j2 + j1)];
  };
  // element Laplacian: w_i2 K(i1,j1) on equal i2, w_i1 K(i2,j2) on equal i1
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2)
      for (int j1 = 0; j1 < n; ++j1)
        for (int j2 = 0; j2 < n; ++j2) {
          double v = 0.0;
          if (i2 == j2)
            for (int k = 0; k < n; ++k) v += w[k] * w[i2] * D[i1 * n + k] * D[j1 * n + k];
          if (i1 == j1)
            for (int k = 0; k < n; ++k) v += w[k] * w[i1] * D[i2 * n + k] * D[j2 * n + k];
          at(i1, i2, j1, j2) = v;
        }
  // consistency terms of the four faces (interior factor 1/2), symmetric
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      const double l = 0.5 * w[j] * D[i * n + 0], r = 0.5 * w[j] * D[i * n + N];
      at(i, j, 0, j) += l;
      at(0, j, i, j) += l;
      at(i, j, N, j) -= r;
      at(N, j, i, j) -= r;
      at(j, i, j, 0) += l;
      at(j, 0, j, i) += l;
      at(j, i, j, N) -= r;
      at(j, N, j, i) -= r;
    }
  // penalty on the face nodes
  for (int i = 0; i < n; ++i) {
    at(N, i, N, i) += pen * w[i];
    at(i, N, i, N) += pen * w[i];
    at(0, i, 0, i) += pen * w[i];
    at(i, 0, i, 0) += pen * w[i];
  }
  // inverse: LU with partial pivoting, then substitution per column
  std::vector<int> piv(nn);
  for (int c = 0; c < nn; ++c) {
    int pr = c;
    for (int r = c + 1; r < nn; ++r)
      if (std::fabs(a[(size_t)r * nn + c]) > std::fabs(a[(size_t)pr * nn + c])) pr = r;
    piv[c] = pr;
    if (a[(size_t)pr * nn + c] == 0.0) return -1;
    if (pr != c)
      for (int k = 0; k < nn; ++k) std::swap(a[(size_t)c * nn + k], a[(size_t)pr * nn + k]);
    for (int r = c + 1; r < nn; ++r) {
      const double f = a[(size_t)r * nn + c] / a[(size_t)c * nn + c];
      a[(size_t)r * nn + c] = f;
      for (int k = c + 1; k < nn; ++k) a[(size_t)r * nn + k] -= f * a[(size_t)c * nn + k];
    }
  }
  std::vector<double> inv((size_t)nn * nn), col(nn);
  for (int j = 0; j < nn; ++j) {
    for (int i = 0; i < nn; ++i) col[i] = (i == j) ? 1.0 : 0.0;
    for (int i = 0; i < nn; ++i) std::swap(col[i], col[piv[i]]);
    for (int i = 0; i < nn; ++i)
      for (int k = 0; k < i; ++k) col[i] -= a[(size_t)i * nn + k] * col[k];
    for (int i = nn - 1; i >= 0; --i) {
      for (int k = i + 1; k < nn; ++k) col[i] -= a[(size_t)i * nn + k] * col[k];
      col[i] /= a[(size_t)i * nn + i];
    }
    for (int i = 0; i < nn; ++i) inv[(size_t)i * nn + j] = col[i];
  }
  auto M = [&](int i1, int i2, int j1, int j2) { return inv[(size_t)nn * (n * i2 + i1) + (n * j2 + j1)]; };
  rows.assign((size_t)nn * R, 0.0);
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2) {
      double* row = &rows[(size_t)(i1 * n + i2) * R];
      int r = 0;
      row[r] = M(i1, i2, i1, i2);
      for (int j = 0; j < n; ++j)
        if (j != i2) row[++r] = M(i1, i2, i1, j);
      for (int j = 0; j < n; ++j)
        if (j != i1) row[++r] = M(i1, i2, j, i2);
    }
  return 0;
}
}  // namespace

// The cross-pattern operators -- the stored volume operator of
// volume_mvm<T, same> (mode_matrix_kernels.hpp:7-65) and the block-Jacobi
// preconditioner applied the same way (sipg_sem_2d.hpp:205-224) -- with value
// r of row (i1,i2) of element e's operator at
// mat[((i1*n + i2)*(2p+1) + r)*mat_noe + (mat_noe == 1 ? 0 : e)] (the
// reference's mode_matrix layout; one operator for every element, mat_noe =
// 1, or one per element, mat_noe = noe) and out(i1,i2,e) = diagonal, then the
// row (i1, j != i2), then the column (j != i1, i2), in the reference kernel's
// order.
//
// One thread per element, kCrossThreads consecutive elements per block: each
// thread first copies its element's n^2 input values into its own column of
// shared memory (plane by plane, so every load is a coalesced run of
// consecutive elements), then forms the n^2 outputs from there.  Every input
// value is read from HBM once (16 B/DoF with the write; per-element operators
// add their (2p+1) values per DoF) -- where a thread per DoF reads each value
// 2p+1 times, from planes far apart in the vector.  A thread reads only the
// column it wrote, so no barrier is needed.  MODE 1 (the PCG step) also forms
// r.z, its deterministic grid reduction and the step's beta.
constexpr int kCrossThreads = 64;

template <int P, int MODE>
__global__ void __launch_bounds__(kCrossThreads)
    k_cross_apply(const double* __restrict__ mat, size_t mat_noe, const double* __restrict__ in,
                  double* __restrict__ out, size_t noe, CgState<double>* st, ReduceScratch red) {
  constexpr int N1 = P + 1, NN = N1 * N1, R = 2 * P + 1;
  __shared__ double col[NN][kCrossThreads];
  __shared__ double sh[32];
  if (MODE == 1 && *(volatile int*)&st->done) return;
  const int t = threadIdx.x;
  const size_t tiles = (noe + kCrossThreads - 1) / kCrossThreads;
  double acc = 0.0;
  for (size_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const size_t e = tile * kCrossThreads + t;
    if (e < noe) {
#pragma unroll
      for (int k = 0; k < NN; ++k) col[k][t] = __ldg(in + (size_t)k * noe + e);
      const size_t me = (mat_noe == 1) ? 0 : e;
#pragma unroll 1
      for (int k = 0; k < NN; ++k) {
        const int i1 = k / N1, i2 = k - i1 * N1;
        const double* row = mat + (size_t)k * R * mat_noe + me;
        int q = 0;
        double v = 0.0;
        v += __ldg(row) * col[k][t];
#pragma unroll
        for (int j = 0; j < N1; ++j)
          if (j != i2) v += __ldg(row + (size_t)(++q) * mat_noe) * col[i1 * N1 + j][t];
#pragma unroll
        for (int j = 0; j < N1; ++j)
          if (j != i1) v += __ldg(row + (size_t)(++q) * mat_noe) * col[j * N1 + i2][t];
        out[(size_t)k * noe + e] = v;
        if (MODE == 1) acc = fma(v, col[k][t], acc);
      }
    }
  }
  if (MODE == 1) {
    const double bt = block_sum<double, kCrossThreads>(acc, sh);
    double total;
    if (grid_sum_last<double, kCrossThreads>(bt, red, gridDim.x, sh, &total) && t == 0) {
      if (!st->first) st->beta = total / st->rr;
      st->rr = total;
      if (!isfinite(total)) {
        st->status = (int)SIPG_ERR_BREAKDOWN;
        st->done = 1;
      }
    }
  }
}

// Launches the cross-pattern operator of degree p; mode 0: out = M in, mode
// 1: z = M r with r.z and beta into st (its reduction over at most
// red.capacity blocks).
cudaError_t launch_cross(int p, int mode, const double* mat, size_t mat_noe, const double* in, double* out,
                         size_t noe, CgState<double>* st, const ReduceScratch& red, cudaStream_t s) {
  const size_t tiles = (noe + kCrossThreads - 1) / kCrossThreads;
  size_t cap = 152 * 32;
  if (mode == 1 && (size_t)red.capacity < cap) cap = (size_t)red.capacity;
  const int grid = (int)std::max<size_t>(1, std::min(tiles, cap));
#define SIPG_CROSS_CASE(PP)                                                                     \
  case PP:                                                                                      \
    if (mode == 1)                                                                              \
      k_cross_apply<PP, 1><<<grid, kCrossThreads, 0, s>>>(mat, mat_noe, in, out, noe, st, red); \
    else                                                                                        \
      k_cross_apply<PP, 0><<<grid, kCrossThreads, 0, s>>>(mat, mat_noe, in, out, noe, st, red); \
    break;
  switch (p) {
    SIPG_CROSS_CASE(1)
    SIPG_CROSS_CASE(2)
    SIPG_CROSS_CASE(3)
    SIPG_CROSS_CASE(4)
    SIPG_CROSS_CASE(5)
    SIPG_CROSS_CASE(6)
    SIPG_CROSS_CASE(7)
    SIPG_CROSS_CASE(8)
    default:
      return cudaErrorInvalidValue;
  }
#undef SIPG_CROSS_CASE
  count_launch();
  return cudaGetLastError();
}

// After r = b - A x: the reference's loop test starts from rr = 1 rather than
// the residual (conjugate_gradient_gpu.hpp:160-165), so its first iteration
// runs whenever the tolerance is below 1; an exactly zero residual stops here
// (its first step would divide 0 by 0).
__global__ void k_pcg_force_start(CgState<double>* st, int max_it) {
  const double rr0 = st->rr;
  st->rres = rr0;
  st->done = !(1.0 > st->stop && 0 < max_it) || rr0 == 0.0 || st->status != (int)SIPG_OK;
}

// x += alpha p, r -= alpha Ap, r.r; it++, and the stop test on sqrt(r.r)
__global__ void __launch_bounds__(kVecThreads) k_pcg_update(double* __restrict__ x, const double* __restrict__ pv,
                                                            double* __restrict__ r, const double* __restrict__ Ap,
                                                            size_t n, CgState<double>* st, ReduceScratch red) {
  __shared__ double sh[32];
  if (*(volatile int*)&st->done) return;
  const double alpha = st->alpha;
  double acc = 0.0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] = fma(alpha, pv[i], x[i]);
    const double ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    acc = fma(ri, ri, acc);
  }
  const double bt = block_sum<double, kVecThreads>(acc, sh);
  double total;
  if (grid_sum_last<double, kVecThreads>(bt, red, gridDim.x, sh, &total) && threadIdx.x == 0) {
    st->it += 1;
    st->first = 0;
    st->rres = total;
    st->done = !(sqrt(total) > st->stop && st->it < st->max_it);
    if (!isfinite(total)) {
      st->status = (int)SIPG_ERR_BREAKDOWN;
      st->done = 1;
    }
  }
}
}  // namespace sipg

namespace {
struct PcgCache {
  size_t n = 0;
  double* rows = nullptr;  // (p+1)^2 x (2p+1)
  double rows_pen = NAN;
  double *r = nullptr, *z = nullptr, *p = nullptr, *Ap = nullptr;
  CgState<double>* st = nullptr;
  CgState<double>* st_host = nullptr;
  ReduceScratch red{};
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
  double* exec_x = nullptr;
  int exec_k = 0, exec_gen = -1;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ~PcgCache() {
    if (exec) cudaGraphExecDestroy(exec);
    if (cap) cudaStreamDestroy(cap);
    cudaFree(rows);
    cudaFree(r);
    cudaFree(z);
    cudaFree(p);
    cudaFree(Ap);
    cudaFree(st);
    cudaFreeHost(st_host);
    cudaFree(red.partials);
    cudaFree(red.counter);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }
};

void pcg_cache_free(void* c) { delete static_cast<PcgCache*>(c); }

int vec_grid(size_t n) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + kVecThreads - 1) / kVecThreads, 152 * 8));
}

// the op's preconditioner rows on the device (built on first use)
sipg_status ensure_rows(sipg_op* op, PcgCache& c) {
  if (c.rows && c.rows_pen == op->pen) return SIPG_OK;
  std::vector<double> rows;
  if (build_prec_rows(op->tab, op->pen, rows)) {
    set_error("block-Jacobi preconditioner: singular diagonal block");
    return SIPG_ERR_INVALID;
  }
  if (!c.rows) SIPG_CUDA_TRY(cudaMalloc(&c.rows, rows.size() * sizeof(double)));
  SIPG_CUDA_TRY(cudaMemcpy(c.rows, rows.data(), rows.size() * sizeof(double), cudaMemcpyHostToDevice));
  c.rows_pen = op->pen;
  return SIPG_OK;
}

sipg_status cache_get(sipg_op* op, bool vectors, PcgCache** out) {
  std::lock_guard<std::mutex> lk(op->mu);
  if (!op->pcg) {
    PcgCache* c = new (std::nothrow) PcgCache;
    if (!c) return SIPG_ERR_NOMEM;
    op->pcg = c;
    op->pcg_free = pcg_cache_free;
  }
  PcgCache& c = *static_cast<PcgCache*>(op->pcg);
  sipg_status st = ensure_rows(op, c);
  if (st != SIPG_OK) return st;
  if (vectors && !c.r) {
    const size_t n = (size_t)op->ndof, bytes = n * sizeof(double);
    const int cap = reduce_capacity(op->dim);
    c.n = n;
    SIPG_CUDA_TRY(cudaMalloc(&c.r, bytes));
    SIPG_CUDA_TRY(cudaMalloc(&c.z, bytes));
    SIPG_CUDA_TRY(cudaMalloc(&c.p, bytes));
    SIPG_CUDA_TRY(cudaMalloc(&c.Ap, bytes));
    SIPG_CUDA_TRY(cudaMalloc(&c.st, sizeof(CgState<double>)));
    SIPG_CUDA_TRY(cudaMemset(c.st, 0, sizeof(CgState<double>)));
    SIPG_CUDA_TRY(cudaMallocHost(&c.st_host, sizeof(CgState<double>)));
    SIPG_CUDA_TRY(cudaMalloc(&c.red.partials, sizeof(double) * cap));
    SIPG_CUDA_TRY(cudaMalloc(&c.red.counter, sizeof(unsigned int)));
    SIPG_CUDA_TRY(cudaMemset(c.red.counter, 0, sizeof(unsigned int)));
    c.red.capacity = cap;
    SIPG_CUDA_TRY(cudaStreamCreateWithFlags(&c.cap, cudaStreamNonBlocking));
    SIPG_CUDA_TRY(cudaEventCreate(&c.ev0));
    SIPG_CUDA_TRY(cudaEventCreate(&c.ev1));
  }
  *out = &c;
  return SIPG_OK;
}

sipg_status enqueue_iteration(sipg_op* op, PcgCache& c, double* x, cudaStream_t s) {
  const int vb = vec_grid(c.n);
  ApplyArgs<double> a{};
  a.in = c.p;
  a.out = c.Ap;
  a.dim = op->dim;
  a.nu = op->pen;
  a.st = c.st;
  a.red = c.red;
  SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_DOT, a, op->tab, s));
  k_pcg_update<<<vb, kVecThreads, 0, s>>>(x, c.p, c.r, c.Ap, c.n, c.st, c.red);
  SIPG_CUDA_TRY(launch_cross(op->p, 1, c.rows, 1, c.r, c.z, (size_t)op->noe, c.st, c.red, s));
  k_cg_direction<double><<<vb, kVecThreads, 0, s>>>(c.p, c.z, c.n, c.st);
  count_launch(2);
  SIPG_CUDA_TRY(cudaGetLastError());
  return SIPG_OK;
}

sipg_status capture(sipg_op* op, PcgCache& c, double* x, int K) {
  if (c.exec && c.exec_x == x && c.exec_k == K && c.exec_gen == op->tile_gen) return SIPG_OK;
  if (c.exec) {
    cudaGraphExecDestroy(c.exec);
    c.exec = nullptr;
  }
  ApplyArgs<double> prep{};
  prep.dim = op->dim;
  SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_PREPARE, prep, op->tab, c.cap));
  SIPG_CUDA_TRY(cudaStreamBeginCapture(c.cap, cudaStreamCaptureModeThreadLocal));
  sipg_status st = SIPG_OK;
  for (int k = 0; k < K && st == SIPG_OK; ++k) st = enqueue_iteration(op, c, x, c.cap);
  cudaGraph_t g = nullptr;
  const cudaError_t end = cudaStreamEndCapture(c.cap, &g);
  if (st != SIPG_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  SIPG_CUDA_TRY(end);
  const cudaError_t inst = cudaGraphInstantiate(&c.exec, g, 0);
  cudaGraphDestroy(g);
  SIPG_CUDA_TRY(inst);
  c.exec_x = x;
  c.exec_k = K;
  c.exec_gen = op->tile_gen;
  return SIPG_OK;
}
}  // namespace

extern "C" {

sipg_status sipg_apply_prec_f64(sipg_op* op, const double* d_in, double* d_out, void* stream) {
  if (!op || !d_in || !d_out || d_in == d_out) {
    set_error("sipg_apply_prec_f64: null or aliased vectors");
    return SIPG_ERR_INVALID;
  }
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  PcgCache* c = nullptr;
  sipg_status st = cache_get(op, false, &c);
  if (st != SIPG_OK) return st;
  const size_t n = (size_t)op->ndof;
  (void)n;
  SIPG_CUDA_TRY(launch_cross(op->p, 0, c->rows, 1, d_in, d_out, (size_t)op->noe, nullptr, ReduceScratch{},
                             (cudaStream_t)stream));
  return SIPG_OK;
}

sipg_status sipg_volume_mvm_f64(int dim, int degree, const double* d_mat, int mat_noe, const double* d_in,
                                double* d_out, void* stream) {
  if (dim < 1 || degree < 1 || degree > SIPG_MAX_DEGREE || !d_mat || !d_in || !d_out || d_in == d_out ||
      !(mat_noe == 1 || (long long)mat_noe == (long long)dim * dim)) {
    set_error("sipg_volume_mvm_f64: need dim >= 1, degree 1..8, mat_noe 1 or dim*dim, distinct non-null vectors");
    return SIPG_ERR_INVALID;
  }
  const size_t noe = (size_t)dim * dim, n = noe * (size_t)(degree + 1) * (degree + 1);
  (void)n;
  SIPG_CUDA_TRY(launch_cross(degree, 0, d_mat, (size_t)mat_noe, d_in, d_out, noe, nullptr, ReduceScratch{},
                             (cudaStream_t)stream));
  return SIPG_OK;
}

sipg_status sipg_pcg_f64(sipg_op* op, double* d_x, const double* d_b, double tol, int tol_relative, int max_it,
                         sipg_cg_result* res, void* stream) {
  if (!op || !d_x || !d_b) {
    set_error("sipg_pcg_f64: null argument");
    return SIPG_ERR_INVALID;
  }
  SIPG_CUDA_TRY(cudaSetDevice(op->device));
  cudaStream_t s = (cudaStream_t)stream;
  PcgCache* cp = nullptr;
  sipg_status st = cache_get(op, true, &cp);
  if (st != SIPG_OK) return st;
  PcgCache& c = *cp;
  const int K = op->ndof <= (1LL << 20) ? 32 : 8;
  st = capture(op, c, d_x, K);
  if (st != SIPG_OK) return st;
  const long long mx = (max_it > 0) ? max_it : op->ndof;
  const int max_i = (int)std::min<long long>(mx, 2000000000LL);
  const int vb = vec_grid(c.n);
  SIPG_CUDA_TRY(cudaEventRecord(c.ev0, s));
  // ||b||, stop, state; r = b - A x; z = M r, (r.z)_old; p = z
  k_cg_init<double><<<vb, kVecThreads, 0, s>>>(d_b, c.n, c.st, tol, tol_relative, max_i, c.red);
  ApplyArgs<double> a{};
  a.in = d_x;
  a.out = c.r;
  a.b = d_b;
  a.dim = op->dim;
  a.nu = op->pen;
  a.st = c.st;
  a.red = c.red;
  SIPG_CUDA_TRY(launch_apply_f64(op->p, op->cfg64, APPLY_RESID, a, op->tab, s));
  k_pcg_force_start<<<1, 1, 0, s>>>(c.st, max_i);
  SIPG_CUDA_TRY(launch_cross(op->p, 1, c.rows, 1, c.r, c.z, (size_t)op->noe, c.st, c.red, s));
  k_cg_direction<double><<<vb, kVecThreads, 0, s>>>(c.p, c.z, c.n, c.st);
  count_launch(4);
  SIPG_CUDA_TRY(cudaGetLastError());
  CgState<double>* hs = c.st_host;
  long long launched = 0;
  for (;;) {
    SIPG_CUDA_TRY(cudaGraphLaunch(c.exec, s));
    count_launch(4ULL * K);
    launched += K;
    SIPG_CUDA_TRY(cudaMemcpyAsync(hs, c.st, sizeof(CgState<double>), cudaMemcpyDeviceToHost, s));
    SIPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs->done) break;
    if (launched > (long long)max_i + K) {
      set_error("sipg_pcg_f64: iteration bookkeeping lost");
      return SIPG_ERR_CUDA;
    }
  }
  SIPG_CUDA_TRY(cudaEventRecord(c.ev1, s));
  SIPG_CUDA_TRY(cudaEventSynchronize(c.ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, c.ev0, c.ev1);
  const bool conv = !(std::sqrt(hs->rres) > hs->stop);
  if (res) {
    res->iterations = hs->it;
    res->rr = hs->rres;
    res->stop = hs->stop;
    res->time_ms = ms;
    res->converged = conv ? 1 : 0;
  }
  if (hs->status == (int)SIPG_ERR_BREAKDOWN) {
    set_error("sipg_pcg_f64: breakdown (p.Ap <= 0 or non-finite scalar)");
    return SIPG_ERR_BREAKDOWN;
  }
  return conv ? SIPG_OK : SIPG_ERR_NOT_CONVERGED;
}

}  // extern "C"
