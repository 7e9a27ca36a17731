/*
 * sipg_oracle.c -- CPU restatement of paogor/CUDA-SIPG-matrix-free's SIPG-SEM
 * Poisson path (tables, mesh, matvec, CG, right-hand side, error norms).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA product path and the
 * timed CPU baseline.  See sipg_oracle.h for the rules on who may call it.
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared (oracle/Makefile); the
 * -ffp-contract=off keeps every product and sum separately rounded, as the
 * reference's code is when it is compiled for a CPU without FMA contraction.
 */
#define _GNU_SOURCE
#include "sipg_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MAX_N 33 /* p <= 32, as the reference's 64-entry tables allow */

/* ------------------------------------------------------------------------- */
/* A small persistent thread pool: or_parallel_for splits [0, n) into equal   */
/* contiguous chunks, one per thread.                                         */
/* ------------------------------------------------------------------------- */
typedef void (*or_task_fn)(void* ctx, long begin, long end);

#define OR_MAX_THREADS 256
static struct {
  pthread_mutex_t mu;
  pthread_cond_t cv_work, cv_done;
  int nthreads; /* workers started */
  long generation;
  int pending;
  or_task_fn fn;
  void* ctx;
  long n;
  int nchunks;
  pthread_t tid[OR_MAX_THREADS];
} g_pool = {PTHREAD_MUTEX_INITIALIZER, PTHREAD_COND_INITIALIZER, PTHREAD_COND_INITIALIZER, 0, 0, 0,
            NULL, NULL, 0, 0, {0}};

static void chunk_bounds(long n, int nchunks, int k, long* b, long* e) {
  const long q = n / nchunks, r = n % nchunks;
  *b = k * q + (k < r ? k : r);
  *e = *b + q + (k < r ? 1 : 0);
}

static void* pool_worker(void* arg) {
  const int me = (int)(long)arg; /* worker k handles chunk k+1; caller does chunk 0 */
  long seen = 0;
  for (;;) {
    pthread_mutex_lock(&g_pool.mu);
    while (g_pool.generation == seen) pthread_cond_wait(&g_pool.cv_work, &g_pool.mu);
    seen = g_pool.generation;
    or_task_fn fn = g_pool.fn;
    void* ctx = g_pool.ctx;
    const long n = g_pool.n;
    const int nchunks = g_pool.nchunks;
    pthread_mutex_unlock(&g_pool.mu);
    if (me + 1 < nchunks) {
      long b, e;
      chunk_bounds(n, nchunks, me + 1, &b, &e);
      if (b < e) fn(ctx, b, e);
    }
    pthread_mutex_lock(&g_pool.mu);
    if (--g_pool.pending == 0) pthread_cond_signal(&g_pool.cv_done);
    pthread_mutex_unlock(&g_pool.mu);
  }
  return NULL;
}

static void or_parallel_for(int nthreads, long n, or_task_fn fn, void* ctx) {
  if (nthreads > OR_MAX_THREADS) nthreads = OR_MAX_THREADS;
  if (nthreads <= 1 || n < 2) {
    if (n > 0) fn(ctx, 0, n);
    return;
  }
  pthread_mutex_lock(&g_pool.mu);
  while (g_pool.nthreads < nthreads - 1) {
    pthread_create(&g_pool.tid[g_pool.nthreads], NULL, pool_worker, (void*)(long)g_pool.nthreads);
    g_pool.nthreads++;
  }
  g_pool.fn = fn;
  g_pool.ctx = ctx;
  g_pool.n = n;
  g_pool.nchunks = nthreads;
  g_pool.pending = g_pool.nthreads;
  g_pool.generation++;
  pthread_cond_broadcast(&g_pool.cv_work);
  pthread_mutex_unlock(&g_pool.mu);
  {
    long b, e;
    chunk_bounds(n, nthreads, 0, &b, &e);
    if (b < e) fn(ctx, b, e);
  }
  pthread_mutex_lock(&g_pool.mu);
  while (g_pool.pending > 0) pthread_cond_wait(&g_pool.cv_done, &g_pool.mu);
  pthread_mutex_unlock(&g_pool.mu);
}

/* ------------------------------------------------------------------------- */
/* Precision-generic pieces                                                   */
/* ------------------------------------------------------------------------- */
#define REAL double
#define FN(name) name##_d
#define REAL_EPS DBL_EPSILON
#define FABS fabs
#define COS cos
#define SIN sin
#include "sipg_oracle_real.inc"
#undef REAL
#undef FN
#undef REAL_EPS
#undef FABS
#undef COS
#undef SIN

#define REAL float
#define FN(name) name##_f
#define REAL_EPS FLT_EPSILON
#define FABS fabsf
#define COS cosf
#define SIN sinf
#include "sipg_oracle_real.inc"
#undef REAL
#undef FN
#undef REAL_EPS
#undef FABS
#undef COS
#undef SIN

int sipg_oracle_lgl(int npts, double* nodes, double* weights) {
  if (npts < 2 || npts > ORACLE_MAX_N) return -1;
  return lgl_d(npts, nodes, weights);
}

int sipg_oracle_dphi(int p, double* D) { return dphi_d(p, D); }

/* laplace_2d::operator() (laplacian_operator.hpp:67-88) over all index pairs,
 * laid out as sem_laplacian_gpu_validation_test.cu:46-63 does */
int sipg_oracle_laplace2d(int p, double* Lout) {
  const int n = p + 1;
  double nodes[ORACLE_MAX_N], w[ORACLE_MAX_N], D[ORACLE_MAX_N * ORACLE_MAX_N];
  if (p < 1 || n > ORACLE_MAX_N) return -1;
  lgl_d(n, nodes, w);
  dphi_d(p, D);
  size_t at = 0;
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2)
      for (int j1 = 0; j1 < n; ++j1)
        for (int j2 = 0; j2 < n; ++j2) {
          double result = 0;
          if (i2 == j2)
            for (int k = 0; k < n; ++k) result += w[k] * w[i2] * D[i1 * n + k] * D[j1 * n + k];
          if (i1 == j1)
            for (int k = 0; k < n; ++k) result += w[k] * w[i1] * D[i2 * n + k] * D[j2 * n + k];
          Lout[at++] = result;
        }
  return 0;
}

/* square_mesh<T>::compute_coordinates (build_square_mesh.hpp:250-288):
 * coordinates are accumulated sums of delta, row 0 at the top */
int sipg_oracle_mesh_coords(int dim, double* x, double* y) {
  if (dim < 1) return -1;
  const long noe = (long)dim * dim;
  const double delta = 1. / (double)dim;
  double xx = 0, yy = 1;
  for (int i = 0; i < dim; ++i) {
    xx = 0;
    yy -= delta;
    for (int j = 0; j < dim; ++j) {
      const long id = (long)i * dim + j;
      x[0 * noe + id] = xx;
      y[0 * noe + id] = yy;
      x[1 * noe + id] = xx + delta;
      y[1 * noe + id] = yy;
      x[2 * noe + id] = xx + delta;
      y[2 * noe + id] = yy + delta;
      x[3 * noe + id] = xx;
      y[3 * noe + id] = yy + delta;
      xx += delta;
    }
  }
  return 0;
}

int sipg_oracle_apply(int p, int dim, double pen, const double* in, double* out, int nthreads) {
  return apply_d(p, dim, pen, in, out, nthreads);
}

int sipg_oracle_apply_f32(int p, int dim, float pen, const float* in, float* out, int nthreads) {
  return apply_f(p, dim, pen, in, out, nthreads);
}

int sipg_oracle_volume(int p, int dim, const double* in, double* out) {
  apply_ctx_d c;
  if (ctx_init_d(&c, p, dim, 0, in, out)) return -1;
  volume_range_d(&c, 0, (long)dim * dim);
  return 0;
}

int sipg_oracle_flux_x(int p, int dim, double pen, const double* in, double* out) {
  apply_ctx_d c;
  if (ctx_init_d(&c, p, dim, pen, in, out)) return -1;
  flux_x_range_d(&c, 0, (long)dim * dim);
  return 0;
}

int sipg_oracle_flux_y(int p, int dim, double pen, const double* in, double* out) {
  apply_ctx_d c;
  if (ctx_init_d(&c, p, dim, pen, in, out)) return -1;
  flux_y_range_d(&c, 0, (long)dim * dim);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Conjugate gradient (conjugate_gradient_gpu.hpp:18-109, with alpha_kernel   */
/* and beta_kernel of conjugate_gradient_kernels.hpp:5-38).  The dot products */
/* are summed in index order on one thread (cuBLAS's order is unspecified);  */
/* with nthreads > 1 they are summed per fixed chunk, chunks in order.        */
/* ------------------------------------------------------------------------- */
typedef struct {
  const double *a, *b;
  double partial[OR_MAX_THREADS];
  long n;
  int nchunks;
} dot_ctx;

static void dot_task(void* vctx, long b, long e) {
  dot_ctx* c = (dot_ctx*)vctx;
  /* identify the chunk from its start */
  for (int k = 0; k < c->nchunks; ++k) {
    long kb, ke;
    chunk_bounds(c->n, c->nchunks, k, &kb, &ke);
    if (kb == b) {
      double s = 0;
      for (long i = b; i < e; ++i) s += c->a[i] * c->b[i];
      c->partial[k] = s;
      return;
    }
  }
}

static double or_dot(const double* a, const double* b, long n, int nthreads) {
  if (nthreads <= 1 || n < 2) {
    double s = 0;
    for (long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
  }
  if (nthreads > OR_MAX_THREADS) nthreads = OR_MAX_THREADS;
  dot_ctx c;
  c.a = a;
  c.b = b;
  c.n = n;
  c.nchunks = nthreads;
  memset(c.partial, 0, sizeof(c.partial));
  or_parallel_for(nthreads, n, dot_task, &c);
  double s = 0;
  for (int k = 0; k < nthreads; ++k) s += c.partial[k];
  return s;
}

typedef struct {
  double *x, *p, *r;
  const double* Ap;
  const double* b;
  double alpha, beta;
  int which;
} axpy_ctx;

static void axpy_task(void* vctx, long b, long e) {
  axpy_ctx* c = (axpy_ctx*)vctx;
  if (c->which == 0) { /* alpha_kernel */
    for (long i = b; i < e; ++i) {
      c->x[i] = c->x[i] + c->alpha * c->p[i];
      c->r[i] = c->r[i] - c->alpha * c->Ap[i];
    }
  } else if (c->which == 1) { /* beta_kernel: p = r + beta p */
    for (long i = b; i < e; ++i) c->p[i] = c->r[i] + c->beta * c->p[i];
  } else { /* beta_kernel(r, b, -1): r = b + (-1) r */
    for (long i = b; i < e; ++i) c->r[i] = c->b[i] + c->beta * c->r[i];
  }
}

int sipg_oracle_cg(int p, int dim, double pen, double* x, const double* b, double tol, int rel,
                   int max_it_in, double* rr_out, int nthreads) {
  const long n = (long)dim * dim * (p + 1) * (p + 1);
  double* r = (double*)malloc(sizeof(double) * n);
  double* pv = (double*)malloc(sizeof(double) * n);
  double* Ap = (double*)malloc(sizeof(double) * n);
  if (!r || !pv || !Ap) {
    free(r);
    free(pv);
    free(Ap);
    return -1;
  }
  const double norm_b = sqrt(or_dot(b, b, n, nthreads));
  axpy_ctx c = {x, pv, r, Ap, b, 0, 0, 0};
  /* r = b - A x */
  apply_d(p, dim, pen, x, r, nthreads);
  c.which = 2;
  c.beta = -1;
  or_parallel_for(nthreads, n, axpy_task, &c);
  memcpy(pv, r, sizeof(double) * n);
  double rr_old = or_dot(r, r, n, nthreads);
  const double stop = rel ? tol * norm_b : tol;
  const long max_it = max_it_in > 0 ? max_it_in : n;
  int it = 0;
  while (sqrt(rr_old) > stop && it < max_it) {
    apply_d(p, dim, pen, pv, Ap, nthreads);
    const double pAp = or_dot(pv, Ap, n, nthreads);
    c.alpha = rr_old / pAp;
    c.which = 0;
    or_parallel_for(nthreads, n, axpy_task, &c);
    const double rr_new = or_dot(r, r, n, nthreads);
    c.beta = rr_new / rr_old;
    c.which = 1;
    or_parallel_for(nthreads, n, axpy_task, &c);
    rr_old = rr_new;
    ++it;
  }
  if (rr_out) *rr_out = rr_old;
  free(r);
  free(pv);
  free(Ap);
  return it;
}

/* ------------------------------------------------------------------------- */
/* Block-Jacobi preconditioner and preconditioned CG (USE_PRECONDITIONER).     */
/* ------------------------------------------------------------------------- */
/* laplace_2d::operator() (laplacian_operator.hpp:67-88), one entry */
static double lap_entry(int n, const double* w, const double* D, int i1, int i2, int j1, int j2) {
  double result = 0;
  if (i2 == j2)
    for (int k = 0; k < n; ++k) result += w[k] * w[i2] * D[i1 * n + k] * D[j1 * n + k];
  if (i1 == j1)
    for (int k = 0; k < n; ++k) result += w[k] * w[i1] * D[i2 * n + k] * D[j2 * n + k];
  return result;
}

/* block_diagonal_preconditioner_2d::build_diagonal_block
 * (laplacian_operator.hpp:133-186): the element Laplacian, the consistency
 * terms of its four faces with the interior factor 1/2, the penalty on the
 * face nodes */
int sipg_oracle_prec_block(int p, double pen_in, double* a) {
  const int N = p, n = p + 1, nn = n * n;
  double nodes[ORACLE_MAX_N], w[ORACLE_MAX_N], D[ORACLE_MAX_N * ORACLE_MAX_N];
  if (p < 1 || n > ORACLE_MAX_N) return -1;
  lgl_d(n, nodes, w);
  dphi_d(p, D);
  const double pen = (double)(int)pen_in; /* the constructor takes `int _pen` (:116) */
#define IDX(i1, i2, j1, j2) (nn * (n * (i2) + (i1)) + (n * (j2) + (j1)))
  for (int i1 = 0; i1 <= N; ++i1)
    for (int i2 = 0; i2 <= N; ++i2)
      for (int j1 = 0; j1 <= N; ++j1)
        for (int j2 = 0; j2 <= N; ++j2) a[IDX(i1, i2, j1, j2)] = lap_entry(n, w, D, i1, i2, j1, j2);
  for (int j = 0; j <= N; ++j)
    for (int i = 0; i <= N; ++i) {
      const double d0 = D[i * n + 0], dN = D[i * n + N];
      a[IDX(i, j, 0, j)] -= -1 * w[j] * d0 * .5; /* LEFT */
      a[IDX(0, j, i, j)] -= -1 * w[j] * d0 * .5;
      a[IDX(i, j, N, j)] -= w[j] * dN * .5; /* RIGHT */
      a[IDX(N, j, i, j)] -= w[j] * dN * .5;
      a[IDX(j, i, j, 0)] -= -1 * w[j] * d0 * .5; /* DOWN */
      a[IDX(j, 0, j, i)] -= -1 * w[j] * d0 * .5;
      a[IDX(j, i, j, N)] -= w[j] * dN * .5; /* UP */
      a[IDX(j, N, j, i)] -= w[j] * dN * .5;
    }
  for (int i = 0; i <= N; ++i) {
    a[IDX(N, i, N, i)] += pen * w[i];
    a[IDX(i, N, i, N)] += pen * w[i];
    a[IDX(0, i, 0, i)] += pen * w[i];
    a[IDX(i, 0, i, 0)] += pen * w[i];
  }
#undef IDX
  return 0;
}

/* The inverse as LAPACK's dgetrf + dgetri compute it (lapack_wrapper.cpp:
 * 29-42): LU with partial pivoting (unit lower triangle, row interchanges in
 * order), then each column of the inverse by forward and back substitution of
 * the interchanged unit vector.  Row-major. */
int sipg_oracle_invert(int n, double* A) {
  int* piv = (int*)malloc(sizeof(int) * n);
  double* inv = (double*)malloc(sizeof(double) * n * n);
  double* col = (double*)malloc(sizeof(double) * n);
  int rc = 0;
  if (!piv || !inv || !col) {
    rc = -1;
    goto out;
  }
  for (int c = 0; c < n; ++c) {
    int pr = c;
    for (int r = c + 1; r < n; ++r)
      if (fabs(A[r * n + c]) > fabs(A[pr * n + c])) pr = r;
    piv[c] = pr;
    if (A[pr * n + c] == 0) {
      rc = -1;
      goto out;
    }
    if (pr != c)
      for (int k = 0; k < n; ++k) {
        const double t = A[c * n + k];
        A[c * n + k] = A[pr * n + k];
        A[pr * n + k] = t;
      }
    for (int r = c + 1; r < n; ++r) {
      const double l = A[r * n + c] / A[c * n + c];
      A[r * n + c] = l;
      for (int k = c + 1; k < n; ++k) A[r * n + k] -= l * A[c * n + k];
    }
  }
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) col[i] = (i == j) ? 1.0 : 0.0;
    for (int i = 0; i < n; ++i) {
      const double t = col[i];
      col[i] = col[piv[i]];
      col[piv[i]] = t;
    }
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < i; ++k) col[i] -= A[i * n + k] * col[k];
    for (int i = n - 1; i >= 0; --i) {
      for (int k = i + 1; k < n; ++k) col[i] -= A[i * n + k] * col[k];
      col[i] /= A[i * n + i];
    }
    for (int i = 0; i < n; ++i) inv[i * n + j] = col[i];
  }
  memcpy(A, inv, sizeof(double) * n * n);
out:
  free(piv);
  free(inv);
  free(col);
  return rc;
}

/* host_preconditioner_matrix (mode_matrix.hpp:474-522): per row (i1,i2) of
 * the inverse, the diagonal, then the same-i1 entries, then the same-i2 ones */
int sipg_oracle_prec_rows(int p, double pen, double* rows) {
  const int n = p + 1, nn = n * n, R = 2 * p + 1;
  double* a = (double*)malloc(sizeof(double) * nn * nn);
  if (!a) return -1;
  if (sipg_oracle_prec_block(p, pen, a) || sipg_oracle_invert(nn, a)) {
    free(a);
    return -1;
  }
#define PREC(i1, i2, j1, j2) a[nn * (n * (i2) + (i1)) + (n * (j2) + (j1))]
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2) {
      double* row = rows + (size_t)(i1 * n + i2) * R;
      int r = 0;
      row[r] = PREC(i1, i2, i1, i2);
      for (int j = 0; j < n; ++j)
        if (j != i2) row[++r] = PREC(i1, i2, i1, j);
      for (int j = 0; j < n; ++j)
        if (j != i1) row[++r] = PREC(i1, i2, j, i2);
    }
#undef PREC
  free(a);
  return 0;
}

/* volume_mvm<T, 1> (mode_matrix_kernels.hpp:7-65) with the rows above */
int sipg_oracle_prec_apply(int p, int dim, const double* rows, const double* in, double* out) {
  const int n = p + 1, R = 2 * p + 1;
  const long noe = (long)dim * dim;
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2) {
      const double* row = rows + (size_t)(i1 * n + i2) * R;
      for (long e = 0; e < noe; ++e) {
        int r = 0;
        double result = 0.;
        result += row[r] * in[(long)(i1 * n + i2) * noe + e];
        for (int i = 0; i < n; ++i)
          if (i != i2) result += row[++r] * in[(long)(i1 * n + i) * noe + e];
        for (int i = 0; i < n; ++i)
          if (i != i1) result += row[++r] * in[(long)(i * n + i2) * noe + e];
        out[(long)(i1 * n + i2) * noe + e] = result;
      }
    }
  return 0;
}

/* preconditioned_conjugate_gradient (conjugate_gradient_gpu.hpp:116-213) */
int sipg_oracle_pcg(int p, int dim, double pen, double* x, const double* b, double tol, int rel, int max_it_in,
                    double* rr_out, int nthreads) {
  const int n1 = p + 1, R = 2 * p + 1;
  const long n = (long)dim * dim * n1 * n1;
  double* rows = (double*)malloc(sizeof(double) * n1 * n1 * R);
  double* r = (double*)malloc(sizeof(double) * n);
  double* pv = (double*)malloc(sizeof(double) * n);
  double* Ap = (double*)malloc(sizeof(double) * n);
  double* z = (double*)malloc(sizeof(double) * n);
  int it = -1;
  if (!rows || !r || !pv || !Ap || !z || sipg_oracle_prec_rows(p, pen, rows)) goto out;
  {
    const double norm_b = sqrt(or_dot(b, b, n, nthreads));
    axpy_ctx c = {x, pv, r, Ap, b, 0, 0, 0};
    apply_d(p, dim, pen, x, r, nthreads); /* r = b - A x */
    c.which = 2;
    c.beta = -1;
    or_parallel_for(nthreads, n, axpy_task, &c);
    sipg_oracle_prec_apply(p, dim, rows, r, z);
    memcpy(pv, z, sizeof(double) * n); /* p = z */
    double rr_old = or_dot(r, z, n, nthreads);
    const double stop = rel ? tol * norm_b : tol;
    const long max_it = max_it_in > 0 ? max_it_in : n;
    double rr = 1;
    it = 0;
    while (sqrt(rr) > stop && it < max_it) {
      apply_d(p, dim, pen, pv, Ap, nthreads);
      const double pAp = or_dot(pv, Ap, n, nthreads);
      c.alpha = rr_old / pAp;
      c.which = 0;
      or_parallel_for(nthreads, n, axpy_task, &c);
      rr = or_dot(r, r, n, nthreads);
      sipg_oracle_prec_apply(p, dim, rows, r, z);
      const double rr_new = or_dot(z, r, n, nthreads);
      /* beta_kernel(p, z, beta): p = z + beta p */
      c.beta = rr_new / rr_old;
      for (long i = 0; i < n; ++i) pv[i] = z[i] + c.beta * pv[i];
      rr_old = rr_new;
      ++it;
    }
    if (rr_out) *rr_out = rr;
  }
out:
  free(rows);
  free(r);
  free(pv);
  free(Ap);
  free(z);
  return it;
}

/* ------------------------------------------------------------------------- */
/* Test problems (validation_tests/analytical_solutions.hpp:7-94 for A..E).   */
/* ------------------------------------------------------------------------- */
static void eval_problem(int sol, const or_modes* m, double x, double y, double* u, double* f, double* dx,
                         double* dy) {
  const double PI = 3.14159265359; /* analytical_solutions.hpp:10 */
  switch (sol) {
    case OR_SOL_A:
      *u = x * y * (y - 1) * (x - 1) * exp(x - y);
      *f = -2 * x * (y - 1) * (y - 2 * x + x * y + 2) * exp(x - y);
      *dx = (x * x + x - 1) * (y - 1) * y * exp(x - y);
      *dy = -1 * (y * y - 3 * y + 1) * (x - 1) * x * exp(x - y);
      break;
    case OR_SOL_B:
      *u = x * (1 - x) * exp(3 * x) * sin(2 * PI * y);
      *f = -sin(2 * PI * y) * exp(3 * x) * ((4 - 3 * x - 9 * x * x) - 4 * PI * PI * (x - x * x));
      *dx = (3 * (1 - x) * x - x + (1 - x)) * exp(3 * x) * sin(2 * PI * y);
      *dy = 2 * PI * (1 - x) * x * exp(3 * x) * cos(2 * PI * y);
      break;
    case OR_SOL_C:
      *u = y * (1 - y) * x * x * x;
      *f = 2 * x * x * x - 6 * x * y * (1 - y);
      *dx = y * (1 - y) * x * x * 3;
      *dy = (1 - 2 * y) * x * x * x;
      break;
    case OR_SOL_D:
      *u = x * x * y * y;
      *f = -2 * y * y - 2 * x * x;
      *dx = 2 * x * y * y;
      *dy = 2 * y * x * x;
      break;
    case OR_SOL_E:
      *u = cos(8 * PI * x) + cos(8 * PI * y);
      *f = 64 * PI * PI * cos(8 * PI * x) + 64 * PI * PI * cos(8 * PI * y);
      *dx = -8 * PI * sin(8 * PI * x);
      *dy = -8 * PI * sin(8 * PI * y);
      break;
    case OR_SOL_SINSIN: {
      const double tp = 2 * M_PI;
      *u = sin(tp * x) * sin(tp * y);
      *f = 2 * tp * tp * sin(tp * x) * sin(tp * y);
      *dx = tp * cos(tp * x) * sin(tp * y);
      *dy = tp * sin(tp * x) * cos(tp * y);
      break;
    }
    case OR_SOL_MODES: {
      double su = 0, sf = 0, sx = 0, sy = 0;
      for (int q = 0; q < m->nmodes; ++q) {
        const double kx = m->k[q] * M_PI, ly = m->l[q] * M_PI;
        const double A = m->amp[q], lam = kx * kx + ly * ly;
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

double sipg_oracle_u_exact(int sol, const or_modes* modes, double x, double y) {
  double u, f, dx, dy;
  eval_problem(sol, modes, x, y, &u, &f, &dx, &dy);
  return u;
}

static double prob_u(int sol, const or_modes* m, double x, double y) {
  double u, f, dx, dy;
  eval_problem(sol, m, x, y, &u, &f, &dx, &dy);
  return u;
}
static double prob_f(int sol, const or_modes* m, double x, double y) {
  double u, f, dx, dy;
  eval_problem(sol, m, x, y, &u, &f, &dx, &dy);
  return f;
}

/* sipg_sem_2d<T>::compute_rhs (sipg_sem_2d.hpp:232-305) */
int sipg_oracle_rhs(int p, int dim, double pen, int sol, const or_modes* modes, double* rhs) {
  const int N = p, n = p + 1;
  const long noe = (long)dim * dim;
  double qn[ORACLE_MAX_N], qw[ORACLE_MAX_N], D[ORACLE_MAX_N * ORACLE_MAX_N];
  double nodes[ORACLE_MAX_N], weights[ORACLE_MAX_N], w[ORACLE_MAX_N];
  if (p < 1 || n > ORACLE_MAX_N || dim < 1) return -1;
  lgl_d(n, qn, qw);
  dphi_d(p, D);
  double* x = (double*)malloc(sizeof(double) * 4 * noe);
  double* y = (double*)malloc(sizeof(double) * 4 * noe);
  if (!x || !y) {
    free(x);
    free(y);
    return -1;
  }
  sipg_oracle_mesh_coords(dim, x, y);
  for (int i = 0; i <= N; ++i) {
    nodes[i] = (qn[i] * .5 + .5) / dim;
    weights[i] = qw[i];
    w[i] = qw[i] * .5 / dim;
  }
#define R(i1, i2, e) rhs[((size_t)(i1) * n + (i2)) * noe + (size_t)(e)]
  for (int i1 = 0; i1 <= N; ++i1)
    for (int i2 = 0; i2 <= N; ++i2)
      for (long e = 0; e < noe; ++e) R(i1, i2, e) = w[i1] * w[i2] * prob_f(sol, modes, x[e] + nodes[i1], y[e] + nodes[i2]);
  for (int xx = 0; xx < dim; ++xx) {
    const long eD = (long)(dim - 1) * dim + xx; /* DOWN */
    const double xeD = x[eD], yeD = y[eD];
    const long eU = xx; /* UP */
    const double xeU = x[eU], yeU = y[eU];
    const long eL = (long)xx * dim; /* LEFT */
    const double xeL = x[eL], yeL = y[eL];
    const long eR = (long)xx * dim + dim - 1; /* RIGHT */
    const double xeR = x[eR], yeR = y[eR];
    for (int i = 0; i <= N; ++i) {
      R(i, 0, eD) += pen * weights[i] * prob_u(sol, modes, xeD + nodes[i], yeD + nodes[0]);
      R(i, N, eU) += pen * weights[i] * prob_u(sol, modes, xeU + nodes[i], yeU + nodes[N]);
      R(0, i, eL) += pen * weights[i] * prob_u(sol, modes, xeL + nodes[0], yeL + nodes[i]);
      R(N, i, eR) += pen * weights[i] * prob_u(sol, modes, xeR + nodes[N], yeR + nodes[i]);
      for (int j = 0; j <= N; ++j) {
        R(i, j, eD) -= -1 * weights[i] * D[j * n + 0] * prob_u(sol, modes, xeD + nodes[i], yeD + nodes[0]);
        R(i, j, eU) -= weights[i] * D[j * n + N] * prob_u(sol, modes, xeU + nodes[i], yeU + nodes[N]);
        R(j, i, eL) -= -1 * weights[i] * D[j * n + 0] * prob_u(sol, modes, xeL + nodes[0], yeL + nodes[i]);
        R(j, i, eR) -= weights[i] * D[j * n + N] * prob_u(sol, modes, xeR + nodes[N], yeR + nodes[i]);
      }
    }
  }
#undef R
  free(x);
  free(y);
  return 0;
}

/* sipg_sem_2d<T>::err_norms (sipg_sem_2d.hpp:311-370): nodal max error, LGL-
 * quadrature L2 and broken H1 errors; phi(j,q) = delta_jq (sem_function.hpp:74-80) */
int sipg_oracle_err_norms(int p, int dim, int sol, const or_modes* modes, const double* u, double* out) {
  const int order = p, n = p + 1;
  const long noe = (long)dim * dim;
  double qn[ORACLE_MAX_N], qw[ORACLE_MAX_N], D[ORACLE_MAX_N * ORACLE_MAX_N];
  double nodes[ORACLE_MAX_N], weights[ORACLE_MAX_N];
  if (p < 1 || n > ORACLE_MAX_N || dim < 1) return -1;
  lgl_d(n, qn, qw);
  dphi_d(p, D);
  double* x = (double*)malloc(sizeof(double) * 4 * noe);
  double* y = (double*)malloc(sizeof(double) * 4 * noe);
  if (!x || !y) {
    free(x);
    free(y);
    return -1;
  }
  sipg_oracle_mesh_coords(dim, x, y);
  for (int i = 0; i <= order; ++i) {
    nodes[i] = (qn[i] * .5 + .5) / dim;
    weights[i] = qw[i] * .5 / dim;
  }
  double max_err = -1, dx_sq = 0, dy_sq = 0, L2_sq = 0;
#define U(i1, i2, e) u[((size_t)(i1) * n + (i2)) * noe + (size_t)(e)]
  for (long e = 0; e < noe; ++e)
    for (int pp = 0; pp <= order; ++pp)
      for (int q = 0; q <= order; ++q) {
        double dx_u = 0, dy_u = 0;
        const double weight2d = weights[pp] * weights[q];
        for (int i = 0; i <= order; ++i)
          for (int j = 0; j <= order; ++j) {
            const double phi_jq = (j == q) ? 1 : 0, phi_ip = (i == pp) ? 1 : 0;
            dx_u += U(i, j, e) * 2 * dim * D[i * n + pp] * phi_jq;
            dy_u += U(i, j, e) * 2 * dim * phi_ip * D[j * n + q];
          }
        const double xe = x[e], ye = y[e];
        double uu, ff, ddx, ddy;
        eval_problem(sol, modes, xe + nodes[pp], ye + nodes[q], &uu, &ff, &ddx, &ddy);
        const double err = fabs(U(pp, q, e) - uu);
        if (err > max_err) max_err = err;
        L2_sq += weight2d * pow(err, 2);
        dx_sq += weight2d * pow(dx_u - ddx, 2);
        dy_sq += weight2d * pow(dy_u - ddy, 2);
      }
#undef U
  out[0] = sqrt(L2_sq);
  out[1] = sqrt(L2_sq + dx_sq + dy_sq);
  out[2] = max_err;
  free(x);
  free(y);
  return 0;
}

void sipg_oracle_fill_uniform(unsigned long long seed, double lo, double hi, double* out, long long n) {
  unsigned long long s = seed;
  for (long long i = 0; i < n; ++i) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    out[i] = lo + (hi - lo) * ((double)(z >> 11) * (1.0 / 9007199254740992.0));
  }
}
