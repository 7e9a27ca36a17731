/*
 * sipg_gb300.h -- C ABI of the GB300-native matrix-free SIPG-SEM Poisson
 * solver (sm_103a).  Plain pointers and sizes only; every call returns a
 * sipg_status and nothing calls exit().
 *
 * Vectors use the reference's node-major layout: value (i1,i2) of element e
 * at ((i1*(p+1)+i2)*noe + e), noe = dim*dim, element e = row*dim + col with row
 * 0 at the top of the unit square (mode_vector.hpp:108-120 and
 * build_square_mesh.hpp:250-288 of paogor/CUDA-SIPG-matrix-free), so the
 * device pointer of a reference mode_vector<T,int> drops straight in.
 *
 * Device pointers ("d_") must be cudaMalloc'ed on the op's device; host
 * pointers ("h_") are ordinary or pinned host memory.  `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).
 */
#ifndef SIPG_GB300_H
#define SIPG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SIPG_OK = 0,
  SIPG_ERR_INVALID = 1,       /* bad argument (null pointer, degree or size out of range) */
  SIPG_ERR_CUDA = 2,          /* a CUDA runtime call failed; see sipg_last_error() */
  SIPG_ERR_NOT_CONVERGED = 3, /* CG reached max_it before the tolerance */
  SIPG_ERR_BREAKDOWN = 4,     /* CG met p.Ap <= 0 or a non-finite scalar */
  SIPG_ERR_UNSUPPORTED = 5,   /* degree outside 1..SIPG_MAX_DEGREE, or no sm_103a device */
  SIPG_ERR_NOMEM = 6,         /* device allocation failed */
  SIPG_ERR_REJECTED = 7,      /* serving: request does not fit the memory budget */
  SIPG_ERR_TIMEOUT = 8        /* a bounded device wait gave up */
} sipg_status;

typedef enum { SIPG_F64 = 0, SIPG_F32 = 1 } sipg_precision;

#define SIPG_MAX_DEGREE 8

/* Analytic test problems for the on-device right-hand side and error norms:
 * 1..5 = the reference's solutions A..E (validation_tests/analytical_solutions.hpp:7-94,
 * with its PI = 3.14159265359); 6 = sin(2 pi x) sin(2 pi y), f = 8 pi^2 u;
 * 7 = sum of modes A_m sin(k_m pi x) sin(l_m pi y) (f), u = f-modes / ((k^2+l^2) pi^2). */
typedef enum {
  SIPG_SOL_A = 1, SIPG_SOL_B = 2, SIPG_SOL_C = 3, SIPG_SOL_D = 4, SIPG_SOL_E = 5,
  SIPG_SOL_SINSIN = 6, SIPG_SOL_MODES = 7
} sipg_solution;

typedef struct {
  int nmodes; /* 0..8 */
  double amp[8];
  int k[8], l[8];
} sipg_modes;

/* One SIPG operator: a dim x dim uniform mesh of the unit square, degree p,
 * penalty `pen` (the reference's kernel penalty nu: interior faces get 2*nu,
 * boundary faces nu, sipg_sem_2d_gpu_kernels.hpp:209,243-244).  Opaque. */
typedef struct sipg_op sipg_op;

typedef struct {
  int iterations;      /* CG iterations performed */
  double rr;           /* final r.r */
  double stop;         /* absolute stop threshold used on sqrt(r.r) */
  double time_ms;      /* device time of the solve (CUDA events) */
  int converged;       /* 1 if sqrt(r.r) <= stop */
} sipg_cg_result;

/* Inner iteration of the mixed-precision solvers.  SIPG_INNER_F32: FP32
 * vectors and the FP32 apply -- fastest, but an FP32 vector's rounding noise,
 * amplified by A, limits it to condition numbers well below 1 / eps_32
 * (~1.7e7; kappa ~ c_p dim^2, c_p = 0.8, 4.8, 12, 26, 46, 76, 114, 167 for
 * p = 1..8 at penalty p^2).  SIPG_INNER_PAIRS: double-float vectors (two FP32
 * planes) and the compensated apply, ~48-bit values on the FP32 pipes -- any
 * condition number.  SIPG_INNER_AUTO picks F32 when kappa * 2^-24 < 0.01. */
typedef enum {
  SIPG_INNER_AUTO = 0,
  SIPG_INNER_F32 = 1,
  SIPG_INNER_PAIRS = 2,
  SIPG_INNER_F64 = 3,
  SIPG_INNER_F32_TWOLEVEL = 4
} sipg_inner_kind;
/* SIPG_INNER_F32_TWOLEVEL (flexible outer kind only; its default): the FP32
 * inner CG preconditioned by the operator's two-level preconditioner -- exact
 * element block-Jacobi plus a coarse correction on the continuous bilinear
 * functions of the element vertices, solved by one multigrid V-cycle (see
 * sipg_apply_twolevel_f32).  Its iteration count no longer grows with the
 * mesh, so the FP32 inner CG works at every condition number of the supported
 * meshes; unpreconditioned (SIPG_INNER_F32) FP32 CG slows down sharply once
 * kappa * eps_32 approaches 1. */
/* SIPG_INNER_F64 is the same reliable-update loop with FP64 vectors and the
 * FP64 apply: the all-FP64 yardstick.  The plain CG (sipg_cg_f64, the
 * reference's algorithm) stops on its recursively updated residual, whose gap
 * to the true b - A x grows with kappa: on 512 x 512, p = 6 its true relative
 * residual stalls near 1e-9 however small the tolerance. */

/* Outer iteration of the mixed-precision solvers.
 * SIPG_OUTER_RELIABLE: defect correction with reliable updates -- the inner
 *   CG runs on, keeping its search direction, and x += e, r = b - A x happen
 *   in FP64 whenever its residual fell by inner_tol.  Each correction is a
 *   unit step, so the inner solution must be accurate in the residual norm:
 *   FP32 inner vectors stall once kappa * eps_32 approaches 1.
 * SIPG_OUTER_FLEXIBLE: flexible CG in FP64 (Notay 2000, truncated to one
 *   previous direction) preconditioned by an FP32 inner CG that starts from
 *   zero on the scaled residual and stops when its residual fell by
 *   inner_tol.  The FP64 step length alpha = d.r / d.Ad (one FP64 apply per
 *   outer step) minimises the error in the energy norm, where the rounding of
 *   an FP32 correction costs only ~sqrt(kappa) * eps_32, so FP32 values and
 *   accumulation serve at any condition number of the supported meshes.
 * SIPG_OUTER_AUTO: flexible (with the two-level-preconditioned FP32 inner CG
 *   unless the caller names SIPG_INNER_F32) unless the caller names
 *   SIPG_INNER_PAIRS or SIPG_INNER_F64 (then reliable). */
typedef enum { SIPG_OUTER_AUTO = 0, SIPG_OUTER_RELIABLE = 1, SIPG_OUTER_FLEXIBLE = 2 } sipg_outer_kind;

typedef struct {
  double inner_tol;    /* reliable: FP64 correction once the inner residual fell by this factor (0.1);
                          flexible: each inner solve stops once its residual fell by this factor */
  double outer_tol;    /* stop at the FP64 relative residual ||b-Ax||/||b|| <= outer_tol (1e-10) */
  int max_outer;       /* cap on FP64 corrections / flexible-CG steps (200) */
  int max_inner;       /* cap on inner iterations in total (0 = DoF) */
  int inner;           /* sipg_inner_kind (0 = auto) */
  int outer;           /* sipg_outer_kind (0 = auto) */
} sipg_mixed_opts;

typedef struct {
  int outer_iterations; /* FP64 corrections (reliable) or flexible-CG steps */
  int inner_iterations; /* summed over all outer steps */
  double rel_residual;  /* final ||b - A x|| / ||b||, recomputed in FP64 from x */
  double time_ms;
  int converged;
  int inner_kind;       /* the sipg_inner_kind used (F32, PAIRS or F64) */
  int outer_kind;       /* the sipg_outer_kind used (RELIABLE or FLEXIBLE) */
  int fp64_applies;     /* FP64 operator applies, residual checks included */
} sipg_mixed_result;

/* ---- tables and mesh (host side, no device needed) ---- */

/* LGL nodes/weights on [-1,1], npts = p+1 in 2..64 (the operator itself
 * supports p <= SIPG_MAX_DEGREE).
 * Replaces LGL_quadrature_table<T>::LGL_quadrature_table (LGL_quadrature_table.hpp:84-146). */
sipg_status sipg_lgl_table(int npts, double* nodes, double* weights);
/* D[mode*(p+1)+node]: derivative of Lagrange basis `mode` at LGL node `node`,
 * degree 1..63.
 * Replaces sem_function<T>::d_phi / DbaseVALUES (sem_function.hpp:86-110, device_const.hpp:115-127). */
sipg_status sipg_dphi_table(int degree, double* D);
/* The element Laplacian as stored rows: (p+1)^2 rows of 2p+1 values on the
 * (i1,.) / (.,i2) cross pattern (the diagonal, then (i1, j != i2), then
 * (j != i1, i2)), in the mode_matrix layout of one shared operator -- value r
 * of row (i1,i2) at (i1*(p+1)+i2)*(2p+1) + r -- the d_mat of
 * sipg_volume_mvm_f64 with mat_noe = 1.  Host memory.
 * Replaces host_laplacian_matrix<T>(1, p) (mode_matrix.hpp:419-466) with
 * laplace_2d<T> (laplacian_operator.hpp:67-88). */
sipg_status sipg_laplacian_rows_f64(int degree, double* rows);
/* Element corner coordinates x[c*noe+e], y[c*noe+e], c=0..3.
 * Replaces square_mesh<T>::compute_coordinates (build_square_mesh.hpp:250-288). */
sipg_status sipg_square_mesh_coords(int dim, double* x, double* y);

/* ---- operator lifetime ---- */

/* Creates the operator on the current CUDA device: builds the degree-p tables
 * (passed to every kernel launch as parameters) and picks the tile shape.
 * Replaces the setup in the sipg_sem_2d<T> constructor (sipg_sem_2d.hpp:96-113)
 * and load_Dphi_table / load_lgl_quadrature_table (device_const.hpp:70-174),
 * without their process-global __constant__ state: operators of different
 * degree coexist in one process. */
sipg_status sipg_op_create(int dim, int degree, double pen, sipg_op** op);
sipg_status sipg_op_destroy(sipg_op* op);
/* Bytes of device memory one FP64 CG solve on this op keeps resident. */
size_t sipg_op_solve_footprint(int dim, int degree, sipg_precision prec);

/* ---- the operator apply (the hot path) ---- */

/* d_out = A d_in, one fused pass (volume + all faces).  Replaces
 * sipg_sem_2d<T>::_mvm (sipg_sem_2d.hpp:167-201: volume, flux_term6a,
 * flux_term6b) and the free function mvm (sipg_sem_2d_gpu_kernels.hpp:320-364). */
sipg_status sipg_apply_f64(const sipg_op* op, const double* d_in, double* d_out, void* stream);
sipg_status sipg_apply_f32(const sipg_op* op, const float* d_in, float* d_out, void* stream);
/* Double-float pair vectors (2 ndof floats: the hi plane, then the lo plane;
 * value = hi + lo) and compensated arithmetic on the FP32 pipes: about 48
 * significant bits, where FP32 keeps 24 -- on a smooth vector the plain FP32
 * apply loses log10(condition number) of them.  The apply of the
 * SIPG_INNER_PAIRS mixed solvers.  No reference counterpart. */
sipg_status sipg_apply_pairs(const sipg_op* op, const float* d_in, float* d_out, void* stream);
/* The same with host buffers: copies h_in to the device, applies, copies the
 * result back, synchronously.  Device staging buffers are kept in the op. */
sipg_status sipg_apply_host_f64(sipg_op* op, const double* h_in, double* h_out, void* stream);

/* ---- tile shapes and the autotuner (no reference counterpart: the
 * reference launches one fixed geometry) ----
 * An apply tile is 32 elements along a mesh row by `rows` rows (2, 4 or 8),
 * with one thread per element (or two, pairs apply only).  The FP64 apply also
 * has the per-node tile: (p+1)^2 threads per element, one per output node,
 * over ex x ey elements per CTA -- ey = 4 at p = 1, else 2; ex = 4 (p <= 2) or
 * 2 (p >= 3), or twice that -- its default for meshes up to 128 x 128, where
 * 32-element rows leave most of GB300's thin FP64 pipes idle.  Every shape
 * gives bit-identical apply results; CG reductions regroup.  Tile indices for
 * the three apply kinds: */
enum { SIPG_TUNE_F64 = 0, SIPG_TUNE_F32 = 1, SIPG_TUNE_PAIRS = 2 /* compensated, pair vectors */ };
typedef struct {
  int elements_per_row[3];     /* 32, or ex of the per-node tile (FP64), by SIPG_TUNE_* */
  int rows[3];                 /* rows per tile */
  int threads_per_element[3];  /* 1, 2 (pairs apply) or (p+1)^2 (per-node FP64 tile) */
  float ms_per_apply[3];       /* the winning candidate's time */
} sipg_tile_choice;
/* Times the tile shapes for each apply kind on this op -- 32 x {2, 4, 8} with
 * one thread per element, for the pairs apply also 32 x {2, 4} with two, for
 * FP64 also both per-node tiles -- on scratch vectors of ndof doubles
 * (allocated and freed here), keeps the fastest, and records it for (degree,
 * dim) so ops created later in this process start with it.  Synchronous; not
 * during stream capture.  `out` may be NULL.  sipg_op_set_tile returns
 * SIPG_ERR_INVALID for a shape that is not compiled. */
sipg_status sipg_op_autotune(sipg_op* op, void* stream, sipg_tile_choice* out);
sipg_status sipg_op_set_tile(sipg_op* op, int kind, int elements_per_row, int rows, int threads_per_element);
sipg_status sipg_op_get_tile(const sipg_op* op, int kind, int* elements_per_row, int* rows, int* threads_per_element);

/* ---- conjugate gradient ---- */

/* Solves A x = b from the x passed in.  Stops when sqrt(r.r) <= tol
 * (tol_relative = 0, the reference's absolute test,
 * conjugate_gradient_gpu.hpp:63-69) or <= tol*||b|| (tol_relative = 1), or
 * after max_it iterations (max_it <= 0: DoF, as the reference).  Replaces
 * conjugate_gradient<T> (conjugate_gradient_gpu.hpp:18-109).  Scalars stay on
 * the device; iterations run as CUDA graphs, or, for FP64 meshes up to 32 x 32
 * on the per-node tile, as one persistent cooperative kernel whose grid
 * barriers give up after about a second (SIPG_ERR_CUDA).  Returns SIPG_OK,
 * SIPG_ERR_NOT_CONVERGED or SIPG_ERR_BREAKDOWN; `res` may be NULL. */
sipg_status sipg_cg_f64(sipg_op* op, double* d_x, const double* d_b, double tol, int tol_relative, int max_it,
                        sipg_cg_result* res, void* stream);
sipg_status sipg_cg_f32(sipg_op* op, float* d_x, const float* d_b, float tol, int tol_relative, int max_it,
                        sipg_cg_result* res, void* stream);

/* The stored-operator apply of the reference's USE_MODE_MATRIX path:
 * d_out = M d_in with M stored per node row on the (i1,.) / (.,i2) cross
 * pattern, 2p+1 values per row in the reference's mode_matrix layout
 * (value r of row (i1,i2) of element e at ((i1*(p+1)+i2)*(2p+1) + r)*mat_noe
 * + e), one operator for all elements (mat_noe = 1) or one per element
 * (mat_noe = dim*dim).  A mode_matrix::data() pointer is a valid d_mat.
 * Replaces volume_mvm<T, 1> and volume_mvm<T, 0>
 * (mode_matrix_kernels.hpp:7-65). */
sipg_status sipg_volume_mvm_f64(int dim, int degree, const double* d_mat, int mat_noe, const double* d_in,
                                double* d_out, void* stream);

/* Block-Jacobi preconditioner (the reference's USE_PRECONDITIONER path):
 * d_out = M d_in, M the inverse of an interior element's diagonal block kept
 * on the (i1,.) / (.,i2) cross pattern, the same for every element, penalty
 * truncated to an integer as the reference does.  Replaces
 * sipg_sem_2d<T>::_prec_mvm (sipg_sem_2d.hpp:205-224) with
 * host_preconditioner_matrix (mode_matrix.hpp:474-522) and
 * block_diagonal_preconditioner_2d (laplacian_operator.hpp:95-186). */
sipg_status sipg_apply_prec_f64(sipg_op* op, const double* d_in, double* d_out, void* stream);
/* Preconditioned CG with that M: stops when sqrt(r.r) <= tol (absolute, as
 * the reference, or tol*||b|| with tol_relative = 1) or after max_it
 * iterations (<= 0: DoF); the first iteration always runs, as the
 * reference's.  res->rr is the final r.r.  Replaces
 * preconditioned_conjugate_gradient (conjugate_gradient_gpu.hpp:116-213). */
sipg_status sipg_pcg_f64(sipg_op* op, double* d_x, const double* d_b, double tol, int tol_relative, int max_it,
                         sipg_cg_result* res, void* stream);

/* Mixed precision: the operator and CG run on the FP32 pipes (FP32 values,
 * or double-float pairs, see sipg_inner_kind) inside FP64 defect correction
 * with reliable updates -- whenever the inner residual has fallen by
 * inner_tol (or after 1000 inner iterations), x += e in FP64, r = b - A x in
 * FP64, and the inner CG continues with its search direction.  The residual
 * b - A x, the update of x and the outer norms stay FP64 on the device.
 * `opts` may be NULL (defaults in sipg_mixed_opts).  No reference
 * counterpart. */
sipg_status sipg_solve_mixed(sipg_op* op, double* d_x, const double* d_b, const sipg_mixed_opts* opts,
                             sipg_mixed_result* res, void* stream);

/* *rel = ||b - A x|| / ||b|| (||b - A x|| if b = 0), with d_r = b - A x when
 * d_r is not NULL: the true residual, evaluated in FP64 with every zero-sum
 * contraction of the operator taken over differences from one value of its
 * element line.  The plain sums of sipg_apply_f64 round each term at the
 * scale of x itself; on a smooth solution their rounding alone puts a floor
 * near 1e-10 under the relative residual at 1024^2, p = 4, which this
 * evaluation lowers about dim-fold.  The mixed solvers decide convergence
 * with it.  Synchronous.  No reference counterpart. */
sipg_status sipg_residual_f64(sipg_op* op, const double* d_x, const double* d_b, double* d_r, double* rel,
                              void* stream);

/* d_z = M d_r, the two-level preconditioner of the flexible mixed solve, on
 * FP32 vectors: M = B^-1 + P V P^T, B^-1 the exact inverse of every element's
 * diagonal block of A, P the continuous bilinear functions of the element
 * vertices sampled at the LGL nodes, V one symmetric multigrid V-cycle (two
 * damped-Jacobi sweeps before and after each coarse correction, Galerkin
 * levels, the coarsest by its dense inverse) for P^T A P.  Built on the first
 * call on an op (synchronous: a few FP64 applies to probe A, then host work;
 * not during stream capture) and kept with the op.  No reference
 * counterpart. */
sipg_status sipg_apply_twolevel_f32(sipg_op* op, const float* d_r, float* d_z, void* stream);

/* The vector steps of the reference's CG, for callers that iterate around
 * their own operator (an abs_mvm implementation).  sipg_dot_* is
 * synchronous and deterministic; the others are stream-ordered.
 *   sipg_dot:      *result = x.y       (replaces cublas_dot, cublas_wrapper.hpp:62-84)
 *   sipg_cg_step:  x += a p, r -= a Ap (replaces alpha_kernel, conjugate_gradient_kernels.hpp:5-23)
 *   sipg_xpby:     y = x + b y         (replaces beta_kernel, conjugate_gradient_kernels.hpp:26-38) */
sipg_status sipg_dot_f64(size_t n, const double* d_x, const double* d_y, double* result, void* stream);
sipg_status sipg_dot_f32(size_t n, const float* d_x, const float* d_y, float* result, void* stream);
sipg_status sipg_cg_step_f64(size_t n, double alpha, double* d_x, const double* d_p, double* d_r, const double* d_Ap,
                             void* stream);
sipg_status sipg_cg_step_f32(size_t n, float alpha, float* d_x, const float* d_p, float* d_r, const float* d_Ap,
                             void* stream);
sipg_status sipg_xpby_f64(size_t n, const double* d_x, double beta, double* d_y, void* stream);
sipg_status sipg_xpby_f32(size_t n, const float* d_x, float beta, float* d_y, void* stream);
/* *result = x.y like sipg_dot_f64, but without allocating any device memory;
 * no counterpart in the reference.  For callers that cannot call cudaMalloc:
 * code whose device memory belongs to another allocator that reserved the pool
 * up front, or that must not risk an allocation's implicit synchronisation or
 * out-of-memory failure mid-sequence.  Its scratch is a fixed 64 KB device
 * array in the library (held by every GPU that loads it until exit), so
 * n <= 16,777,216; larger n returns SIPG_ERR_INVALID.  The first call on each
 * device looks up the array's device address and keeps it for the life of the
 * process, so after a cudaDeviceReset of a device this entry point must not
 * be called on that device again.  All calls share the array: calls that overlap on the GPU
 * (concurrent streams or threads) race and must be serialised by the caller.
 * Each call returns only once the result is in *result (it waits for the
 * stream); deterministic. */
sipg_status sipg_dot_f64_noalloc(size_t n, const double* d_x, const double* d_y, double* result, void* stream);

/* ---- many problems at once (no reference counterpart) ---- */

/* One problem of a batch: a dim x dim mesh, degree 1..SIPG_MAX_DEGREE, penalty. */
typedef struct {
  int dim;
  int degree;
  double pen;
} sipg_problem;

/* A batch keeps, for each problem, an operator (shared by problems with equal
 * dim, degree and pen), FP32 CG vectors, an FP64 residual, device CG states and
 * reduction scratch, all resident until sipg_batch_destroy.  Opaque. */
typedef struct sipg_batch sipg_batch;

sipg_status sipg_batch_create(int n, const sipg_problem* problems, sipg_batch** batch);
sipg_status sipg_batch_destroy(sipg_batch* batch);
/* The operator of problem i (owned by the batch), e.g. for sipg_rhs_f64. */
sipg_status sipg_batch_op(const sipg_batch* batch, int i, sipg_op** op);
/* Device bytes the batch holds (besides the callers' x and b). */
size_t sipg_batch_footprint(const sipg_batch* batch);
/* Solves A_i x_i = b_i for every problem with the flexible mixed-precision
 * scheme of sipg_solve_mixed (flexible CG in FP64 around an FP32 inner CG to
 * relative opts->inner_tol, default 1e-2), all problems together: the FP32
 * inner iterations of every problem are one batched FP32 apply launch per
 * degree present plus a batched direction and a batched update launch,
 * replayed as a CUDA graph; the FP64 outer steps of the problems due one run
 * as batched launches between replays; problems retire as they converge, each
 * once b - A x recomputed in FP64 is under opts->outer_tol ||b||.  opts->inner
 * and opts->outer must be AUTO or F32 / FLEXIBLE (else SIPG_ERR_INVALID).
 * d_x[i], d_b[i]: FP64 device vectors (x holds x0).  res (array of n, may be
 * NULL) gets each problem's outer steps, FP32 iterations, FP64 applies and
 * final FP64 relative residual; time_ms is the whole batch's. */
sipg_status sipg_batch_solve_mixed(sipg_batch* batch, double* const* d_x, const double* const* d_b,
                                   const sipg_mixed_opts* opts, sipg_mixed_result* res, void* stream);

/* ---- continuous-batching server (no reference counterpart) ---- */

typedef struct {
  size_t budget_bytes;  /* device memory the active requests may hold (150 GB) */
  int max_active;       /* requests solved concurrently, 1..4096 (256) */
  int iters_per_step;   /* CG iterations per sipg_server_step (8) */
  double inner_tol;     /* mixed requests: each FP32 inner solve stops once its residual fell by this (1e-2) */
} sipg_server_opts;

typedef struct {
  int dim;
  int degree;
  double pen;
  int sol;              /* test problem (sipg_solution) whose right-hand side is built on the device */
  sipg_modes modes;     /* for SIPG_SOL_MODES */
  double tol;           /* relative FP64 residual ||b - Ax|| <= tol ||b|| */
  int precision;        /* SIPG_F32: mixed (flexible CG in FP64 around an FP32 inner CG); SIPG_F64: plain FP64 CG */
} sipg_request;

typedef struct {
  int done;             /* 1 once the request retired */
  sipg_status status;   /* SIPG_OK, SIPG_ERR_NOT_CONVERGED, SIPG_ERR_BREAKDOWN, SIPG_ERR_REJECTED */
  int iterations;       /* CG iterations (FP32 inner ones for mixed requests) */
  int corrections;      /* flexible FP64 outer steps (mixed) */
  double rel_residual;  /* final FP64 ||b - Ax|| / ||b|| */
  double queue_ms;      /* submit -> admission */
  double latency_ms;    /* submit -> retirement */
} sipg_request_result;

typedef struct {
  int queued;
  int active;
  unsigned long long completed;
  unsigned long long rejected;
  size_t bytes_in_use;
  double setup_ms;  /* admission time on the stepping thread (cumulative) */
  double prep_ms;   /* busy time of the preparation threads that build mixed requests' operators and
                       preconditioners while they wait (cumulative) */
} sipg_server_stats_t;

typedef struct sipg_server sipg_server;

/* opts may be NULL (defaults in sipg_server_opts).  The server starts up to
 * six preparation threads (half the host's hardware threads; joined by
 * sipg_server_destroy). */
sipg_status sipg_server_create(const sipg_server_opts* opts, sipg_server** server);
sipg_status sipg_server_destroy(sipg_server* server);
/* Queues a request (FIFO); returns SIPG_ERR_REJECTED (and a retired result)
 * when its device footprint alone exceeds the budget.  A mixed request's
 * operator and two-level preconditioner are built by a preparation thread
 * from here on, beside the lanes' work. */
sipg_status sipg_server_submit(sipg_server* server, const sipg_request* req, unsigned long long* id);
/* One scheduling step: admit what fits and is prepared (FIFO), then for each of three
 * size-class lanes (up to 2^18 DoF, up to 2^22, larger; each on its own
 * stream, the smaller the higher its priority) whose previous round has
 * ended: correct / retire its requests and queue its next round of
 * iters_per_step CG iterations in batched launches.  Returns once at least
 * one lane has made progress (it waits only when every lane with work is
 * mid-round); n_active counts admitted, unfinished requests. */
sipg_status sipg_server_step(sipg_server* server, int* n_active, int* n_completed);
sipg_status sipg_server_poll(sipg_server* server, unsigned long long id, sipg_request_result* result);
/* Copies a retired request's solution (n = its DoF) to host memory; the
 * solution stays on the device until sipg_server_release. */
sipg_status sipg_server_solution(sipg_server* server, unsigned long long id, double* h_x, size_t n);
/* Forgets a retired request: frees its solution and result. */
sipg_status sipg_server_release(sipg_server* server, unsigned long long id);
sipg_status sipg_server_stats(const sipg_server* server, sipg_server_stats_t* stats);

/* Self-test of the bounded waits of the persistent small-mesh CG: runs its
 * grid barrier with a target that no arrival count reaches, on 4 CTAs.  Every
 * wait gives up (well under a second), raises the abort flag and returns;
 * *gave_up = 1 when all four did and the context is still usable.  No
 * reference counterpart. */
sipg_status sipg_selftest_barrier_timeout(int* gave_up);

/* ---- either side of the solve ---- */

/* d_b = the right-hand side of test problem `sol` (f term + Nitsche terms of
 * the Dirichlet data u_exact).  Replaces sipg_sem_2d<T>::compute_rhs
 * (sipg_sem_2d.hpp:232-305), on the device.  `modes` is used by SIPG_SOL_MODES.
 * Stream-ordered: d_b is complete once the work queued on `stream` is; the
 * call itself does not wait. */
sipg_status sipg_rhs_f64(const sipg_op* op, int sol, const sipg_modes* modes, double* d_b, void* stream);
/* err[0] = L2, err[1] = broken H1, err[2] = max nodal error of d_u against
 * test problem `sol`, at the LGL nodes as sipg_sem_2d<T>::err_norms
 * (sipg_sem_2d.hpp:311-370), on the device.  Synchronous. */
sipg_status sipg_err_norms_f64(const sipg_op* op, int sol, const sipg_modes* modes, const double* d_u, double* err,
                               void* stream);

/* ---- diagnostics ---- */

/* Text of the last error on this host thread. */
const char* sipg_last_error(void);
/* Library version string. */
const char* sipg_version(void);
/* Kernel launches issued by this process so far (all entry points). */
unsigned long long sipg_launch_count(void);
/* FP64 and FP32 FMA throughput of the current device in TFLOP/s, measured with
 * independent FMA chains (about 0.1 s); the denominator of the FP64-pipe
 * fraction that bench.py reports beside the HBM roofline. */
sipg_status sipg_probe_fma_peak(double* fp64_tflops, double* fp32_tflops);

#ifdef __cplusplus
}
#endif
#endif
