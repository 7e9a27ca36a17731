/*
 * sipg_oracle.h -- CPU restatement of the reference SIPG-SEM algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it may be linked or
 * loaded by tests/, by __graft_entry__.smoke() and by the cpu_baseline /
 * --impl reference legs of bench.py, and by nothing else.  The product path
 * (libsipg_gb300.so) never calls it and fails loudly without its CUDA build.
 *
 * Every function restates one piece of paogor/CUDA-SIPG-matrix-free and cites
 * the reference file:line it follows.  Arithmetic is written in the same
 * operation order as the reference and compiled with -ffp-contract=off, so the
 * results are bit-identical to the reference's own code run on a CPU (see
 * oracle/build_ref.py, which builds that emulation from the reference sources
 * and is how the golden fixtures under tests/golden/ were produced).
 *
 * Layout everywhere: node-major SoA, value (i1,i2) of element e at
 * ((i1*(p+1)+i2)*noe + e), noe = dim*dim, element e = row*dim + col with row 0
 * at the top of the unit square (mode_vector.hpp:108-120,
 * build_square_mesh.hpp:250-288).
 */
#ifndef SIPG_ORACLE_H
#define SIPG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Analytic test problems.  1..5 are the reference's solutions A..E
 * (validation_tests/analytical_solutions.hpp:7-94, PI = 3.14159265359);
 * 6 is u = sin(2 pi x) sin(2 pi y), f = 8 pi^2 u (with the C library's pi);
 * 7 is a sum of modes A_m sin(k_m pi x) sin(l_m pi y) given by `modes`. */
enum { OR_SOL_A = 1, OR_SOL_B, OR_SOL_C, OR_SOL_D, OR_SOL_E, OR_SOL_SINSIN, OR_SOL_MODES };

typedef struct {
  int nmodes;            /* <= 8 */
  double amp[8];
  int k[8], l[8];
} or_modes;

/* LGL nodes and weights, npts = p+1 points (LGL_quadrature_table.hpp:84-146). */
int sipg_oracle_lgl(int npts, double* nodes, double* weights);
/* D[mode*(p+1)+node] = derivative of Lagrange basis `mode` at LGL node `node`
 * (sem_function.hpp:86-110, device_const.hpp:115-127). */
int sipg_oracle_dphi(int p, double* D);
/* Element Laplacian, (p+1)^4 entries L[((i1*n+i2)*n+j1)*n+j2]
 * (laplacian_operator.hpp:67-88). */
int sipg_oracle_laplace2d(int p, double* L);
/* Element corner coordinates, x[c*noe+e], y[c*noe+e], c = 0..3
 * (build_square_mesh.hpp:250-288). */
int sipg_oracle_mesh_coords(int dim, double* x, double* y);

/* One SIPG matvec out = A in: volume (volume_gpu_kernels.hpp:9-86), then
 * flux_term6a (sipg_sem_2d_gpu_kernels.hpp:189-253), then flux_term6b
 * (:256-316).  nthreads <= 1 runs on the calling thread. */
int sipg_oracle_apply(int p, int dim, double pen, const double* in, double* out, int nthreads);
int sipg_oracle_apply_f32(int p, int dim, float pen, const float* in, float* out, int nthreads);
/* The three pieces separately (same arithmetic as sipg_oracle_apply). */
int sipg_oracle_volume(int p, int dim, const double* in, double* out);
int sipg_oracle_flux_x(int p, int dim, double pen, const double* in, double* out);
int sipg_oracle_flux_y(int p, int dim, double pen, const double* in, double* out);

/* Conjugate gradient of conjugate_gradient_gpu.hpp:18-109: stops when
 * sqrt(r.r) <= tol (absolute, as the reference) or after max_it iterations
 * (max_it <= 0 means DoF, as the reference).  If rel != 0 the stop is
 * tol * ||b||.  x holds x0 on entry.  Returns the iteration count; *rr_out
 * receives the final r.r. */
int sipg_oracle_cg(int p, int dim, double pen, double* x, const double* b, double tol, int rel,
                   int max_it, double* rr_out, int nthreads);

/* Block-Jacobi preconditioner of the reference's USE_PRECONDITIONER path.
 * sipg_oracle_prec_block: the interior element's diagonal block of the SIPG
 * matrix, (p+1)^2 x (p+1)^2, row (p+1)*i2+i1, column (p+1)*j2+j1
 * (laplacian_operator.hpp:104-186; the penalty is truncated to an int as the
 * reference's constructor parameter does, :116).
 * sipg_oracle_invert: the inverse in place by LU with partial pivoting and
 * substitution, the computation of LAPACK's dgetrf + dgetri that the
 * reference calls (lapack_wrapper.cpp:29-42; another LAPACK build agrees to
 * rounding).  Returns -1 for a singular matrix.
 * sipg_oracle_prec_rows: the inverse kept on the "cross" pattern of the
 * stored-operator kernel, 2p+1 entries per row in that kernel's order --
 * (i1,i2), then (i1,j) j != i2, then (j,i2) j != i1 -- at
 * rows[((i1*(p+1)+i2)*(2p+1)) + r] (mode_matrix.hpp:491-518).
 * sipg_oracle_prec_apply: out = M in with those rows, element by element
 * (volume_mvm<T,1>, mode_matrix_kernels.hpp:7-65).
 * sipg_oracle_pcg: preconditioned CG of conjugate_gradient_gpu.hpp:116-213
 * (stop on sqrt(r.r) <= tol, absolute, or tol*||b|| if rel; the first
 * iteration always runs, as the reference's rr starts at 1). */
int sipg_oracle_prec_block(int p, double pen, double* A);
int sipg_oracle_invert(int n, double* A);
int sipg_oracle_prec_rows(int p, double pen, double* rows);
int sipg_oracle_prec_apply(int p, int dim, const double* rows, const double* in, double* out);
int sipg_oracle_pcg(int p, int dim, double pen, double* x, const double* b, double tol, int rel, int max_it,
                    double* rr_out, int nthreads);

/* compute_rhs (sipg_sem_2d.hpp:232-305) for test problem `sol`. */
int sipg_oracle_rhs(int p, int dim, double pen, int sol, const or_modes* modes, double* b);
/* err_norms (sipg_sem_2d.hpp:311-370): out[0]=L2, out[1]=H1, out[2]=max. */
int sipg_oracle_err_norms(int p, int dim, int sol, const or_modes* modes, const double* u, double* out);

/* Exact solution value of a test problem (for tests). */
double sipg_oracle_u_exact(int sol, const or_modes* modes, double x, double y);

/* Portable seeded generator for synthetic inputs: splitmix64 stream -> uniform
 * doubles in [lo, hi), written in linear index order. */
void sipg_oracle_fill_uniform(unsigned long long seed, double lo, double hi, double* out, long long n);

#ifdef __cplusplus
}
#endif
#endif
