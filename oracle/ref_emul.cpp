/*
 * ref_emul.cpp -- C entry points around the reference's own code, run on the
 * CPU through cuda_emul.h.  Compiled by oracle/build_ref.py against the
 * reference headers (kernel launches rewritten for the emulation) into
 * oracle/_ref/libref_emul.so.
 *
 * TEST INFRASTRUCTURE ONLY: it produces the golden fixtures under
 * tests/golden/ (tests/golden/make_golden.py) that pin the oracle.
 */
#include "cuda_emul.h"

#include <build_square_mesh.hpp>
#include <conjugate_gradient_kernels.hpp>
#include <device_const.hpp>
#include <laplacian_operator.hpp>
#include <mode_matrix_kernels.hpp>
#include <sipg_sem_2d.hpp>
#include <sipg_sem_2d_gpu_kernels.hpp>
#include <volume_gpu_kernels.hpp>

/* The five manufactured solutions of analytical_solutions.hpp, selected there
 * by the compile-time EXACT_SOLUTION_NO; included once per solution. */
#define EXACT_SOLUTION_NO 1
namespace solA_impl {
#include <analytical_solutions.hpp>
}
#undef __ANALYTICAL_SOLUTIONS_HPP__
#undef EXACT_SOLUTION_NO
#define EXACT_SOLUTION_NO 2
namespace solB_impl {
#include <analytical_solutions.hpp>
}
#undef __ANALYTICAL_SOLUTIONS_HPP__
#undef EXACT_SOLUTION_NO
#define EXACT_SOLUTION_NO 3
namespace solC_impl {
#include <analytical_solutions.hpp>
}
#undef __ANALYTICAL_SOLUTIONS_HPP__
#undef EXACT_SOLUTION_NO
#define EXACT_SOLUTION_NO 4
namespace solD_impl {
#include <analytical_solutions.hpp>
}
#undef __ANALYTICAL_SOLUTIONS_HPP__
#undef EXACT_SOLUTION_NO
#define EXACT_SOLUTION_NO 5
namespace solE_impl {
#include <analytical_solutions.hpp>
}

#define REF_SOLUTION_DEF(NS)                                                               \
  namespace NS {                                                                           \
  static double u_ex(double x, double y) { return NS##_impl::test_func::u_ex(x, y); }       \
  static double f(double x, double y) { return NS##_impl::test_func::f(x, y); }             \
  static double dx_u_ex(double x, double y) { return NS##_impl::test_func::dx_u_ex(x, y); } \
  static double dy_u_ex(double x, double y) { return NS##_impl::test_func::dy_u_ex(x, y); } \
  }
REF_SOLUTION_DEF(solA)
REF_SOLUTION_DEF(solB)
REF_SOLUTION_DEF(solC)
REF_SOLUTION_DEF(solD)
REF_SOLUTION_DEF(solE)

/* u = sin(2 pi x) sin(2 pi y), f = 8 pi^2 u: the 16x16, p=4 Poisson case's own
 * manufactured solution (not one of the reference's A..E), fed to the
 * reference driver the same way */
namespace solS {
static const double TP = 2 * M_PI;
static double u_ex(double x, double y) { return std::sin(TP * x) * std::sin(TP * y); }
static double f(double x, double y) { return 2 * TP * TP * std::sin(TP * x) * std::sin(TP * y); }
static double dx_u_ex(double x, double y) { return TP * std::cos(TP * x) * std::sin(TP * y); }
static double dy_u_ex(double x, double y) { return TP * std::sin(TP * x) * std::cos(TP * y); }
}  // namespace solS

typedef double (*fn2)(double, double);

static int pick_solution(int sol, fn2* u, fn2* f, fn2* dx, fn2* dy) {
  switch (sol) {
#define CASE(K, NS)     \
  case K:               \
    *u = NS::u_ex;      \
    *f = NS::f;         \
    *dx = NS::dx_u_ex;  \
    *dy = NS::dy_u_ex;  \
    return 0;
    CASE(1, solA)
    CASE(2, solB)
    CASE(3, solC)
    CASE(4, solD)
    CASE(5, solE)
    CASE(6, solS)
#undef CASE
  }
  return -1;
}

template <class T>
static int apply_t(int p, int dim, T pen, const T* in, T* out) {
  load_Dphi_table<T>(p);
  load_lgl_quadrature_table<T>(p);
  square_mesh<T> mesh(dim);
  const int noe = dim * dim;
  const size_t n = (size_t)noe * (p + 1) * (p + 1);
  std::vector<T> hin(in, in + n);
  mode_vector<T, int> din(noe, p + 1, hin.data()), dout(noe, p + 1, out);
  /* launch geometry of sipg_sem_2d.hpp:103-113 and the launches of :177-188 */
  const int blockD = 128;
  const dim3 vg((noe + blockD - 1) / blockD, p + 1, p + 1), vb(blockD, 1, 1);
  const int dimx = mesh.device_info.get_dimx(), dimy = mesh.device_info.get_dimy();
  const dim3 fg((dimx + 31) / 32, (dimy + 3) / 4, 1), fb(32, 4, 1);
  emu::launch([&](auto&&... a) { volume<T>(a...); }, vg, vb)(p, din, dout);
  emu::launch([&](auto&&... a) { flux_term6a<T>(a...); }, fg, fb)(p, mesh.device_info, din, dout, pen);
  emu::launch([&](auto&&... a) { flux_term6b<T>(a...); }, fg, fb)(p, mesh.device_info, din, dout, pen);
  mesh.device_info.free();
  return 0;
}

extern "C" {

int ref_lgl(int npts, double* nodes, double* weights) {
  LGL_quadrature_table<double> qt(npts);
  for (int i = 0; i < npts; ++i) {
    nodes[i] = qt.node(i);
    weights[i] = qt.weight(i);
  }
  return 0;
}

int ref_lgl_f32(int npts, float* nodes, float* weights) {
  LGL_quadrature_table<float> qt(npts);
  for (int i = 0; i < npts; ++i) {
    nodes[i] = qt.node(i);
    weights[i] = qt.weight(i);
  }
  return 0;
}

int ref_dphi(int p, double* D) {
  std::vector<double> v;
  DbaseVALUES<double>(p, v);
  for (size_t i = 0; i < v.size(); ++i) D[i] = v[i];
  return 0;
}

/* (p+1)^4 entries, in the order of sem_laplacian_gpu_validation_test.cu:46-63 */
int ref_laplace2d(int p, double* L) {
  laplace_2d<double> lap(p);
  size_t at = 0;
  for (int i1 = 0; i1 <= p; ++i1)
    for (int i2 = 0; i2 <= p; ++i2)
      for (int j1 = 0; j1 <= p; ++j1)
        for (int j2 = 0; j2 <= p; ++j2) L[at++] = lap(i1, i2, j1, j2);
  return 0;
}

int ref_mesh_coords(int dim, double* x, double* y) {
  square_mesh<double> mesh(dim);
  const int noe = dim * dim;
  for (int i = 0; i < 4 * noe; ++i) {
    x[i] = mesh.x_coord()[i];
    y[i] = mesh.y_coord()[i];
  }
  mesh.device_info.free();
  return 0;
}

int ref_apply(int p, int dim, double pen, const double* in, double* out) { return apply_t<double>(p, dim, pen, in, out); }

int ref_apply_f32(int p, int dim, float pen, const float* in, float* out) { return apply_t<float>(p, dim, pen, in, out); }

/* volume_mvm<double, 1> with host_laplacian_matrix(1, p): the USE_MODE_MATRIX
 * volume path (sipg_sem_2d.hpp:116-119,172-176) */
int ref_volume_mvm(int p, int dim, const double* in, double* out) {
  load_Dphi_table<double>(p);
  load_lgl_quadrature_table<double>(p);
  const int noe = dim * dim;
  const size_t n = (size_t)noe * (p + 1) * (p + 1);
  std::vector<double> hin(in, in + n);
  mode_vector<double, int> din(noe, p + 1, hin.data()), dout(noe, p + 1, out);
  host_laplacian_matrix<double, int> hm(1, p);
  mode_matrix<double, int> dm;
  dm = hm;
  const int blockD = 128;
  emu::launch([&](auto&&... a) { volume_mvm<double, 1>(a...); }, dim3((noe + blockD - 1) / blockD, p + 1, p + 1),
              dim3(blockD, 1, 1))(p, dm, din, dout);
  dm.free();
  return 0;
}

/* The whole reference driver: sipg_sem_2d<double>(p, square_mesh(dim), f, u_ex,
 * dx_u_ex, dy_u_ex, pen, tol) -- RHS, CG (absolute tolerance), copy back and
 * error norms (sipg_sem_2d.hpp:83-145).  stats = {iterations, L2, H1, max}. */
int ref_solve(int p, int dim, double pen, double tol, int sol, double* u_out, double* stats) {
  fn2 u, f, dx, dy;
  if (pick_solution(sol, &u, &f, &dx, &dy)) return -1;
  square_mesh<double> mesh(dim);
  {
    sipg_sem_2d<double> prob(p, mesh, f, u, dx, dy, pen, tol);
    stats[0] = prob.iterations;
    stats[1] = prob.L2_err;
    stats[2] = prob.H1_err;
    stats[3] = prob.max_err;
    if (u_out) {
      const size_t n = (size_t)dim * dim * (p + 1) * (p + 1);
      const double* s = prob.solution.data();
      for (size_t i = 0; i < n; ++i) u_out[i] = s[i];
    }
  }
  mesh.device_info.free();
  return 0;
}

/* The right-hand side alone, read from the sipg_sem_2d driver with tol = inf
 * (CG exits before its first iteration, so d_rhs is compute_rhs's output). */
int ref_rhs(int p, int dim, double pen, int sol, double* b) {
  fn2 u, f, dx, dy;
  if (pick_solution(sol, &u, &f, &dx, &dy)) return -1;
  square_mesh<double> mesh(dim);
  {
    sipg_sem_2d<double> prob(p, mesh, f, u, dx, dy, pen, 1e300);
    const size_t n = (size_t)dim * dim * (p + 1) * (p + 1);
    std::memcpy(b, prob.d_rhs.data(), n * sizeof(double));
  }
  mesh.device_info.free();
  return 0;
}

#ifdef USE_PRECONDITIONER
/* Built a second time with -DUSE_PRECONDITIONER into libref_emul_pcg.so:
 * the block-Jacobi path.  ref_solve above then runs the preconditioned CG
 * (sipg_sem_2d.hpp:121-134).  ref_prec_block: the block the reference builds
 * (laplacian_operator.hpp:133-186) before, and its inverse after, the LAPACK
 * calls (lapacke_emul/lapacke.h stands in for LAPACK).  ref_prec_rows: the
 * (2p+1) entries per row of host_preconditioner_matrix (mode_matrix.hpp:
 * 474-522), rows[((i1*(p+1)+i2)*(2p+1)) + r]. */
int ref_prec_block(int p, double pen, double* block, double* inverse) {
  block_diagonal_preconditioner_2d prec(p, pen);
  const size_t nn = (size_t)(p + 1) * (p + 1);
  const std::vector<double>& a0 = lapacke_emul::last_factored();
  if (a0.size() != nn * nn) return -1;
  for (size_t i = 0; i < nn * nn; ++i) {
    block[i] = a0[i];
    inverse[i] = prec.a[i];
  }
  return 0;
}

int ref_prec_rows(int p, double pen, double* rows) {
  host_preconditioner_matrix<double, int> m(1, p, pen);
  const int n = p + 1, R = 2 * p + 1;
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2)
      for (int r = 0; r < R; ++r) rows[(size_t)(i1 * n + i2) * R + r] = m(i1, i2, r, 0);
  return 0;
}
#endif
}
