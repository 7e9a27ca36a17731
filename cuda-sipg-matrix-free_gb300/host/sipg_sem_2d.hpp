// sipg_sem_2d.hpp -- the SIPG-SEM Poisson problem with the reference's class
// interface (sipg_sem_2d.hpp:32-228): the constructor builds the right-hand
// side, solves with conjugate_gradient (absolute tolerance) and computes the
// error norms; the public members are those of the reference.  The operator is
// the library's fused apply (one kernel instead of volume + flux_term6a +
// flux_term6b), the CG the library's fused, graph-driven CG.
//
// With host callbacks (f, u_ex, dx_u_ex, dy_u_ex) the right-hand side and the
// norms are computed on the host in FLOAT_TYPE, as the reference does
// (compute_rhs :232-305, err_norms :311-370).  With a built-in problem id
// (FP64) both run on the device (sipg_rhs_f64, sipg_err_norms_f64).
// Defining USE_MODE_MATRIX (the reference's stored-operator volume kernel,
// volume_mvm<T,1> with host_laplacian_matrix) changes nothing here: the
// stored Laplacian is the volume term the fused apply computes, so both
// settings solve the same system (the stored form is available as
// sipg_laplacian_rows_f64 + sipg_volume_mvm_f64).
// As in the reference, defining USE_PRECONDITIONER before including this
// header makes the solve the block-Jacobi preconditioned CG and _prec_mvm the
// block-Jacobi preconditioner (sipg_apply_prec_f64 / sipg_pcg_f64; FP64);
// without it _prec_mvm copies its input (the reference's leaves the output
// untouched).
#pragma once

#include <cmath>
#include <iomanip>
#include <iostream>
#include <type_traits>
#include <vector>

#include "CUDA_TIMER.hpp"
#include "build_square_mesh.hpp"
#include "conjugate_gradient_gpu.hpp"
#include "sem_function.hpp"

template <typename FLOAT_TYPE>
class sipg_sem_2d : public abs_mvm<FLOAT_TYPE>, public fused_cg_operator<FLOAT_TYPE> {
  static_assert(std::is_same<FLOAT_TYPE, double>::value || std::is_same<FLOAT_TYPE, float>::value,
                "sipg_sem_2d<T>: T must be double or float");
  typedef FLOAT_TYPE (*fn2)(FLOAT_TYPE, FLOAT_TYPE);

  int order;
  square_mesh<FLOAT_TYPE> mesh;
  LGL_quadrature_table<FLOAT_TYPE> qt;
  sem_function<FLOAT_TYPE> basis;
  FLOAT_TYPE pen;
  sipg_op* op = nullptr;
  CUDA_TIMER system_solution_time;

  void setup(int _order, const square_mesh<FLOAT_TYPE>& _mesh) {
    order = _order;
    mesh = _mesh;
    sipg_host::check(sipg_op_create(mesh.dim(), order, (double)pen, &op), "sipg_op_create");
    host_mode_vector<FLOAT_TYPE, int> zeros(mesh.noe(), order + 1);
    copy(zeros, d_u);
  }

  void solve(FLOAT_TYPE tol) {
    system_solution_time.start();
#ifdef USE_PRECONDITIONER
    iterations = preconditioned_conjugate_gradient(*this, d_u, d_rhs, tol);
#else
    iterations = conjugate_gradient(*this, d_u, d_rhs, tol);
#endif
    system_solution_time.stop();
    copy(d_u, solution);
  }

 public:
  FLOAT_TYPE max_err = 0, L2_err = 0, H1_err = 0;
  int iterations = 0;
  mode_vector<FLOAT_TYPE, int> d_u, d_rhs;
  host_mode_vector<FLOAT_TYPE, int> solution;

  sipg_sem_2d(int _order, const square_mesh<FLOAT_TYPE>& _mesh, fn2 f, fn2 u_ex, fn2 dx_u_ex, fn2 dy_u_ex,
              FLOAT_TYPE _pen, FLOAT_TYPE _tol)
      : qt(_order + 1), basis(_order), pen(_pen) {
    setup(_order, _mesh);
    compute_rhs(f, u_ex);
    solve(_tol);
    err_norms(solution, u_ex, dx_u_ex, dy_u_ex);
  }

  // built-in test problem (sipg_solution), right-hand side and norms on the device; FP64
  sipg_sem_2d(int _order, const square_mesh<FLOAT_TYPE>& _mesh, sipg_solution sol, FLOAT_TYPE _pen, FLOAT_TYPE _tol)
      : qt(_order + 1), basis(_order), pen(_pen) {
    static_assert(std::is_same<FLOAT_TYPE, double>::value, "device right-hand side is FP64");
    setup(_order, _mesh);
    d_rhs = mode_vector<FLOAT_TYPE, int>(mesh.noe(), order + 1);
    sipg_host::check(sipg_rhs_f64(op, sol, nullptr, d_rhs.data(), nullptr), "sipg_rhs_f64");
    solve(_tol);
    double e[3];
    sipg_host::check(sipg_err_norms_f64(op, sol, nullptr, d_u.data(), e, nullptr), "sipg_err_norms_f64");
    L2_err = e[0];
    H1_err = e[1];
    max_err = e[2];
  }

  ~sipg_sem_2d() {
    d_rhs.free();
    d_u.free();
    sipg_op_destroy(op);
  }
  sipg_sem_2d(const sipg_sem_2d&) = delete;
  sipg_sem_2d& operator=(const sipg_sem_2d&) = delete;

  float solution_time() { return system_solution_time.elapsed_millisecs(); }

  int _mvm(mode_vector<FLOAT_TYPE, int> input, mode_vector<FLOAT_TYPE, int> output) const override {
    if (std::is_same<FLOAT_TYPE, double>::value)
      return (int)sipg_apply_f64(op, (const double*)input.data(), (double*)output.data(), nullptr);
    return (int)sipg_apply_f32(op, (const float*)input.data(), (float*)output.data(), nullptr);
  }

  int _prec_mvm(mode_vector<FLOAT_TYPE, int> input, mode_vector<FLOAT_TYPE, int> output) const override {
#ifdef USE_PRECONDITIONER
    if (std::is_same<FLOAT_TYPE, double>::value)
      return (int)sipg_apply_prec_f64(op, (const double*)input.data(), (double*)output.data(), nullptr);
#endif
    return (int)cudaMemcpy(output.data(), input.data(), sizeof(FLOAT_TYPE) * (size_t)input.size(),
                           cudaMemcpyDeviceToDevice);
  }

  int fused_pcg(mode_vector<FLOAT_TYPE, int> x, mode_vector<FLOAT_TYPE, int> b, FLOAT_TYPE tol) const override {
#ifdef USE_PRECONDITIONER
    if (std::is_same<FLOAT_TYPE, double>::value) {
      sipg_cg_result r;
      const sipg_status s = sipg_pcg_f64(op, (double*)x.data(), (const double*)b.data(), (double)tol, 0, 0, &r, nullptr);
      if (s != SIPG_OK && s != SIPG_ERR_NOT_CONVERGED) sipg_host::check(s, "sipg_pcg_f64");
      return r.iterations;
    }
#endif
    (void)x;
    (void)b;
    (void)tol;
    return -1;
  }

  int fused_cg(mode_vector<FLOAT_TYPE, int> x, mode_vector<FLOAT_TYPE, int> b, FLOAT_TYPE tol) const override {
    sipg_cg_result r;
    sipg_status s;
    if (std::is_same<FLOAT_TYPE, double>::value)
      s = sipg_cg_f64(op, (double*)x.data(), (const double*)b.data(), (double)tol, 0, 0, &r, nullptr);
    else
      s = sipg_cg_f32(op, (float*)x.data(), (const float*)b.data(), (float)tol, 0, 0, &r, nullptr);
    if (s != SIPG_OK && s != SIPG_ERR_NOT_CONVERGED) sipg_host::check(s, "sipg_cg");
    return r.iterations;
  }

  // compute_rhs of the reference: quadrature of f, then the Nitsche terms of
  // the Dirichlet data u_ex on the four boundary strips (penalty pen * w_i * g,
  // consistency -/+ w_i D[j][0 or p] g)
  void compute_rhs(fn2 f, fn2 u_ex) {
    const int N = order, dim = mesh.dim(), noe = mesh.noe();
    host_mode_vector<FLOAT_TYPE, int> rhs(noe, N + 1);
    const std::vector<FLOAT_TYPE>& x = mesh.x_coord();
    const std::vector<FLOAT_TYPE>& y = mesh.y_coord();
    std::vector<FLOAT_TYPE> nodes(N + 1), weights(N + 1), w(N + 1);
    for (int i = 0; i <= N; ++i) {
      nodes[i] = (qt.node(i) * .5 + .5) / dim;
      weights[i] = qt.weight(i);
      w[i] = qt.weight(i) * .5 / dim;
    }
    for (int i1 = 0; i1 <= N; ++i1)
      for (int i2 = 0; i2 <= N; ++i2)
        for (int e = 0; e < noe; ++e) rhs(i1, i2, e) = w[i1] * w[i2] * f(x[e] + nodes[i1], y[e] + nodes[i2]);
    for (int xx = 0; xx < dim; ++xx) {
      const int eD = (dim - 1) * dim + xx, eU = xx, eL = xx * dim, eR = xx * dim + dim - 1;
      for (int i = 0; i <= N; ++i) {
        const FLOAT_TYPE gD = u_ex(x[eD] + nodes[i], y[eD] + nodes[0]);
        const FLOAT_TYPE gU = u_ex(x[eU] + nodes[i], y[eU] + nodes[N]);
        const FLOAT_TYPE gL = u_ex(x[eL] + nodes[0], y[eL] + nodes[i]);
        const FLOAT_TYPE gR = u_ex(x[eR] + nodes[N], y[eR] + nodes[i]);
        rhs(i, 0, eD) += pen * weights[i] * gD;
        rhs(i, N, eU) += pen * weights[i] * gU;
        rhs(0, i, eL) += pen * weights[i] * gL;
        rhs(N, i, eR) += pen * weights[i] * gR;
        for (int j = 0; j <= N; ++j) {
          rhs(i, j, eD) -= -1 * weights[i] * basis.d_phi(j, 0) * gD;
          rhs(i, j, eU) -= weights[i] * basis.d_phi(j, N) * gU;
          rhs(j, i, eL) -= -1 * weights[i] * basis.d_phi(j, 0) * gL;
          rhs(j, i, eR) -= weights[i] * basis.d_phi(j, N) * gR;
        }
      }
    }
    copy(rhs, d_rhs);
  }

  // err_norms of the reference: nodal max error, LGL-quadrature L2 and broken H1
  void err_norms(host_mode_vector<FLOAT_TYPE, int>& u, fn2 u_ex, fn2 dx_u_ex, fn2 dy_u_ex) {
    const int dim = mesh.dim(), noe = mesh.noe(), n = order + 1;
    std::vector<FLOAT_TYPE> nodes(n), weights(n);
    for (int i = 0; i < n; ++i) {
      nodes[i] = (qt.node(i) * .5 + .5) / dim;
      weights[i] = qt.weight(i) * .5 / dim;
    }
    FLOAT_TYPE dxs = 0, dys = 0, l2s = 0;
    max_err = -1;
    for (int e = 0; e < noe; ++e)
      for (int p = 0; p < n; ++p)
        for (int q = 0; q < n; ++q) {
          FLOAT_TYPE dx_u = 0, dy_u = 0;
          for (int i = 0; i < n; ++i) {
            dx_u += u(i, q, e) * 2 * dim * basis.d_phi(i, p);
            dy_u += u(p, i, e) * 2 * dim * basis.d_phi(i, q);
          }
          const FLOAT_TYPE xe = mesh.x_coord()[e], ye = mesh.y_coord()[e];
          const FLOAT_TYPE w2 = weights[p] * weights[q];
          const FLOAT_TYPE err = std::fabs(u(p, q, e) - u_ex(xe + nodes[p], ye + nodes[q]));
          if (err > max_err) max_err = err;
          l2s += w2 * err * err;
          const FLOAT_TYPE ex = dx_u - dx_u_ex(xe + nodes[p], ye + nodes[q]);
          const FLOAT_TYPE ey = dy_u - dy_u_ex(xe + nodes[p], ye + nodes[q]);
          dxs += w2 * ex * ex;
          dys += w2 * ey * ey;
        }
    L2_err = std::sqrt(l2s);
    H1_err = std::sqrt(l2s + dxs + dys);
  }

  void print_result() {
    const int noe = mesh.noe(), dim = mesh.dim();
    for (int e = 0; e < noe; ++e) {
      for (int i = 0; i <= order; ++i)
        for (int j = 0; j <= order; ++j)
          std::cerr << std::setw(10) << mesh.x_coord()[e] + (qt.node(i) * .5 + .5) / dim << "\t" << std::setw(10)
                    << mesh.y_coord()[e] + (qt.node(j) * .5 + .5) / dim << "\t" << std::setw(10)
                    << solution(i, j, e) << std::endl;
      std::cerr << std::endl;
    }
  }
};
