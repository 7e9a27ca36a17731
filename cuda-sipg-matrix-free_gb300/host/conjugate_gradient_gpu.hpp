// conjugate_gradient_gpu.hpp -- the reference's CG entry points
// (conjugate_gradient_gpu.hpp:18-213) over any abs_mvm operator.
//
// conjugate_gradient(problem, x, b, tol): stops when sqrt(r.r) <= tol
// (absolute) or after b.size() iterations; returns the iteration count.  An
// operator that offers a fused CG (sipg_sem_2d) runs it -- device-resident
// scalars, graph-captured iterations; any other abs_mvm runs the reference's
// loop with the library's vector steps (sipg_dot / sipg_cg_step / sipg_xpby).
// preconditioned_conjugate_gradient: the reference's PCG loop
// (conjugate_gradient_gpu.hpp:116-213) with problem._prec_mvm; on an operator
// of this library, its fused, graph-driven form (sipg_pcg_f64).
#pragma once

#include <cmath>

#include "abs_mvm.hpp"

namespace sipg_host {

inline sipg_status vdot(size_t n, const double* x, const double* y, double* r) { return sipg_dot_f64(n, x, y, r, nullptr); }
inline sipg_status vdot(size_t n, const float* x, const float* y, float* r) { return sipg_dot_f32(n, x, y, r, nullptr); }
inline sipg_status vstep(size_t n, double a, double* x, const double* p, double* r, const double* Ap) {
  return sipg_cg_step_f64(n, a, x, p, r, Ap, nullptr);
}
inline sipg_status vstep(size_t n, float a, float* x, const float* p, float* r, const float* Ap) {
  return sipg_cg_step_f32(n, a, x, p, r, Ap, nullptr);
}
inline sipg_status vxpby(size_t n, const double* x, double b, double* y) { return sipg_xpby_f64(n, x, b, y, nullptr); }
inline sipg_status vxpby(size_t n, const float* x, float b, float* y) { return sipg_xpby_f32(n, x, b, y, nullptr); }

template <typename T>
T dot(const mode_vector<T, int>& a, const mode_vector<T, int>& b) {
  T r = 0;
  check(vdot((size_t)a.size(), a.data(), b.data(), &r), "sipg_dot");
  return r;
}

}  // namespace sipg_host

template <typename FLOAT_TYPE>
int conjugate_gradient(const abs_mvm<FLOAT_TYPE>& problem, mode_vector<FLOAT_TYPE, int> x,
                       mode_vector<FLOAT_TYPE, int> b, FLOAT_TYPE tol) {
  using namespace sipg_host;
  if (auto* fused = dynamic_cast<const fused_cg_operator<FLOAT_TYPE>*>(&problem)) return fused->fused_cg(x, b, tol);
  const int noe = x.get_noe(), nompe = x.get_nompe();
  const size_t n = (size_t)b.size();
  mode_vector<FLOAT_TYPE, int> r(noe, nompe), p(noe, nompe), Ap(noe, nompe);
  // r = b - A x
  check((sipg_status)problem._mvm(x, r), "_mvm");
  check(vxpby(n, b.data(), FLOAT_TYPE(-1), r.data()), "sipg_xpby");
  check_cuda(cudaMemcpy(p.data(), r.data(), n * sizeof(FLOAT_TYPE), cudaMemcpyDeviceToDevice), "cudaMemcpy");
  FLOAT_TYPE rr_old = dot(r, r);
  const int max_it = b.size();
  int it = 0;
  while (std::sqrt(rr_old) > tol && it < max_it) {
    check((sipg_status)problem._mvm(p, Ap), "_mvm");
    const FLOAT_TYPE alpha = rr_old / dot(p, Ap);
    check(vstep(n, alpha, x.data(), p.data(), r.data(), Ap.data()), "sipg_cg_step");
    const FLOAT_TYPE rr_new = dot(r, r);
    check(vxpby(n, r.data(), rr_new / rr_old, p.data()), "sipg_xpby");
    rr_old = rr_new;
    ++it;
  }
  r.free();
  p.free();
  Ap.free();
  return it;
}

template <typename FLOAT_TYPE>
int preconditioned_conjugate_gradient(const abs_mvm<FLOAT_TYPE>& problem, mode_vector<FLOAT_TYPE, int> x,
                                      mode_vector<FLOAT_TYPE, int> b, FLOAT_TYPE tol) {
  using namespace sipg_host;
  if (auto* fused = dynamic_cast<const fused_cg_operator<FLOAT_TYPE>*>(&problem)) {
    const int it = fused->fused_pcg(x, b, tol);
    if (it >= 0) return it;
  }
  const int noe = x.get_noe(), nompe = x.get_nompe();
  const size_t n = (size_t)b.size();
  mode_vector<FLOAT_TYPE, int> r(noe, nompe), p(noe, nompe), Ap(noe, nompe), z(noe, nompe);
  check((sipg_status)problem._mvm(x, r), "_mvm");
  check(vxpby(n, b.data(), FLOAT_TYPE(-1), r.data()), "sipg_xpby");
  check((sipg_status)problem._prec_mvm(r, z), "_prec_mvm");
  check_cuda(cudaMemcpy(p.data(), z.data(), n * sizeof(FLOAT_TYPE), cudaMemcpyDeviceToDevice), "cudaMemcpy");
  FLOAT_TYPE rz_old = dot(r, z), rr = 1;
  const int max_it = b.size();
  int it = 0;
  while (std::sqrt(rr) > tol && it < max_it) {
    check((sipg_status)problem._mvm(p, Ap), "_mvm");
    const FLOAT_TYPE alpha = rz_old / dot(p, Ap);
    check(vstep(n, alpha, x.data(), p.data(), r.data(), Ap.data()), "sipg_cg_step");
    rr = dot(r, r);
    check((sipg_status)problem._prec_mvm(r, z), "_prec_mvm");
    const FLOAT_TYPE rz_new = dot(z, r);
    check(vxpby(n, z.data(), rz_new / rz_old, p.data()), "sipg_xpby");
    rz_old = rz_new;
    ++it;
  }
  r.free();
  p.free();
  Ap.free();
  z.free();
  return it;
}
