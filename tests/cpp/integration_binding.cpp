// The reference-side binding shown in INTEGRATION.md, compiled against the
// host headers that restate the reference's classes (compile-only check in
// test_capi_cpu.py: the documented snippet stays valid).
#include <stdexcept>

#include <abs_mvm.hpp>
#include <mode_vector.hpp>

#include "sipg_gb300.h"

class sipg_gb300_mvm : public abs_mvm<double> {
  sipg_op* op_ = nullptr;

 public:
  sipg_gb300_mvm(int dim, int degree, double pen) {
    if (sipg_op_create(dim, degree, pen, &op_) != SIPG_OK) throw std::runtime_error(sipg_last_error());
  }
  ~sipg_gb300_mvm() { sipg_op_destroy(op_); }
  int _mvm(mode_vector<double, int> in, mode_vector<double, int> out) const override {
    return sipg_apply_f64(op_, in.data(), out.data(), nullptr);  // 0 == SIPG_OK
  }
  int _prec_mvm(mode_vector<double, int> in, mode_vector<double, int> out) const override {
    return (int)cudaMemcpy(out.data(), in.data(), in.size() * sizeof(double), cudaMemcpyDeviceToDevice);
  }
  // the fused, graph-driven CG (absolute tolerance, as conjugate_gradient)
  int solve(mode_vector<double, int> x, mode_vector<double, int> b, double tol) {
    sipg_cg_result r;
    sipg_status s = sipg_cg_f64(op_, x.data(), b.data(), tol, 0, 0, &r, nullptr);
    return (s == SIPG_OK || s == SIPG_ERR_NOT_CONVERGED) ? r.iterations : -1;
  }
};

int main() { return 0; }
