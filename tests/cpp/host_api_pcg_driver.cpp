// host_api_pcg_driver.cpp -- the reference's preconditioned configuration
// (sipg_2d_h_adaptivity.cu defines USE_PRECONDITIONER before including the
// headers) driven through the C++ host API: h-sweep rows, and a user operator
// whose _prec_mvm is the library's block-Jacobi preconditioner, solved by the
// generic preconditioned_conjugate_gradient loop.  One JSON object per line
// for tests/test_gpu_pcg.py.
#define USE_PRECONDITIONER
#include <cmath>
#include <cstdio>

#include "sipg_sem_2d.hpp"

namespace test_func {
// solution E of the reference's validation (cos 8 pi x + cos 8 pi y), with its PI literal
const double PI = 3.14159265359;
double u_ex(double x, double y) { return std::cos(8 * PI * x) + std::cos(8 * PI * y); }
double f(double x, double y) { return 64 * PI * PI * std::cos(8 * PI * x) + 64 * PI * PI * std::cos(8 * PI * y); }
double dx_u_ex(double x, double) { return -8 * PI * std::sin(8 * PI * x); }
double dy_u_ex(double, double y) { return -8 * PI * std::sin(8 * PI * y); }
}  // namespace test_func

class user_operator : public abs_mvm<double> {
  sipg_op* op;

 public:
  user_operator(int dim, int p, double pen) { sipg_host::check(sipg_op_create(dim, p, pen, &op), "create"); }
  ~user_operator() { sipg_op_destroy(op); }
  int _mvm(mode_vector<double, int> in, mode_vector<double, int> out) const override {
    return (int)sipg_apply_f64(op, in.data(), out.data(), nullptr);
  }
  int _prec_mvm(mode_vector<double, int> in, mode_vector<double, int> out) const override {
    return (int)sipg_apply_prec_f64(op, in.data(), out.data(), nullptr);
  }
};

int main() {
  using namespace test_func;
  for (int p = 2; p <= 4; ++p)
    for (int dim = 4; dim <= 16; dim *= 2) {
      square_mesh<double> mesh(dim);
      sipg_sem_2d<double> prob(p, mesh, f, u_ex, dx_u_ex, dy_u_ex, 100.0 * p * p, 1e-15);
      std::printf("{\"case\": \"pcg\", \"dim\": %d, \"p\": %d, \"pen\": %g, \"tol\": 1e-15, \"it\": %d, \"L2\": %.17g, "
                  "\"H1\": %.17g, \"max\": %.17g}\n",
                  dim, p, 100.0 * p * p, prob.iterations, prob.L2_err, prob.H1_err, prob.max_err);
    }
  {
    const int dim = 12, p = 3;
    const double pen = 9.0, tol = 1e-12;
    square_mesh<double> mesh(dim);
    sipg_sem_2d<double> prob(p, mesh, f, u_ex, dx_u_ex, dy_u_ex, pen, tol);
    user_operator uop(dim, p, pen);
    mode_vector<double, int> x(dim * dim, p + 1);
    cudaMemset(x.data(), 0, sizeof(double) * x.size());
    const int it = preconditioned_conjugate_gradient(uop, x, prob.d_rhs, tol);
    host_mode_vector<double, int> hx(x);
    double diff = 0, ref = 0;
    for (int i = 0; i < hx.size(); ++i) {
      diff = std::fmax(diff, std::fabs(hx.data()[i] - prob.solution.data()[i]));
      ref = std::fmax(ref, std::fabs(prob.solution.data()[i]));
    }
    std::printf("{\"case\": \"generic\", \"it_generic\": %d, \"it_fused\": %d, \"rel_diff\": %.3g}\n", it,
                prob.iterations, diff / ref);
    x.free();
  }
  return 0;
}
