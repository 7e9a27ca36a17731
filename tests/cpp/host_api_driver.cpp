// host_api_driver.cpp -- drives the C++ host API the way the reference's
// validation drivers drive theirs (sipg_2d_p_adaptivity.cu,
// sipg_2d_h_adaptivity.cu): construct square_mesh and sipg_sem_2d with host
// callbacks, read iterations and error norms.  Prints one JSON object per line
// for tests/test_gpu_host_api.py.
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
float u_ex_f(float x, float y) { return (float)u_ex(x, y); }
float f_f(float x, float y) { return (float)f(x, y); }
float dx_f(float x, float y) { return (float)dx_u_ex(x, y); }
float dy_f(float x, float y) { return (float)dy_u_ex(x, y); }
}  // namespace test_func

// a user operator that is not sipg_sem_2d: the generic conjugate_gradient path
class wrapped_operator : public abs_mvm<double> {
  sipg_op* op;

 public:
  wrapped_operator(int dim, int p, double pen) { sipg_host::check(sipg_op_create(dim, p, pen, &op), "create"); }
  ~wrapped_operator() { sipg_op_destroy(op); }
  int _mvm(mode_vector<double, int> in, mode_vector<double, int> out) const override {
    return (int)sipg_apply_f64(op, in.data(), out.data(), nullptr);
  }
  int _prec_mvm(mode_vector<double, int> in, mode_vector<double, int> out) const override {
    return (int)cudaMemcpy(out.data(), in.data(), sizeof(double) * in.size(), cudaMemcpyDeviceToDevice);
  }
};

int main() {
  using namespace test_func;
  // p-adaptivity shape: 16 x 16 mesh, p = 1..8, penalty p^2, absolute tolerance 1e-14
  {
    square_mesh<double> mesh(16);
    for (int p = 1; p <= 8; ++p) {
      sipg_sem_2d<double> prob(p, mesh, f, u_ex, dx_u_ex, dy_u_ex, double(p * p), 1e-14);
      std::printf("{\"case\": \"p\", \"dim\": 16, \"p\": %d, \"pen\": %g, \"tol\": 1e-14, \"it\": %d, \"L2\": %.17g, "
                  "\"H1\": %.17g, \"max\": %.17g}\n",
                  p, double(p * p), prob.iterations, prob.L2_err, prob.H1_err, prob.max_err);
    }
    mesh.device_info.free();
  }
  // h-adaptivity shape: p = 2..4, dim = 4..32, penalty 100 p^2 (the thesis' tables)
  for (int p = 2; p <= 4; ++p)
    for (int dim = 4; dim <= 32; dim *= 2) {
      square_mesh<double> mesh(dim);
      sipg_sem_2d<double> prob(p, mesh, f, u_ex, dx_u_ex, dy_u_ex, 100.0 * p * p, 1e-15);
      std::printf("{\"case\": \"h\", \"dim\": %d, \"p\": %d, \"pen\": %g, \"tol\": 1e-15, \"it\": %d, \"L2\": %.17g, "
                  "\"H1\": %.17g, \"max\": %.17g, \"ms\": %g}\n",
                  dim, p, 100.0 * p * p, prob.iterations, prob.L2_err, prob.H1_err, prob.max_err,
                  prob.solution_time());
    }
  // built-in problem, device RHS and norms
  {
    square_mesh<double> mesh(16);
    sipg_sem_2d<double> prob(4, mesh, SIPG_SOL_E, 1600.0, 1e-15);
    std::printf("{\"case\": \"device\", \"dim\": 16, \"p\": 4, \"pen\": 1600, \"it\": %d, \"L2\": %.17g, \"H1\": %.17g}\n",
                prob.iterations, prob.L2_err, prob.H1_err);
  }
  // FP32 instantiation
  {
    square_mesh<float> mesh(8);
    sipg_sem_2d<float> prob(3, mesh, f_f, u_ex_f, dx_f, dy_f, 9.0f, 1e-4f);
    std::printf("{\"case\": \"f32\", \"dim\": 8, \"p\": 3, \"it\": %d, \"L2\": %.9g, \"H1\": %.9g}\n", prob.iterations,
                prob.L2_err, prob.H1_err);
  }
  // a user abs_mvm through the generic conjugate_gradient loop
  {
    const int dim = 12, p = 3;
    const double pen = 9.0;
    square_mesh<double> mesh(dim);
    sipg_sem_2d<double> prob(p, mesh, f, u_ex, dx_u_ex, dy_u_ex, pen, 1e-12);
    wrapped_operator wop(dim, p, pen);
    mode_vector<double, int> x(dim * dim, p + 1);
    cudaMemset(x.data(), 0, sizeof(double) * x.size());
    const int it = conjugate_gradient(wop, x, prob.d_rhs, 1e-12);
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
