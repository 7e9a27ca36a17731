// abs_mvm.hpp -- the operator interface consumed by conjugate_gradient, with
// the reference's signatures (abs_mvm.hpp:10-19): _mvm(in, out) applies the
// operator, _prec_mvm(in, out) the preconditioner; both return 0 on success.
#pragma once

#include "mode_vector.hpp"

template <typename FLOAT_TYPE>
class abs_mvm {
 public:
  virtual ~abs_mvm() {}
  virtual int _mvm(mode_vector<FLOAT_TYPE, int>, mode_vector<FLOAT_TYPE, int>) const = 0;
  virtual int _prec_mvm(mode_vector<FLOAT_TYPE, int>, mode_vector<FLOAT_TYPE, int>) const = 0;
};

// Implemented by operators that have a fused, graph-driven CG of their own
// (sipg_sem_2d); conjugate_gradient() uses it when the operator offers it.
template <typename FLOAT_TYPE>
class fused_cg_operator {
 public:
  virtual ~fused_cg_operator() {}
  // absolute tolerance on sqrt(r.r), max_it = DoF, as conjugate_gradient
  virtual int fused_cg(mode_vector<FLOAT_TYPE, int> x, mode_vector<FLOAT_TYPE, int> b, FLOAT_TYPE tol) const = 0;
  // the same with the operator's block-Jacobi preconditioner, as
  // preconditioned_conjugate_gradient; -1 where the operator has none
  virtual int fused_pcg(mode_vector<FLOAT_TYPE, int>, mode_vector<FLOAT_TYPE, int>, FLOAT_TYPE) const { return -1; }
};
