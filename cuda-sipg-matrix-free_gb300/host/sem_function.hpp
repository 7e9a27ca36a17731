// sem_function.hpp -- nodal Lagrange basis on the LGL nodes, with the
// reference's interface (sem_function.hpp:15-57): phi(mode, node) is the
// Kronecker delta, d_phi(mode, node) the derivative of basis `mode` at LGL node
// `node` (library table sipg_dphi_table).
#pragma once

#include <vector>

#include "LGL_quadrature_table.hpp"

template <typename FLOAT_TYPE>
class sem_function {
  int _degree;
  std::vector<FLOAT_TYPE> _D;

 public:
  LGL_quadrature_table<FLOAT_TYPE> _qt;

  explicit sem_function(int degree) : _degree(degree), _qt(degree + 1) {
    std::vector<double> D((degree + 1) * (degree + 1));
    sipg_host::check(sipg_dphi_table(degree, D.data()), "sipg_dphi_table");
    _D.assign(D.begin(), D.end());
  }
  int non() const { return _degree + 1; }
  int nom() const { return _degree + 1; }
  FLOAT_TYPE phi(int mode, int node_index) const { return mode == node_index ? FLOAT_TYPE(1) : FLOAT_TYPE(0); }
  FLOAT_TYPE d_phi(int mode, int node_index) const { return _D[mode * (_degree + 1) + node_index]; }
};
