// LGL_quadrature_table.hpp -- Legendre-Gauss-Lobatto nodes and weights on
// [-1, 1] with the reference's interface (LGL_quadrature_table.hpp:16-66),
// computed by the library (sipg_lgl_table, up to 64 points).
#pragma once

#include <vector>

#include "sipg_host_common.hpp"

template <typename FLOAT_TYPE>
class LGL_quadrature_table {
  std::vector<FLOAT_TYPE> _nodes, _weights;
  int _number_of_points;

 public:
  explicit LGL_quadrature_table(int number_of_points) : _number_of_points(number_of_points) {
    std::vector<double> x(number_of_points), w(number_of_points);
    sipg_host::check(sipg_lgl_table(number_of_points, x.data(), w.data()), "sipg_lgl_table");
    _nodes.assign(x.begin(), x.end());
    _weights.assign(w.begin(), w.end());
  }
  int nop() const { return _number_of_points; }
  const FLOAT_TYPE& node(int i) const { return _nodes[i]; }
  const FLOAT_TYPE& weight(int i) const { return _weights[i]; }
  const FLOAT_TYPE* nodes_array() const { return _nodes.data(); }
  const FLOAT_TYPE* weights_array() const { return _weights.data(); }
};
