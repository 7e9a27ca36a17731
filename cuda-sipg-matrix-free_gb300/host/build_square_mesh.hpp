// build_square_mesh.hpp -- the uniform dim x dim quad mesh of the unit square
// with the reference's interface (build_square_mesh.hpp:39-202): element
// id = row*dim + col, row 0 at the top, corner coordinates x[c*noe+e] (c = 0..3
// counter-clockwise from the lower-left corner).  The fused kernels derive
// neighbours by index arithmetic, so `device_info` carries only the sizes and
// the neighbour rule of quadrilateral_mesh_info (mesh_info.hpp:278-309);
// its free() exists for source compatibility and releases nothing.
#pragma once

#include <cassert>
#include <vector>

#include "sipg_host_common.hpp"

template <typename FLOAT_TYPE>
struct quadrilateral_mesh_info {
  int dimx = 0, dimy = 0;
  int get_dimx() const { return dimx; }
  int get_dimy() const { return dimy; }
  int get_noe() const { return dimx * dimy; }
  int compute_idx(int x, int y) const { return dimx * y + x; }
  int get_neighborhood_DOWN(int x, int y) const { return dimy - 1 == y ? -1 : dimx * (y + 1) + x; }
  int get_neighborhood_RIGHT(int x, int y) const { return dimx - 1 == x ? -2 : dimx * y + x + 1; }
  int get_neighborhood_UP(int x, int y) const { return 0 == y ? -3 : dimx * (y - 1) + x; }
  int get_neighborhood_LEFT(int x, int y) const { return 0 == x ? -4 : dimx * y + x - 1; }
  void free() {}
};

template <typename FLOAT_TYPE>
class square_mesh {
  int _dim = 0, _noe = 0;
  std::vector<FLOAT_TYPE> _x_coord, _y_coord;

 public:
  quadrilateral_mesh_info<FLOAT_TYPE> device_info;

  square_mesh() {}
  explicit square_mesh(int dim) : _dim(dim), _noe(dim * dim) {
    std::vector<double> x(4 * (size_t)_noe), y(4 * (size_t)_noe);
    sipg_host::check(sipg_square_mesh_coords(dim, x.data(), y.data()), "sipg_square_mesh_coords");
    _x_coord.assign(x.begin(), x.end());
    _y_coord.assign(y.begin(), y.end());
    device_info.dimx = dim;
    device_info.dimy = dim;
  }
  int noe() const { return _noe; }
  int dim() const { return _dim; }
  const std::vector<FLOAT_TYPE>& x_coord() const { return _x_coord; }
  const std::vector<FLOAT_TYPE>& y_coord() const { return _y_coord; }
  const FLOAT_TYPE& get_x(int c, int element) const { return _x_coord[(size_t)c * _noe + element]; }
  const FLOAT_TYPE& get_y(int c, int element) const { return _y_coord[(size_t)c * _noe + element]; }
  // n = 0 DOWN, 1 RIGHT, 2 UP, 3 LEFT; negative ids mark the boundary
  int get_neighbor(int n, int element) const {
    const int x = element % _dim, y = element / _dim;
    switch (n) {
      case 0: return device_info.get_neighborhood_DOWN(x, y);
      case 1: return device_info.get_neighborhood_RIGHT(x, y);
      case 2: return device_info.get_neighborhood_UP(x, y);
      case 3: return device_info.get_neighborhood_LEFT(x, y);
    }
    assert(false);
    return 0;
  }
};
