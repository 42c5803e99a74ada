/* Test infrastructure: the part of boost::multi_array<T, 3> that the reference's
 * include/mesh_builder.h uses (construction from boost::extents[a][b][c], shape(),
 * element access grid[i][j][k]), written for this project so that header compiles for
 * the host without Boost.  Element access is bounds-checked and aborts: the oracle's
 * golden inputs never leave the grid. */
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace boost {

template <std::size_t D>
struct extent_list {
  std::size_t n[D];
  extent_list<D + 1> operator[](std::size_t k) const {
    extent_list<D + 1> e;
    for (std::size_t c = 0; c < D; ++c) e.n[c] = n[c];
    e.n[D] = k;
    return e;
  }
};

struct extent_root {
  extent_list<1> operator[](std::size_t k) const { return extent_list<1>{{k}}; }
};
static const extent_root extents{};

template <class T, std::size_t D>
class multi_array;

template <class T>
class multi_array<T, 3> {
  std::vector<T> data_;
  std::size_t shape_[3];

  static std::size_t checked(std::size_t i, std::size_t n) {
    if (i >= n) {
      std::fprintf(stderr, "multi_array index %zu outside extent %zu\n", i, n);
      std::abort();
    }
    return i;
  }

 public:
  struct Row {
    T* p;
    std::size_t n;
    T& operator[](std::size_t k) const { return p[checked(k, n)]; }
  };
  struct Plane {
    T* p;
    std::size_t n1, n2;
    Row operator[](std::size_t j) const { return Row{p + checked(j, n1) * n2, n2}; }
  };
  explicit multi_array(const extent_list<3>& e) : data_(e.n[0] * e.n[1] * e.n[2]) {
    for (int c = 0; c < 3; ++c) shape_[c] = e.n[c];
  }
  const std::size_t* shape() const { return shape_; }
  Plane operator[](std::size_t i) { return Plane{data_.data() + checked(i, shape_[0]) * shape_[1] * shape_[2], shape_[1], shape_[2]}; }
  T* data() { return data_.data(); }
};

}  // namespace boost
