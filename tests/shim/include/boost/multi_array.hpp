// Test stand-in for the part of boost::multi_array that the reference-side
// shim uses: two-dimensional arrays resized with boost::extents[a][b] and
// indexed a[i][j].  Boost itself is not available here.
#pragma once
#include <cstddef>
#include <vector>

namespace boost {
struct Extents2 {
  size_t a, b;
};
struct Extents1 {
  size_t a;
  Extents2 operator[](size_t b) const { return {a, b}; }
};
struct ExtentGen {
  Extents1 operator[](size_t a) const { return {a}; }
};
static ExtentGen const extents{};

template <typename T, size_t N>
class multi_array;

template <typename T>
class multi_array<T, 2> {
 public:
  void resize(Extents2 e) {
    a_ = e.a;
    b_ = e.b;
    v_.assign(a_ * b_, T());
  }
  T *operator[](size_t i) { return v_.data() + i * b_; }
  T const *operator[](size_t i) const { return v_.data() + i * b_; }
  size_t num_elements() const { return v_.size(); }

 private:
  size_t a_ = 0, b_ = 0;
  std::vector<T> v_;
};
}  // namespace boost
