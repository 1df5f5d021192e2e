// Minimal stand-in for libristra's ristra::math::array (the reference's
// ristra submodule is empty).  Only what flecsale/eqns/euler_eqns.h and
// flecsale/eqns/flux.h use: indexing, constexpr size(), element-wise + and -,
// scalar *, and the in-place scalar ops.  Test infrastructure only.
#pragma once
#include <cstddef>

namespace ristra {
namespace math {

template <typename T, std::size_t N>
struct array {
  T data_[N];
  array() = default;
  array(T v) { for (std::size_t i = 0; i < N; ++i) data_[i] = v; }
  T &operator[](std::size_t i) { return data_[i]; }
  const T &operator[](std::size_t i) const { return data_[i]; }
  static constexpr std::size_t size() { return N; }
};

template <typename T, std::size_t N>
array<T, N> operator+(const array<T, N> &a, const array<T, N> &b) {
  array<T, N> r;
  for (std::size_t i = 0; i < N; ++i) r[i] = a[i] + b[i];
  return r;
}

template <typename T, std::size_t N>
array<T, N> operator-(const array<T, N> &a, const array<T, N> &b) {
  array<T, N> r;
  for (std::size_t i = 0; i < N; ++i) r[i] = a[i] - b[i];
  return r;
}

template <typename S, typename T, std::size_t N>
array<T, N> operator*(const S &s, const array<T, N> &a) {
  array<T, N> r;
  for (std::size_t i = 0; i < N; ++i) r[i] = s * a[i];
  return r;
}

// sum from zero in index order
template <typename T, std::size_t N>
T dot_product(const array<T, N> &a, const array<T, N> &b) {
  T s(0);
  for (std::size_t i = 0; i < N; ++i) s += a[i] * b[i];
  return s;
}

template <typename T, std::size_t N, typename S>
void divides_equal(array<T, N> &a, const S &s) {
  for (std::size_t i = 0; i < N; ++i) a[i] /= s;
}

template <typename T, std::size_t N, typename S>
void multiplies_equal(array<T, N> &a, const S &s) {
  for (std::size_t i = 0; i < N; ++i) a[i] *= s;
}

}  // namespace math
}  // namespace ristra
