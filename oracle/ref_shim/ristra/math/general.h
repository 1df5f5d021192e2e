// Stand-in for libristra's general math header.
#pragma once
#include <cmath>
#include "array.h"
#include "tuple.h"
namespace ristra {
namespace math {
using std::abs;
}  // namespace math
namespace utils {
template <typename T>
struct reference_wrapper_t;
}  // namespace utils
}  // namespace ristra
