// Stand-in for libristra's tuple header: std::tuple and std::get.
#pragma once
#include <tuple>
namespace ristra {
namespace math {
using std::get;
template <typename... Ts>
using tuple = std::tuple<Ts...>;
}  // namespace math
}  // namespace ristra
