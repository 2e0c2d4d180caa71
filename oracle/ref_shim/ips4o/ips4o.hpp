// ips4o/ips4o.hpp -- the two sort calls KaMSTa takes from IPS4o (submodule
// external/ips4o, pin unknown, empty here), for the oracle's reference
// build.  Only the order of the result matters to the reference, so the
// standard library's (parallel-mode) comparison sorts stand in.
#pragma once
#include <algorithm>
#include <parallel/algorithm>

namespace ips4o {
template <typename It, typename Less>
inline void sort(It begin, It end, Less less) {
  std::sort(begin, end, less);
}
template <typename It>
inline void sort(It begin, It end) {
  std::sort(begin, end);
}
namespace parallel {
template <typename It, typename Less>
inline void sort(It begin, It end, Less less) {
  __gnu_parallel::sort(begin, end, less);
}
template <typename It>
inline void sort(It begin, It end) {
  __gnu_parallel::sort(begin, end);
}
}  // namespace parallel
}  // namespace ips4o
