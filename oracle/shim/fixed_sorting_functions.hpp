// Oracle build shim (test infrastructure only).
//
// The reference's network_flow/fixed_sorting_functions.hpp is generated by
// network_flow/make_sorting_functions.py and is absent from the checkout.  This
// header supplies fixed_sorter<T, n> as the same published algorithm the
// generator emits: the bitonic sorter for arbitrary n (recursive split
// m = n/2 sorted down then up, merged with a compare distance equal to the
// largest power of two below n), applied as a fixed sequence of
// compare-exchange steps.  PossibleNeighbor compares heights only
// (network_flow/pr_auxilary_structures.hpp:13-15), so ties keep the order this
// network produces, exactly as in the generated header.
#ifndef LF_ORACLE_FIXED_SORTING_SHIM_HPP
#define LF_ORACLE_FIXED_SORTING_SHIM_HPP
#include <algorithm>
#include <utility>
#include <vector>
#include "common.hpp"

namespace latticeQBP {

namespace lf_oracle_detail {
struct CmpEx { int lo, hi; };

inline int largest_pow2_below(int n) {
  int k = 1;
  while (k < n) k *= 2;
  return k / 2;
}

inline void merge_steps(std::vector<CmpEx>& out, int start, int n, bool up) {
  if (n <= 1) return;
  int m = largest_pow2_below(n);
  for (int i = start; i < start + n - m; ++i)
    out.push_back(up ? CmpEx{i, i + m} : CmpEx{i + m, i});
  merge_steps(out, start, m, up);
  merge_steps(out, start + m, n - m, up);
}

inline void sort_steps(std::vector<CmpEx>& out, int start, int n, bool up) {
  if (n <= 1) return;
  int m = n / 2;
  sort_steps(out, start, m, !up);
  sort_steps(out, start + m, n - m, up);
  merge_steps(out, start, n, up);
}

inline const std::vector<CmpEx>& network(int n) {
  static std::vector<std::vector<CmpEx> > cache(129);
  static std::vector<bool> built(129, false);
  if (!built[n]) { sort_steps(cache[n], 0, n, true); built[n] = true; }
  return cache[n];
}
}  // namespace lf_oracle_detail

template <typename dtype, int n>
struct fixed_sorter {
  template <typename It>
  static inline void sort(It start, It end) {
    if (n >= 128) { std::sort(start, end); return; }
    const auto& net = lf_oracle_detail::network(n);
    for (const auto& c : net) {
      auto& a = *(start + c.lo);
      auto& b = *(start + c.hi);
      if (b < a) std::swap(a, b);
    }
  }
};

}  // namespace latticeQBP
#endif
