// Serial stand-in for oneTBB parallel_sort, used only to compile the
// reference's k-mer counting sources for the oracle build (test
// infrastructure).  Ordering results are identical: std::sort with the same
// comparator.
#ifndef PK_REF_TBB_PARALLEL_SORT_H
#define PK_REF_TBB_PARALLEL_SORT_H
#include <algorithm>
#include <functional>
#include <iterator>
namespace oneapi { namespace tbb {
template <typename It>
void parallel_sort(It b, It e) { std::sort(b, e); }
template <typename It, typename Cmp>
void parallel_sort(It b, It e, const Cmp& c) { std::sort(b, e, c); }
template <typename Range, typename Cmp>
void parallel_sort(Range& r, const Cmp& c) { std::sort(std::begin(r), std::end(r), c); }
}}  // namespace oneapi::tbb
#endif
