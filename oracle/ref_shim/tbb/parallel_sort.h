// Stand-in for oneTBB (test infrastructure for oracle/_ref): std::sort.
#pragma once
#include <algorithm>
#include <functional>

namespace tbb {
template <typename It, typename Cmp>
inline void parallel_sort(It b, It e, const Cmp& c) { std::sort(b, e, c); }
template <typename It>
inline void parallel_sort(It b, It e) { std::sort(b, e); }
}
