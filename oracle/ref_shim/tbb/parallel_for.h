// Stand-in for oneTBB (test infrastructure for oracle/_ref): serial loops.
#pragma once
#include <tbb/blocked_range.h>

namespace tbb {
template <typename Range, typename Body>
inline void parallel_for(const Range& range, const Body& body) { body(range); }
template <typename Index, typename Body>
inline void parallel_for(Index first, Index last, const Body& body)
{
    for (Index i = first; i < last; ++i)
        body(i);
}
}
