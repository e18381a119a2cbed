// Stand-in for oneTBB (test infrastructure for oracle/_ref): a std::vector.
#pragma once
#include <vector>

namespace tbb {
template <typename T>
class concurrent_vector : public std::vector<T> {
public:
    using std::vector<T>::vector;
};
}
