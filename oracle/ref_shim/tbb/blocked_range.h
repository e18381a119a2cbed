// Stand-in for oneTBB (test infrastructure for oracle/_ref): the reference's TBB loops run serially.
#pragma once
#include <cstddef>

namespace tbb {
template <typename T>
class blocked_range {
public:
    blocked_range(T b, T e, size_t = 1) : m_b(b), m_e(e) {}
    T begin() const { return m_b; }
    T end() const { return m_e; }
    size_t size() const { return size_t(m_e - m_b); }
    bool empty() const { return !(m_b < m_e); }
private:
    T m_b, m_e;
};
}
