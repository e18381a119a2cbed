// Stand-in for robin_hood hashing (test infrastructure for oracle/_ref). On the Transform-DAG path
// the reference uses these maps for lookups, so std::unordered_map gives the same results.
// One loop (find_translation.cpp:910-914) erases through an iterator and then increments that same
// iterator, which a flat robin_hood table tolerates and a node-based map does not. Those erasures
// only drop hash keys whose candidate range has become empty, and a lookup that finds an empty
// range yields no candidates, just as a lookup that finds nothing. So erase-by-iterator keeps the
// entry here, which leaves every result unchanged.
#pragma once
#include <functional>
#include <unordered_map>
#include <unordered_set>

namespace robin_hood {
template <typename T>
using hash = std::hash<T>;
template <typename K, typename V, typename H = std::hash<K>, typename E = std::equal_to<K>>
class unordered_flat_map : public std::unordered_map<K, V, H, E> {
public:
    using std::unordered_map<K, V, H, E>::unordered_map;
    void compact() { this->rehash(0); }
    template <typename It>
    void erase(It) { }
};
template <typename K, typename V, typename H = std::hash<K>, typename E = std::equal_to<K>>
using unordered_node_map = unordered_flat_map<K, V, H, E>;
template <typename K, typename V, typename H = std::hash<K>, typename E = std::equal_to<K>>
using unordered_map = unordered_flat_map<K, V, H, E>;
template <typename K, typename H = std::hash<K>, typename E = std::equal_to<K>>
using unordered_flat_set = std::unordered_set<K, H, E>;
template <typename K, typename H = std::hash<K>, typename E = std::equal_to<K>>
using unordered_set = std::unordered_set<K, H, E>;
}
