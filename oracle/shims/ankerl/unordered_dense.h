// Stand-in for ankerl::unordered_dense (v4.5.0), which Spira fetches at build
// time and which is not present offline. Spira uses it only as a hash map
// container; std::unordered_map gives the same results (iteration order only
// permutes inserts that lock() sorts again).
#pragma once
#include <unordered_map>
namespace ankerl::unordered_dense {
template <class K, class V> using map = std::unordered_map<K, V>;
}
