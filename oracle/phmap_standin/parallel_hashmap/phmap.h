// Project-written stand-in for the parallel-hashmap header, which the reference includes from an
// empty git submodule.  The reference's hot-path sources only need the include to resolve; the
// two aliases cover the kron builders should a harness ever compile them.  Test infrastructure
// for oracle/_ref only.
#pragma once
#include <unordered_map>
#include <unordered_set>

namespace phmap {
template <class K, class V, class H = std::hash<K>, class E = std::equal_to<K>>
using flat_hash_map = std::unordered_map<K, V, H, E>;
template <class K, class H = std::hash<K>, class E = std::equal_to<K>>
using flat_hash_set = std::unordered_set<K, H, E>;
}  // namespace phmap
