// Serial stand-in for oneTBB concurrent_unordered_map (oracle build only).
#ifndef PK_REF_TBB_CONCURRENT_UNORDERED_MAP_H
#define PK_REF_TBB_CONCURRENT_UNORDERED_MAP_H
#include <unordered_map>
namespace oneapi { namespace tbb {
template <typename K, typename V, typename H = std::hash<K>>
using concurrent_unordered_map = std::unordered_map<K, V, H>;
}}  // namespace oneapi::tbb
#endif
