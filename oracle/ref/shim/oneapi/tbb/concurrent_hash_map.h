// Serial stand-in for oneTBB concurrent_hash_map (oracle build only).  Only
// the accessor/insert/iterate/clear surface used by the reference compiles.
#ifndef PK_REF_TBB_CONCURRENT_HASH_MAP_H
#define PK_REF_TBB_CONCURRENT_HASH_MAP_H
#include <unordered_map>
#include <utility>
namespace oneapi { namespace tbb {
template <typename K, typename V>
class concurrent_hash_map : public std::unordered_map<K, V> {
 public:
  explicit concurrent_hash_map(size_t n = 0) { this->reserve(n); }
  class accessor {
   public:
    std::pair<const K, V>* p = nullptr;
    std::pair<const K, V>* operator->() const { return p; }
    std::pair<const K, V>& operator*() const { return *p; }
    void release() { p = nullptr; }
  };
  bool insert(accessor& a, const K& k) {
    auto r = this->emplace(k, V());
    a.p = &*r.first;
    return r.second;
  }
};
}}  // namespace oneapi::tbb
#endif
