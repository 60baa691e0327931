// Serial stand-in for oneTBB concurrent_vector (oracle build only).
#ifndef PK_REF_TBB_CONCURRENT_VECTOR_H
#define PK_REF_TBB_CONCURRENT_VECTOR_H
#include <vector>
namespace oneapi { namespace tbb {
template <typename T>
class concurrent_vector : public std::vector<T> {
 public:
  using std::vector<T>::vector;
  typename std::vector<T>::iterator grow_by(size_t n) {
    size_t old = this->size();
    this->resize(old + n);
    return this->begin() + old;
  }
};
}}  // namespace oneapi::tbb
#endif
