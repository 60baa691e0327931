// libstdc++'s std::sort restated for the ranking inside MacroNode::setup_wiring, shared
// by the compaction kernels (pk_compact.cu) and a host harness that pins it against
// libstdc++ itself.  Plain integer code, callable on the host and the device.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define PK_HD __host__ __device__
#else
#define PK_HD
#endif

namespace pk_sort {

constexpr int kSortMax = 32;  // the lists the device ranks hold at most this many entries

PK_HD inline int floor_log2(int n) {
  int lg = 0;
  while ((1 << (lg + 1)) <= n) lg++;
  return lg;
}

// -------------------------------------------------------------- std::sort ---------
// libstdc++'s std::sort (introsort: 16-element threshold, median-of-three pivot,
// unguarded partition, heap sort past depth 2*floor(log2 n); final insertion sort)
// on n <= kSortMax indices.  The wiring ranks list entries with it and equal entries
// land where it leaves them, so the device follows the same steps.
struct RankLess {
  const int32_t* vis;
  const int32_t* cnt;
  PK_HD bool operator()(int i, int j) const {
    return vis[i] > vis[j] || (vis[i] == vis[j] && cnt[i] > cnt[j]);
  }
};

PK_HD inline void heap_adjust(int* a, int hole, int len, int value, const RankLess& less) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (less(a[child], a[child - 1])) child--;
    a[hole] = a[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    a[hole] = a[child - 1];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top && less(a[parent], value)) {
    a[hole] = a[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  a[hole] = value;
}

PK_HD inline void heap_sort(int* a, int len, const RankLess& less) {
  if (len >= 2) {
    for (int parent = (len - 2) / 2;; parent--) {
      heap_adjust(a, parent, len, a[parent], less);
      if (parent == 0) break;
    }
  }
  for (int last = len; last > 1;) {
    last--;
    const int v = a[last];
    a[last] = a[0];
    heap_adjust(a, 0, last, v, less);
  }
}

PK_HD inline void swp(int* a, int i, int j) {
  const int t = a[i];
  a[i] = a[j];
  a[j] = t;
}

PK_HD inline void std_sort(int* a, int n, const RankLess& less) {
  if (n < 2) return;
  struct Frame {
    int8_t first, last, depth;
  };
  Frame st[kSortMax];
  int sp = 0;
  st[sp++] = Frame{0, (int8_t)n, (int8_t)(2 * floor_log2(n))};
  while (sp) {
    Frame f = st[--sp];
    int first = f.first, last = f.last, depth = f.depth;
    while (last - first > 16) {
      if (depth == 0) {
        heap_sort(a + first, last - first, less);
        break;
      }
      depth--;
      const int mid = first + (last - first) / 2, x = first + 1, y = mid, z = last - 1;
      if (less(a[x], a[y])) {
        if (less(a[y], a[z])) swp(a, first, y);
        else if (less(a[x], a[z])) swp(a, first, z);
        else swp(a, first, x);
      } else if (less(a[x], a[z])) {
        swp(a, first, x);
      } else if (less(a[y], a[z])) {
        swp(a, first, z);
      } else {
        swp(a, first, y);
      }
      int lo = first + 1, hi = last;
      while (true) {
        while (less(a[lo], a[first])) lo++;
        hi--;
        while (less(a[first], a[hi])) hi--;
        if (!(lo < hi)) break;
        swp(a, lo, hi);
        lo++;
      }
      st[sp++] = Frame{(int8_t)lo, (int8_t)last, (int8_t)depth};
      last = lo;
    }
  }
  const int lim = n > 16 ? 16 : n;
  for (int i = 1; i < lim; i++) {  // insertion sort of the first min(n, 16)
    const int v = a[i];
    if (less(v, a[0])) {
      for (int j = i; j > 0; j--) a[j] = a[j - 1];
      a[0] = v;
    } else {
      int j = i - 1;
      while (less(v, a[j])) {
        a[j + 1] = a[j];
        j--;
      }
      a[j + 1] = v;
    }
  }
  for (int i = 16; i < n; i++) {  // unguarded insertion of the rest
    const int v = a[i];
    int j = i - 1;
    while (less(v, a[j])) {
      a[j + 1] = a[j];
      j--;
    }
    a[j + 1] = v;
  }
}

}  // namespace pk_sort
