// Host harness for the device's std::sort restatement (pakman_plus_gb300/csrc/
// pk_stdsort.cuh, compiled here as plain C++): the same input format and output as
// oracle/ref/stdsort_harness.cpp, so a test can compare both line by line.
//
// stdin : lines "n v0 c0 v1 c1 ..." (n <= 32) ; stdout : the sorted index permutation
#include <stdio.h>

#include <vector>

#include "../../pakman_plus_gb300/csrc/pk_stdsort.cuh"

int main() {
  int n;
  while (scanf("%d", &n) == 1) {
    std::vector<int32_t> vis(n), cnt(n);
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) {
      if (scanf("%d %d", &vis[i], &cnt[i]) != 2) return 1;
      idx[i] = i;
    }
    if (n > pk_sort::kSortMax) return 2;
    pk_sort::std_sort(idx.data(), n, pk_sort::RankLess{vis.data(), cnt.data()});
    for (int i = 0; i < n; i++) printf("%d%c", idx[i], i + 1 < n ? ' ' : '\n');
    if (n == 0) printf("\n");
  }
  return 0;
}
