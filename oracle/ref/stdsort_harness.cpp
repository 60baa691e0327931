// libstdc++'s std::sort on (visit, count) pairs ranked the way MacroNode::setup_wiring
// ranks them (Comp_rev, includes/distribute_kmers.h:495-506), for pinning the oracle's
// restatement of that sort (TEST INFRASTRUCTURE ONLY).
//
// stdin : lines "n v0 c0 v1 c1 ..." ; stdout : the sorted index permutation per line
#include <stdio.h>

#include <algorithm>
#include <numeric>
#include <utility>
#include <vector>

int main() {
  int n;
  while (scanf("%d", &n) == 1) {
    std::vector<std::pair<int, int>> v(n);
    for (int i = 0; i < n; i++) scanf("%d %d", &v[i].second, &v[i].first);
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int i, int j) {
      return v[i].second > v[j].second || (v[i].second == v[j].second && v[i].first > v[j].first);
    });
    for (int i = 0; i < n; i++) printf("%d%c", idx[i], i + 1 < n ? ' ' : '\n');
    if (n == 0) printf("\n");
  }
  return 0;
}
