// Drives the link-level drop-in (pakman_plus_gb300/host/pakman_dropin.cpp) in the order
// the reference's driver calls it (src/distribute_kmers.cpp:147-203: counting, macro-node
// construction, initial wiring, iterative compaction, begin k-mers), built against the
// stand-in header in dropin_standin/, and writes what the adapter leaves in the
// reference's data structures to files that tests/test_gpu_dropin.py compares with the
// golden fixtures and with the C ABI's own results.
//
//   dropin_check <fasta> <coverage> <t> <node_threshold> <outdir>
//
//   table.bin      kmer_proc_buf after perform_kmer_counting (packed KmerPairs)
//   mn_built.txt   MN_map after begin_mnode_construction
//   mn_wired.txt   MN_map after initiate_mnode_wiring
//   mn_compact.txt MN_map after begin_iterative_compaction
//   partial.txt    partial_contig_list, one contig of base codes per line
//   begins.txt     identify_begin_kmers: node key and terminal prefix index per line
// A node line: key (hi and lo words in hex), the k_1_mer bases, then every suffix and
// prefix entry as bases:count:visit:terminal, the wiring_info triples and the
// prefix_begin_info pairs.
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <utility>
#include <vector>

#include "distribute_kmers.h"

std::vector<KmerPairs> kmer_proc_buf;
int rank = 0, size = 1;
int coverage = 0, num_buckets = 0, read_length = 100, node_threashold = 0;
size_t MAX_KMER_COUNT = 100000000;

void perform_kmer_counting(const char* read_data, size_t length);
void begin_mnode_construction(std::vector<std::pair<kmer_t, MacroNode>>& MN_map);
void initiate_mnode_wiring(std::vector<std::pair<kmer_t, MacroNode>>& MN_map);
size_t begin_iterative_compaction(std::vector<std::pair<kmer_t, MacroNode>>& MN_map,
                                  std::vector<BasePairVector>& partial_contig_list);
void identify_begin_kmers(std::vector<std::pair<kmer_t, MacroNode>>& MN_map,
                          std::vector<BeginMN>& list_of_begin_kmers);

namespace {

std::string bases(const BasePairVector& v) {
  std::string s;
  for (size_t i = 0; i < v.size(); i++) s.push_back((char)('0' + v[i]));
  return s;
}

void put_key(FILE* f, kmer_t k) {
  fprintf(f, "%016llx:%016llx", (unsigned long long)(k >> 32 >> 32), (unsigned long long)(uint64_t)k);
}

void entries(FILE* f, char tag, const std::vector<BasePairVector>& ext, const std::vector<bool>& term,
             const std::vector<std::pair<int, int>>& cnt) {
  fprintf(f, " %c", tag);
  for (size_t e = 0; e < ext.size(); e++)
    fprintf(f, " %s:%d:%d:%d", bases(ext[e]).c_str(), cnt[e].first, cnt[e].second, (int)term[e]);
}

void dump(const std::string& path, const std::vector<std::pair<kmer_t, MacroNode>>& map) {
  FILE* f = fopen(path.c_str(), "w");
  if (!f) { perror(path.c_str()); exit(2); }
  for (const auto& kv : map) {
    const MacroNode& mn = kv.second;
    put_key(f, kv.first);
    fprintf(f, " %s", bases(mn.k_1_mer).c_str());
    entries(f, 'S', mn.suffixes, mn.suffixes_terminal, mn.suffix_count);
    entries(f, 'P', mn.prefixes, mn.prefixes_terminal, mn.prefix_count);
    fprintf(f, " W");
    for (const WireInfo& w : mn.wiring_info) fprintf(f, " %d,%d,%d", w.suffix_id, w.offset_in_suffix, w.count);
    fprintf(f, " B");
    for (const PrefixInfo& p : mn.prefix_begin_info) fprintf(f, " %d,%d", p.prefix_pos, p.num_wires);
    fprintf(f, "\n");
  }
  fclose(f);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: %s <fasta> <coverage> <t> <node_threshold> <outdir>\n", argv[0]);
    return 2;
  }
  coverage = atoi(argv[2]);
  num_buckets = atoi(argv[3]);
  node_threashold = atoi(argv[4]);
  const std::string out = argv[5];
  FILE* in = fopen(argv[1], "rb");
  if (!in) { perror(argv[1]); return 2; }
  std::vector<char> data;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), in)) > 0) data.insert(data.end(), buf, buf + n);
  fclose(in);

  perform_kmer_counting(data.data(), data.size());
  FILE* t = fopen((out + "/table.bin").c_str(), "wb");
  if (!kmer_proc_buf.empty()) fwrite(kmer_proc_buf.data(), sizeof(KmerPairs), kmer_proc_buf.size(), t);
  fclose(t);

  std::vector<std::pair<kmer_t, MacroNode>> MN_map;
  begin_mnode_construction(MN_map);
  if (!kmer_proc_buf.empty()) { fprintf(stderr, "kmer_proc_buf was not freed\n"); return 3; }
  dump(out + "/mn_built.txt", MN_map);
  initiate_mnode_wiring(MN_map);
  dump(out + "/mn_wired.txt", MN_map);
  std::vector<BasePairVector> partial;
  begin_iterative_compaction(MN_map, partial);
  dump(out + "/mn_compact.txt", MN_map);
  FILE* p = fopen((out + "/partial.txt").c_str(), "w");
  for (const BasePairVector& c : partial) fprintf(p, "%s\n", bases(c).c_str());
  fclose(p);
  std::vector<BeginMN> begins;
  identify_begin_kmers(MN_map, begins);
  FILE* b = fopen((out + "/begins.txt").c_str(), "w");
  for (const BeginMN& x : begins) {
    put_key(b, x.node);
    fprintf(b, " %d\n", x.terminal_prefix_id);
  }
  fclose(b);
  return 0;
}
