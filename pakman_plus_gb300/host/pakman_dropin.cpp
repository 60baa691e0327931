// Link-level drop-in for the reference's counting, histogram and macro-node phases.
//
// Compile this file inside the PaKman tree (it includes the reference's own
// includes/distribute_kmers.h for kmer_t, KmerPairs, MacroNode and BasePairVector)
// and link it with libpakman_gb300.so *instead of* src/kmer_counting.cpp,
// src/kmer_histogram.cpp and src/mn_construct.cpp.  It defines the three functions the
// reference driver calls (src/distribute_kmers.cpp:147, :168):
//
//   perform_kmer_counting(const char*, size_t)          src/kmer_counting.cpp:3351
//   begin_mnode_construction(vector<pair<kmer_t,MacroNode>>&)  src/mn_construct.cpp:479
//   free_kmer_count_buffers()                            src/kmer_counting.cpp:3343
//
// with the same contracts: kmer_proc_buf receives the sorted unique (k-mer, count)
// table; begin_mnode_construction prints the reference's summary lines, aborts when
// nothing reaches the cutoff, and fills MN_map sorted by (k-1)-mer with suffixes and
// prefixes in ascending extension order and (count, ceil(count/coverage)) pairs.
//
// For the reference's contig-generation build (PERFORM_CONTIG_GENERATION,
// COMPACT_PGRAGH; src/distribute_kmers.cpp:156-203) it also replaces
// src/wire.cpp, src/iterative_compaction.cpp and src/merge_mn.cpp:
//
//   initiate_mnode_wiring(MN_map)                         src/wire.cpp:66-121
//   begin_iterative_compaction(MN_map, partial_contig_list)  src/iterative_compaction.cpp:131-464
//   identify_begin_kmers(MN_map, list_of_begin_kmers)     src/iterative_compaction.cpp:65-93
//   generate_compacted_pakgraph(MN_map, global_MN_map)    src/iterative_compaction.cpp:96-128
//
// The wiring and the compaction run on the device.  MN_map is refilled from the
// device after each call, and the reference's own walk (src/walk.cpp, linked
// unchanged) traverses it.  With one rank the gather is a copy.
// One MPI rank drives one GPU; the device counts the rank's whole buffer at once, so
// the -b batch size changes nothing (the reference's table is the same for any -b).
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <utility>
#include <vector>

#include "distribute_kmers.h"
#include "pakman_gb300.h"

extern std::vector<KmerPairs> kmer_proc_buf;
extern int coverage;
extern int num_buckets;
extern int read_length;
extern size_t MAX_KMER_COUNT;

namespace {

pk_ctx* g_ctx = nullptr;
pk_job* g_job = nullptr;

void die(pk_status s, const char* where) {
  fprintf(stderr, "[pakman-gb300] %s: %s (%s)\n", where, pk_status_string(s), pk_last_error());
  MPI_Abort(MPI_COMM_WORLD, -99);
}

void ensure_job() {
  if (g_job) return;
  pk_status s = pk_ctx_create(0, 0, &g_ctx);
  if (s != PK_OK) die(s, "pk_ctx_create");
  s = pk_job_create(g_ctx, nullptr, &g_job);
  if (s != PK_OK) die(s, "pk_job_create");
}

pk_params params() {
  pk_params p;
  pk_params_default(&p);
  p.k = KMER_LENGTH;
  p.lmer_length = LMER_LENGTH;
  p.num_buckets = num_buckets ? num_buckets : 21;
  p.coverage = coverage ? coverage : 1;
  p.read_length = read_length;
  p.batch_kmers = MAX_KMER_COUNT;
  return p;
}

int visit(int count) {  // (int)ceil((double)count / coverage), src/mn_construct.cpp:75-79
  int q = count / coverage, r = count % coverage;
  if (r != 0 && ((r > 0) == (coverage > 0))) q++;
  return q;
}

kmer_t key_at(const std::vector<uint64_t>& words, size_t i) {
#ifdef EXTEND_KMER
  return ((kmer_t)words[2 * i + 1] << 64) | (kmer_t)words[2 * i];
#else
  return (kmer_t)words[i];
#endif
}

}  // namespace

void perform_kmer_counting(const char* read_data, size_t length) {
  ensure_job();
  pk_params p = params();
  pk_status s = pk_count(g_job, read_data, length, &p);
  if (s == PK_ERR_FORMAT) {
    fprintf(stderr, "[pakman-gb300] a FASTA record does not start with '>'\n");
    abort();  // the reference's assert(ptr[p]=='>')
  }
  if (s != PK_OK) die(s, "pk_count");
  uint64_t u = 0, windows = 0, reads = 0;
  s = pk_table_info(g_job, &u, &windows, &reads);
  if (s != PK_OK) die(s, "pk_table_info");
  kmer_proc_buf.resize(u);
  // KmerPairs is packed {kmer_t seq; int k_count;}: the device writes that exact layout
  s = pk_copy_table_packed(g_job, kmer_proc_buf.data(), u);
  if (s != PK_OK) die(s, "pk_copy_table_packed");
  if (rank == 0) {
    printf("Total distinct k-mer entries across all proc's: %lu\n", (unsigned long)u);
    printf("Number of batch iterations: %d \n", 1);
  }
}

void free_kmer_count_buffers() {
  kmer_proc_buf.clear();
  kmer_proc_buf.shrink_to_fit();
}

void begin_mnode_construction(std::vector<std::pair<kmer_t, MacroNode>>& MN_map) {
  ensure_job();
  uint32_t cutoff = 0;
  uint64_t kept = 0;
  pk_status s = pk_cutoff(g_job, num_buckets, &cutoff, nullptr, &kept);
  if (rank == 0) {
    printf("Number of threads: %d\n", 1);
    printf("Total valid (>= min_bucket(%d)) k-mer entries across all proc's: %lu \n", (int)cutoff,
           (unsigned long)kept);
  }
  free_kmer_count_buffers();  // the reference frees the table here (src/kmer_histogram.cpp:186)
  if (s == PK_ERR_EMPTY) {
    std::cerr << "Number of k-mers post pruning based on frequency cuttoff at: " << cutoff
              << " are null. Contig generation cannot proceed." << std::endl;
    MPI_Abort(MPI_COMM_WORLD, -99);
  }
  if (s != PK_OK) die(s, "pk_cutoff");
  uint64_t m = 0;
  s = pk_build_macro_nodes(g_job, 0, &m);
  if (s != PK_OK) die(s, "pk_build_macro_nodes");
  const size_t words = sizeof(kmer_t) / 8;
  std::vector<uint64_t> keys(m * words);
  std::vector<uint32_t> suf(4 * m), pre(4 * m);
  s = pk_copy_macro_nodes(g_job, keys.data(), suf.data(), pre.data(), m);
  if (s != PK_OK) die(s, "pk_copy_macro_nodes");
  MN_map.clear();
  MN_map.reserve(m);
  for (size_t i = 0; i < m; i++) {
    const kmer_t key = key_at(keys, i);
    MacroNode mn;
    for (int b = 0; b < MN_LENGTH; b++) mn.k_1_mer.push_back(kmerel_mn(key, b));
    for (int e = 0; e < 4; e++) {
      const int c = (int)suf[4 * i + e];
      if (!c) continue;
      BasePairVector ext;
      ext.push_back((BasePair)e);
      mn.suffixes.push_back(ext);
      mn.suffixes_terminal.push_back(false);
      mn.suffix_count.push_back(std::make_pair(c, visit(c)));
    }
    for (int e = 0; e < 4; e++) {
      const int c = (int)pre[4 * i + e];
      if (!c) continue;
      BasePairVector ext;
      ext.push_back((BasePair)e);
      mn.prefixes.push_back(ext);
      mn.prefixes_terminal.push_back(false);
      mn.prefix_count.push_back(std::make_pair(c, visit(c)));
    }
    MN_map.push_back(std::make_pair(key, mn));
  }
  if (rank == 0) printf("Total number of macro_nodes across all proc's: %lu\n", (unsigned long)m);
}

// ---- contig generation ---------------------------------------------------------
extern int node_threashold;

namespace {

void put_ext(BasePairVector& v, const uint8_t* b, uint32_t n) {
  for (uint32_t i = 0; i < n; i++) v.push_back((BasePair)b[i]);
}

}  // namespace

void initiate_mnode_wiring(std::vector<std::pair<kmer_t, MacroNode>>& MN_map) {
  ensure_job();
  pk_status s = pk_wire_macro_nodes(g_job, coverage);
  if (s != PK_OK) die(s, "pk_wire_macro_nodes");
  std::vector<pk_wiring> w(MN_map.size() + 1);
  s = pk_copy_wiring(g_job, w.data(), MN_map.size());
  if (s != PK_OK) die(s, "pk_copy_wiring");
  for (size_t i = 0; i < MN_map.size(); i++) {
    MacroNode& mn = MN_map[i].second;
    const pk_wiring& r = w[i];
    mn.prefixes.push_back(BasePairVector{});
    mn.prefixes_terminal.push_back(true);
    mn.prefix_count.push_back(std::make_pair(1, r.terminal_prefix_visit));
    mn.suffixes.push_back(BasePairVector{});
    mn.suffixes_terminal.push_back(true);
    mn.suffix_count.push_back(std::make_pair(1, r.terminal_suffix_visit));
    const int nw = (int)(mn.prefixes.size() + mn.suffixes.size() + 1);
    // a node has at most four prefixes and four suffixes plus the terminal entries, which
    // is what pk_wiring holds; anything else means the map and the wiring disagree
    const int max_wires = (int)(sizeof(r.wire) / sizeof(r.wire[0]));
    const size_t max_prefixes = sizeof(r.prefix_begin) / sizeof(r.prefix_begin[0]);
    if (nw > max_wires || mn.prefixes.size() > max_prefixes || r.n_wires > max_wires ||
        r.n_prefixes != (int32_t)mn.prefixes.size() || r.n_suffixes != (int32_t)mn.suffixes.size()) {
      fprintf(stderr, "initiate_mnode_wiring: node %zu has %zu prefixes and %zu suffixes, its wiring "
                      "%d and %d (%d wires)\n", i, mn.prefixes.size(), mn.suffixes.size(), r.n_prefixes,
              r.n_suffixes, r.n_wires);
      die(PK_ERR_DEVICE, "pk_copy_wiring");
    }
    mn.wiring_info.assign(nw, WireInfo{0, 0, 0});
    for (int x = 0; x < nw; x++) mn.wiring_info[x] = WireInfo{r.wire[x][0], r.wire[x][1], r.wire[x][2]};
    mn.prefix_begin_info.assign(mn.prefixes.size(), PrefixInfo{0, 0});
    for (size_t p = 0; p < mn.prefixes.size(); p++)
      mn.prefix_begin_info[p] = PrefixInfo{r.prefix_begin[p][0], r.prefix_begin[p][1]};
  }
}

size_t begin_iterative_compaction(std::vector<std::pair<kmer_t, MacroNode>>& MN_map,
                                  std::vector<BasePairVector>& partial_contig_list) {
  ensure_job();
  if (rank == 0) fprintf(stderr, "Starting phase 2 iterative phase\n");
  pk_compaction_info ci;
  pk_status s = pk_compact(g_job, (uint64_t)node_threashold, coverage, &ci);
  if (s != PK_OK) die(s, "pk_compact");
  const size_t words = sizeof(kmer_t) / 8;
  std::vector<uint64_t> keys(ci.n_nodes * words + 1), eoff(ci.n_nodes + 1);
  std::vector<uint32_t> npre(ci.n_nodes + 1);
  std::vector<pk_compact_entry> ent(ci.n_entries + 1);
  std::vector<int32_t> wires(3 * (ci.n_entries + ci.n_nodes) + 3);
  std::vector<uint8_t> bases(ci.ext_bases + 1);
  s = pk_copy_compacted(g_job, keys.data(), eoff.data(), npre.data(), ent.data(), wires.data(), bases.data());
  if (s != PK_OK) die(s, "pk_copy_compacted");
  MN_map.clear();
  MN_map.reserve(ci.n_nodes);
  for (uint64_t i = 0; i < ci.n_nodes; i++) {
    const kmer_t key = key_at(keys, i);
    MacroNode mn;
    for (int b = 0; b < MN_LENGTH; b++) mn.k_1_mer.push_back(kmerel_mn(key, b));
    for (uint64_t e = eoff[i]; e < eoff[i + 1]; e++) {
      BasePairVector x;
      put_ext(x, bases.data() + ent[e].ext_offset, ent[e].ext_length);
      const bool is_pre = e - eoff[i] < npre[i];
      (is_pre ? mn.prefixes : mn.suffixes).push_back(x);
      (is_pre ? mn.prefix_count : mn.suffix_count).push_back(std::make_pair(ent[e].count, ent[e].visit));
      (is_pre ? mn.prefixes_terminal : mn.suffixes_terminal).push_back(ent[e].terminal != 0);
      if (is_pre) mn.prefix_begin_info.push_back(PrefixInfo{ent[e].prefix_pos, ent[e].num_wires});
    }
    for (uint64_t w = eoff[i] + i; w <= eoff[i + 1] + i; w++)
      mn.wiring_info.push_back(WireInfo{wires[3 * w], wires[3 * w + 1], wires[3 * w + 2]});
    MN_map.push_back(std::make_pair(key, mn));
  }
  std::vector<uint64_t> coff(ci.n_contigs + 1);
  std::vector<uint8_t> cb(ci.contig_bases + 1);
  s = pk_copy_partial_contigs(g_job, coff.data(), cb.data());
  if (s != PK_OK) die(s, "pk_copy_partial_contigs");
  for (uint64_t c = 0; c < ci.n_contigs; c++) {
    BasePairVector x;
    put_ext(x, cb.data() + coff[c], (uint32_t)(coff[c + 1] - coff[c]));
    partial_contig_list.push_back(x);
  }
  if (rank == 0) fprintf(stderr, "Completed iterative phase 2\n");
  return ci.n_nodes;
}

// every terminal prefix with visits, map order then prefix order
void identify_begin_kmers(std::vector<std::pair<kmer_t, MacroNode>>& MN_map,
                          std::vector<BeginMN>& list_of_begin_kmers) {
  for (size_t i = 0; i < MN_map.size(); i++) {
    const MacroNode& mn = MN_map[i].second;
    for (size_t l = 0; l < mn.prefixes.size(); l++)
      if (mn.prefix_count[l].second > 0 && mn.prefixes_terminal[l])
        list_of_begin_kmers.push_back(BeginMN{MN_map[i].first, (int)l});
  }
}

// one rank: every node is already local
void generate_compacted_pakgraph(std::vector<std::pair<kmer_t, MacroNode>>& MN_map,
                                 std::vector<std::pair<kmer_t, MacroNode>>& global_MN_map) {
  global_MN_map = MN_map;
}
