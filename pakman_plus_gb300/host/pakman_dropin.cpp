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
