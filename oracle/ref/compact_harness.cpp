// Dump harness around the reference's iterative compaction (TEST INFRASTRUCTURE ONLY).
//
// Linked with the reference sources compiled unmodified from the read-only reference
// tree (the counting and macro-node objects of the dump harness plus
// src/iterative_compaction.cpp, src/merge_mn.cpp and src/walk.cpp) and the single-rank
// MPI shim.  It follows the reference driver's contig-generation order
// (src/distribute_kmers.cpp:166-182):
//   begin_mnode_construction -> initiate_mnode_wiring -> begin_iterative_compaction
// and writes the wired macro-node map before compaction, the map left when the node
// count reached the -n threshold, and the partial contigs the rounds emitted.
//
// usage: pakman_compact_k<K> OUT_PREFIX -f FASTA -r READLEN -c COV -n THRESHOLD [-t T]
//
// OUT_PREFIX.before / OUT_PREFIX.after : "PKC1" u32 k, u64 M, per node (map order):
//     u64 lo, u64 hi,
//     for suffixes then prefixes: u32 n, n x {u32 len, len x u8 base, i32 count,
//                                             i32 visit, u8 terminal},
//     u32 nw, nw x {i32 suffix_id, i32 offset_in_suffix, i32 count},
//     u32 np, np x {i32 prefix_pos, i32 num_wires}
// OUT_PREFIX.contigs : "PKP1" u64 n, n x {u32 len, len x u8 base}
// stdout last line : {"compact_s": .., "walk_s": .., "M0": .., "M1": .., "contigs": ..}
//
// With PK_REF_WALK=1 in the environment the harness then runs the reference's walk on
// the compacted map (identify_begin_kmers, src/iterative_compaction.cpp:65-93, and
// traverse_pakgraph, src/walk.cpp:401-533), which writes contigs_out_r0.fa (walk
// contigs longer than 400 bases) and contigs_par_r0.fa (partial contigs longer than
// 400 bases) into the working directory.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string>
#include <vector>

#include "distribute_kmers.h"

extern std::string inputFileName;
extern int read_length;
void parseCommandLine(const int argc, char* const argv[]);
void set_num_threads();
size_t begin_iterative_compaction(std::vector<std::pair<kmer_t, MacroNode>>& MN_map,
                                  std::vector<BasePairVector>& partial_contig_list);
void identify_begin_kmers(std::vector<std::pair<kmer_t, MacroNode>>& MN_map, std::vector<BeginMN>& list_of_begin_kmers);
void traverse_pakgraph(std::vector<std::pair<kmer_t, MacroNode>>& global_MN_map,
                       std::vector<BeginMN>& list_of_begin_kmers, std::vector<BasePairVector>& partial_contig_list);

static void put_key(FILE* f, kmer_t key) {
  uint64_t lo = (uint64_t)key;
#ifdef EXTEND_KMER
  uint64_t hi = (uint64_t)(key >> 64);
#else
  uint64_t hi = 0;
#endif
  fwrite(&lo, 8, 1, f);
  fwrite(&hi, 8, 1, f);
}

static void put_bases(FILE* f, const BasePairVector& v) {
  uint32_t n = (uint32_t)v.size();
  fwrite(&n, 4, 1, f);
  for (uint32_t i = 0; i < n; i++) {
    uint8_t b = (uint8_t)v[i];
    fwrite(&b, 1, 1, f);
  }
}

static void put_list(FILE* f, const std::vector<BasePairVector>& ext,
                     const std::vector<std::pair<int, int>>& cnt, const std::vector<bool>& term) {
  uint32_t n = (uint32_t)ext.size();
  fwrite(&n, 4, 1, f);
  for (uint32_t i = 0; i < n; i++) {
    put_bases(f, ext[i]);
    int32_t c = cnt[i].first, v = cnt[i].second;
    uint8_t t = term[i] ? 1 : 0;
    fwrite(&c, 4, 1, f);
    fwrite(&v, 4, 1, f);
    fwrite(&t, 1, 1, f);
  }
}

static void dump_map(const std::string& path, const std::vector<std::pair<kmer_t, MacroNode>>& map) {
  FILE* f = fopen(path.c_str(), "wb");
  uint32_t k = KMER_LENGTH;
  uint64_t m = map.size();
  fwrite("PKC1", 1, 4, f);
  fwrite(&k, 4, 1, f);
  fwrite(&m, 8, 1, f);
  for (const auto& kv : map) {
    put_key(f, kv.first);
    const MacroNode& mn = kv.second;
    put_list(f, mn.suffixes, mn.suffix_count, mn.suffixes_terminal);
    put_list(f, mn.prefixes, mn.prefix_count, mn.prefixes_terminal);
    uint32_t nw = (uint32_t)mn.wiring_info.size();
    fwrite(&nw, 4, 1, f);
    for (const WireInfo& w : mn.wiring_info) {
      int32_t a[3] = {w.suffix_id, w.offset_in_suffix, w.count};
      fwrite(a, 4, 3, f);
    }
    uint32_t np = (uint32_t)mn.prefix_begin_info.size();
    fwrite(&np, 4, 1, f);
    for (const PrefixInfo& pi : mn.prefix_begin_info) {
      int32_t a[2] = {pi.prefix_pos, pi.num_wires};
      fwrite(a, 4, 2, f);
    }
  }
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s OUT_PREFIX <pkmer options>\n", argv[0]);
    return 2;
  }
  std::string out = argv[1];
  MPI_Init(&argc, &argv);
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  MPI_Comm_size(MPI_COMM_WORLD, &size);
  parseCommandLine(argc - 1, argv + 1);
  set_num_threads();

  input_read_data rdata = perform_input_reading(rank, size, inputFileName, read_length);
  perform_kmer_counting(rdata.read_data, rdata.read_data_size);
  free(rdata.read_data);

  std::vector<std::pair<kmer_t, MacroNode>> MN_map;
  begin_mnode_construction(MN_map);
  initiate_mnode_wiring(MN_map);
  const uint64_t m0 = MN_map.size();
  dump_map(out + ".before", MN_map);

  std::vector<BasePairVector> contigs;
  double t0 = MPI_Wtime();
  begin_iterative_compaction(MN_map, contigs);
  double t1 = MPI_Wtime();
  dump_map(out + ".after", MN_map);
  {
    FILE* f = fopen((out + ".contigs").c_str(), "wb");
    uint64_t n = contigs.size();
    fwrite("PKP1", 1, 4, f);
    fwrite(&n, 8, 1, f);
    for (const BasePairVector& c : contigs) put_bases(f, c);
    fclose(f);
  }
  const uint64_t m1 = MN_map.size(), np = contigs.size();
  double t2 = t1, t3 = t1;
  const char* w = getenv("PK_REF_WALK");
  if (w && w[0] == '1') {
    std::vector<BeginMN> begins;
    t2 = MPI_Wtime();
    identify_begin_kmers(MN_map, begins);
    traverse_pakgraph(MN_map, begins, contigs);
    t3 = MPI_Wtime();
  }
  printf("{\"compact_s\": %.6f, \"walk_s\": %.6f, \"M0\": %llu, \"M1\": %llu, \"contigs\": %llu}\n",
         t1 - t0, t3 - t2, (unsigned long long)m0, (unsigned long long)m1, (unsigned long long)np);
  fflush(stdout);
  MPI_Finalize();
  return 0;
}
