// Dump harness around the reference's own hot path (TEST INFRASTRUCTURE ONLY).
//
// Linked with the reference sources compiled unmodified from the read-only
// reference tree (src/distribute_kmers.cpp with its `main` renamed,
// src/input_reading.cpp, src/kmer_counting.cpp, src/kmer_histogram.cpp,
// src/mn_construct.cpp, src/timers.cpp) plus the single-rank MPI shim.  It
// follows the reference driver's order (src/distribute_kmers.cpp:132-168):
//   parseCommandLine -> perform_input_reading -> perform_kmer_counting
//   -> begin_mnode_construction
// and writes the k-mer table (`kmer_proc_buf`, src/distribute_kmers.cpp:87) and
// the macro-node map (`MN_map`) to binary files, so tests can pin the oracle
// against the reference's own outputs.
//
// usage: pakman_ref_k<K> OUT_PREFIX -f FASTA -r READLEN -c COV [-t T] [-b B] [-p V]
//
// OUT_PREFIX.table : "PKT1" u32 k, u64 U, U x {u64 lo, u64 hi, i32 count}
// OUT_PREFIX.mn    : "PKM1" u32 k, u64 M, per node:
//                    u64 lo, u64 hi, u32 k1len, k1len x u8 base,
//                    u32 nsuf, nsuf x {u8 ext, i32 count, i32 visit, u8 term},
//                    u32 npre, npre x {u8 ext, i32 count, i32 visit, u8 term}
// OUT_PREFIX.wire  : "PKW1" u64 M, per node after initiate_mnode_wiring
//                    (src/wire.cpp:66-121): for suffixes then prefixes u32 n,
//                    n x {u8 ext (0xff = terminal), i32 count, i32 visit};
//                    u32 nw, nw x {i32 suffix_id, i32 offset_in_suffix, i32 count};
//                    u32 np, np x {i32 prefix_pos, i32 num_wires}
// stdout last line : {"count_s": .., "mn_s": .., "U": .., "M": ..}
#include <stdio.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "distribute_kmers.h"

extern std::vector<KmerPairs> kmer_proc_buf;
extern std::string inputFileName;
extern int read_length;
void parseCommandLine(const int argc, char* const argv[]);
void set_num_threads();

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

static void put_ext_list(FILE* f, const std::vector<BasePairVector>& ext,
                         const std::vector<std::pair<int, int>>& cnt, const std::vector<bool>& term) {
  uint32_t n = (uint32_t)ext.size();
  fwrite(&n, 4, 1, f);
  for (uint32_t i = 0; i < n; i++) {
    uint8_t e = ext[i].size() ? (uint8_t)ext[i][0] : (uint8_t)0xff;
    int32_t c = cnt[i].first, v = cnt[i].second;
    uint8_t t = term[i] ? 1 : 0;
    fwrite(&e, 1, 1, f);
    fwrite(&c, 4, 1, f);
    fwrite(&v, 4, 1, f);
    fwrite(&t, 1, 1, f);
  }
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

  double t0 = MPI_Wtime();
  perform_kmer_counting(rdata.read_data, rdata.read_data_size);
  double t1 = MPI_Wtime();
  free(rdata.read_data);

  uint32_t k = KMER_LENGTH;
  uint64_t u = kmer_proc_buf.size();
  {
    FILE* f = fopen((out + ".table").c_str(), "wb");
    fwrite("PKT1", 1, 4, f);
    fwrite(&k, 4, 1, f);
    fwrite(&u, 8, 1, f);
    for (const KmerPairs& kp : kmer_proc_buf) {
      put_key(f, kp.seq);
      int32_t c = kp.k_count;
      fwrite(&c, 4, 1, f);
    }
    fclose(f);
  }

  std::vector<std::pair<kmer_t, MacroNode>> MN_map;
  double t2 = MPI_Wtime();
  begin_mnode_construction(MN_map);
  double t3 = MPI_Wtime();

  {
    FILE* f = fopen((out + ".mn").c_str(), "wb");
    uint64_t m = MN_map.size();
    fwrite("PKM1", 1, 4, f);
    fwrite(&k, 4, 1, f);
    fwrite(&m, 8, 1, f);
    for (const auto& kv : MN_map) {
      put_key(f, kv.first);
      const MacroNode& mn = kv.second;
      uint32_t kl = (uint32_t)mn.k_1_mer.size();
      fwrite(&kl, 4, 1, f);
      for (uint32_t i = 0; i < kl; i++) {
        uint8_t b = (uint8_t)mn.k_1_mer[i];
        fwrite(&b, 1, 1, f);
      }
      put_ext_list(f, mn.suffixes, mn.suffix_count, mn.suffixes_terminal);
      put_ext_list(f, mn.prefixes, mn.prefix_count, mn.prefixes_terminal);
    }
    fclose(f);
  }
  // initial wiring on the same map, then its dump
  initiate_mnode_wiring(MN_map);
  {
    FILE* f = fopen((out + ".wire").c_str(), "wb");
    uint64_t m = MN_map.size();
    fwrite("PKW1", 1, 4, f);
    fwrite(&m, 8, 1, f);
    for (const auto& kv : MN_map) {
      const MacroNode& mn = kv.second;
      const std::vector<BasePairVector>* lists[2] = {&mn.suffixes, &mn.prefixes};
      const std::vector<std::pair<int, int>>* counts[2] = {&mn.suffix_count, &mn.prefix_count};
      for (int side = 0; side < 2; side++) {
        uint32_t n = (uint32_t)lists[side]->size();
        fwrite(&n, 4, 1, f);
        for (uint32_t i = 0; i < n; i++) {
          uint8_t e = (*lists[side])[i].size() ? (uint8_t)(*lists[side])[i][0] : (uint8_t)0xff;
          int32_t c = (*counts[side])[i].first, v = (*counts[side])[i].second;
          fwrite(&e, 1, 1, f);
          fwrite(&c, 4, 1, f);
          fwrite(&v, 4, 1, f);
        }
      }
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
  printf("{\"count_s\": %.6f, \"mn_s\": %.6f, \"U\": %llu, \"M\": %llu}\n", t1 - t0, t3 - t2,
         (unsigned long long)u, (unsigned long long)MN_map.size());
  fflush(stdout);
  MPI_Finalize();
  return 0;
}
