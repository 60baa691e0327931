// Test driver for include/pakman_gb300.hpp: runs one builder call and writes what
// the caller observes (processor calls, graph nodes) to a binary file that the
// Python tests compare with the oracle.
//
//   builders_check counter   FASTA KLEN READ_LEN MAX_KMERS WIDE(0|1) VARIANT OUT
//   builders_check graph     TABLE KLEN THRESHOLD COV NPARTS OUT
//   builders_check build     FASTA K THRESHOLD COV OUT
//
// OUT of counter: per processor call u64 n, then n x {u64 lo, u64 hi, u64 count};
// stdout: "reads R calls C".
// OUT of graph/build: u64 M, per node u64 lo, u64 hi, then for suffixes and prefixes
// u32 n, n x {u8 base char, u64 count, i32 visit, u8 terminal}.
// TABLE: u64 n, n x {u64 lo, u64 hi, u64 count}.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <string>
#include <vector>

#include "pakman_gb300.hpp"

typedef unsigned __int128 u128;

static std::vector<char> slurp(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) { perror(path); exit(2); }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::vector<char> v(n > 0 ? n : 0);
  if (n > 0 && fread(v.data(), 1, n, f) != (size_t)n) exit(2);
  fclose(f);
  return v;
}

template <typename kmer_t>
struct recorder {
  FILE* out;
  mutable size_t calls = 0;
  template <typename It>
  void operator()(It b, It e) const {
    std::vector<It> items;
    for (It i = b; i != e; ++i) items.push_back(i);
    uint64_t n = items.size();
    fwrite(&n, 8, 1, out);
    for (It i : items) {
      uint64_t lo = (uint64_t)i->first, hi = (uint64_t)((u128)i->first >> 64), c = (uint64_t)i->second;
      fwrite(&lo, 8, 1, out);
      fwrite(&hi, 8, 1, out);
      fwrite(&c, 8, 1, out);
    }
    calls++;
  }
};

template <typename kmer_t>
static int run_counter(const std::vector<char>& in, size_t klen, size_t read_len, size_t max, const char* variant,
                       const char* outp) {
  FILE* out = fopen(outp, "wb");
  intel::esc::Concurrent_Kmer_Partial_Counter<kmer_t> c(klen, in.data(), in.data() + in.size(), read_len, max);
  recorder<kmer_t> rec{out};
  size_t reads = 0;
  if (!strcmp(variant, "default")) reads = c.default_count_and_process(rec);
  else if (!strcmp(variant, "omp_v3")) reads = c.concurrent_count_and_process_omp_v3(rec);
  else if (!strcmp(variant, "omp_explicit")) reads = c.concurrent_count_and_process_omp_explicit(rec);
  else if (!strcmp(variant, "sort")) reads = c.default_count_and_process_sort(rec);
  else return 3;
  fclose(out);
  printf("reads %zu calls %zu\n", reads, rec.calls);
  return 0;
}

template <typename kmer_t>
static void write_graph(const intel::esc::Pakman_Subgraph<kmer_t>& g, const char* outp) {
  FILE* out = fopen(outp, "wb");
  uint64_t m = g.size();
  fwrite(&m, 8, 1, out);
  for (const auto& nd : g.nodes()) {
    uint64_t lo = (uint64_t)nd.k1mer, hi = (uint64_t)((u128)nd.k1mer >> 64);
    fwrite(&lo, 8, 1, out);
    fwrite(&hi, 8, 1, out);
    for (const auto* side : {&nd.suffixes_, &nd.prefixes_}) {
      uint32_t n = side->size();
      fwrite(&n, 4, 1, out);
      for (const auto& e : *side) {
        uint8_t ch = (uint8_t)e.ext[0], t = e.terminal;
        uint64_t c = e.count;
        int32_t v = e.visit;
        fwrite(&ch, 1, 1, out);
        fwrite(&c, 8, 1, out);
        fwrite(&v, 4, 1, out);
        fwrite(&t, 1, 1, out);
      }
    }
  }
  fclose(out);
}

template <typename kmer_t>
static int run_graph(const char* table, size_t klen, size_t threshold, size_t cov, size_t nparts, const char* outp) {
  std::vector<char> raw = slurp(table);
  uint64_t n;
  memcpy(&n, raw.data(), 8);
  // partitions as std::map (ordered) and the rows dealt round-robin over them
  std::vector<std::map<kmer_t, size_t>> parts(nparts);
  for (uint64_t i = 0; i < n; i++) {
    uint64_t lo, hi, c;
    memcpy(&lo, raw.data() + 8 + 24 * i, 8);
    memcpy(&hi, raw.data() + 16 + 24 * i, 8);
    memcpy(&c, raw.data() + 24 + 24 * i, 8);
    kmer_t x = (kmer_t)(((u128)hi << 64) | lo);
    parts[i % nparts][x] = c;
  }
  intel::esc::Pakman_Subgraph<kmer_t> g(klen);
  g.build_graph(parts, threshold, cov);
  write_graph(g, outp);
  return 0;
}

struct k32_traits { static size_t kmer_length() { return 32; } };
struct k63_traits { static size_t kmer_length() { return 63; } };

int main(int argc, char** argv) {
  if (argc < 2) return 3;
  std::string mode = argv[1];
  try {
    if (mode == "counter" && argc == 9) {
      std::vector<char> in = slurp(argv[2]);
      size_t klen = strtoull(argv[3], 0, 10), rl = strtoull(argv[4], 0, 10);
      size_t max = strtoull(argv[5], 0, 10);
      if (!strcmp(argv[5], "inf")) max = (size_t)-1;
      if (atoi(argv[6])) return run_counter<u128>(in, klen, rl, max, argv[7], argv[8]);
      return run_counter<size_t>(in, klen, rl, max, argv[7], argv[8]);
    }
    if (mode == "graph" && argc == 8) {
      size_t klen = strtoull(argv[3], 0, 10);
      if (klen > 32)
        return run_graph<u128>(argv[2], klen, strtoull(argv[4], 0, 10), strtoull(argv[5], 0, 10),
                               strtoull(argv[6], 0, 10), argv[7]);
      return run_graph<uint64_t>(argv[2], klen, strtoull(argv[4], 0, 10), strtoull(argv[5], 0, 10),
                                 strtoull(argv[6], 0, 10), argv[7]);
    }
    if (mode == "build" && argc == 7) {
      size_t k = strtoull(argv[3], 0, 10), thr = strtoull(argv[4], 0, 10), cov = strtoull(argv[5], 0, 10);
      if (k == 63) {
        intel::esc::Distributed_Pak_Graph<u128, k63_traits, void> d;
        d.default_build(argv[2], thr, cov);
        write_graph(d.graph(), argv[6]);
      } else {
        intel::esc::Distributed_Pak_Graph<uint64_t, k32_traits, void> d;
        d.default_build(argv[2], thr, cov);
        write_graph(d.graph(), argv[6]);
      }
      return 0;
    }
  } catch (const pakman_gb300::device_error& e) {
    fprintf(stderr, "device_error %d: %s\n", (int)e.status, e.what());
    return 4;
  }
  return 3;
}
