// Stand-in for the PaKman header the link-level drop-in is compiled against
// (includes/distribute_kmers.h in the PaKman tree), for testing the adapter without the
// reference sources.  It restates only the interface the adapter touches, with the
// reference's layouts where they matter to the adapter:
//   kmer_t             uint64_t, or unsigned __int128 with EXTEND_KMER (:82-89)
//   KmerPairs          packed {kmer_t seq; int k_count;} (:702-714)
//   MacroNode          its nine member vectors, in the reference's order (:533-658)
//   WireInfo, PrefixInfo, BeginMN   plain structs of ints (:516-531, :674-679)
//   KMER_LENGTH, MN_LENGTH, kmerel_mn   (:74-76, :767-771)
// BasePairVector keeps one base per byte here (the reference packs 2-bit bases into
// words); the adapter only appends bases and never looks at the storage.
// MPI_Abort ends the process with the low byte of its code, as an MPI launcher reports
// the reference's MPI_Abort(-99) (exit status 157).
#ifndef PK_DROPIN_STANDIN_H
#define PK_DROPIN_STANDIN_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <iostream>
#include <utility>
#include <vector>

#ifndef WINDW_SIZE
#error "WINDW_SIZE (k - 1) must be defined, as in the reference's build"
#endif
#ifndef LMER_LENGTH
#define LMER_LENGTH 8
#endif
#define KMER_LENGTH (WINDW_SIZE + 1)
#define MN_LENGTH (KMER_LENGTH - 1)

#ifdef EXTEND_KMER
typedef unsigned __int128 kmer_t;
#else
typedef uint64_t kmer_t;
#endif

typedef uint8_t BasePair;
typedef BasePair ElType;

extern int rank, size;

class BasePairVector {
 public:
  void push_back(BasePair b) { bases_.push_back(b); }
  size_t size() const { return bases_.size(); }
  BasePair operator[](size_t i) const { return bases_[i]; }

 private:
  std::vector<BasePair> bases_;
};

struct WireInfo {
  int suffix_id;
  int offset_in_suffix;
  int count;
};

struct PrefixInfo {
  int prefix_pos;
  int num_wires;
};

struct MacroNode {
  std::vector<BasePairVector> suffixes;
  std::vector<bool> suffixes_terminal;
  std::vector<std::pair<int, int>> suffix_count;
  std::vector<BasePairVector> prefixes;
  std::vector<bool> prefixes_terminal;
  std::vector<std::pair<int, int>> prefix_count;
  BasePairVector k_1_mer;
  std::vector<WireInfo> wiring_info;
  std::vector<PrefixInfo> prefix_begin_info;
};

typedef struct __attribute__((__packed__)) kmer_pairs {
  kmer_t seq;
  int k_count;
} KmerPairs;
static_assert(sizeof(KmerPairs) == sizeof(kmer_t) + sizeof(int), "KmerPairs is packed");

typedef struct begin_kmer_id {
  kmer_t node;
  int terminal_prefix_id;
} BeginMN;

// base `pos` of a (k-1)-mer, first base in the most significant bits
inline ElType kmerel_mn(kmer_t kmer, unsigned pos) {
  return (ElType)((kmer >> ((MN_LENGTH - pos - 1) * 2)) & 0x3);
}

#define MPI_COMM_WORLD 0
inline int MPI_Abort(int, int code) {
  fflush(stdout);
  fflush(stderr);
  exit(code & 0xff);
}

#endif  // PK_DROPIN_STANDIN_H
