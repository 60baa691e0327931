// pakman_gb300.hpp -- C++ builder interfaces of PaKman over the GB300 C ABI.
//
// Header-only.  The classes keep the reference's names and call signatures so the
// reference's callers compile against them unchanged; all counting and macro-node
// work runs on the GPU through pakman_gb300.h (link with -lpakman_gb300).
//
//   intel::esc::Concurrent_Kmer_Partial_Counter<kmer_t>
//       the k-mer table builder of src/concurrent_kmer_counter.hpp:21-2140 (callers:
//       src/concurrent_kmer_table_builder.cpp:97-116,
//       src/default_kmer_table_builder.cpp:68-82, src/concurrent_kmer_counter_test.cpp)
//   intel::esc::Pakman_Subgraph<kmer_t>::build_graph(freq_table, threshold, cov)
//       the PaK-Graph builder of src/pakman_graph.hpp:592-673
//   intel::esc::Distributed_Pak_Graph<kmer_t, kmer_traits_t, node_traits_t>::default_build
//       the FASTA-to-graph driver called by src/default_pakgraph_builder.cpp:48
//
// Errors throw pakman_gb300::device_error (a std::runtime_error carrying the
// pk_status), where the reference throws std::logic_error or aborts.
#ifndef PAKMAN_GB300_HPP
#define PAKMAN_GB300_HPP

#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pakman_gb300.h"

namespace pakman_gb300 {

class device_error : public std::runtime_error {
 public:
  device_error(pk_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  pk_status status;
};

inline void check(pk_status s, const char* what) {
  if (s != PK_OK)
    throw device_error(s, std::string(what) + ": " + pk_status_string(s) + " (" + pk_last_error() + ")");
}

// One context per process on device 0 unless a caller passes its own.
inline pk_ctx* default_context() {
  static std::once_flag once;
  static pk_ctx* ctx = nullptr;
  static pk_status st = PK_OK;
  std::call_once(once, [] { st = pk_ctx_create(0, 0, &ctx); });
  check(st, "pk_ctx_create");
  return ctx;
}

struct job_deleter {
  void operator()(pk_job* j) const { pk_job_destroy(j); }
};
using job_ptr = std::unique_ptr<pk_job, job_deleter>;

inline job_ptr make_job(pk_ctx* ctx) {
  pk_job* j = nullptr;
  check(pk_job_create(ctx ? ctx : default_context(), nullptr, &j), "pk_job_create");
  return job_ptr(j);
}

inline char base_char(unsigned code) { return "ACTG"[code & 3]; }

}  // namespace pakman_gb300

namespace intel {
namespace esc {

// The k-mer table builder.  Semantics kept from the reference: a read is the
// `read_len` bytes after a header (skip_symbol ... delimiter), clipped at the buffer
// end; reads shorter than klen are skipped and not counted; symbols map A0 C1 T2 G3
// and anything else to 0; the k-mer register is not masked, so a key holds the last
// 8*sizeof(kmer_t)/2 bases (bases before the read start are A).  The processor is
// called with [begin, end) iterators over elements whose ->first is the k-mer and
// ->second the count; elements come in ascending k-mer order (the reference's order
// is that of its hash map, i.e. unspecified).
template <typename kmer_t, template <typename T> class allocator_t = std::allocator>
class Concurrent_Kmer_Partial_Counter {
 public:
  typedef std::pair<kmer_t, size_t> kmer_count_t;

  Concurrent_Kmer_Partial_Counter(size_t klen = 32, const char* symbol_begin = NULL,
                                  const char* symbol_end = NULL, size_t read_len = 100,
                                  size_t max_kmer_count = 1000000, char delimiter = '\n',
                                  char skip_symbol = '>', pk_ctx* ctx = nullptr)
      : klen_(klen), symbol_begin_(symbol_begin), symbol_end_(symbol_end), read_len_(read_len),
        max_kmer_count_(max_kmer_count), delimiter_(delimiter), skip_symbol_(skip_symbol), ctx_(ctx) {}

  void reset(char const* begin, char const* end) {
    symbol_begin_ = begin;
    symbol_end_ = end;
  }

  // src/concurrent_kmer_counter.hpp:2018-2082: the map is flushed to the processor
  // whenever it holds more than max_kmer_count distinct k-mers after a read, and once
  // more at the end (possibly empty).
  template <typename processor_t>
  size_t default_count_and_process(processor_t& processor) {
    prepare();
    const size_t R = read_off_.size();
    size_t s = 0;
    std::vector<kmer_count_t> table;
    while (s < R && max_kmer_count_ != (size_t)-1 && distinct(s, R) > max_kmer_count_) {
      // the first read r >= s after which reads [s, r] hold more than the limit:
      // an exponential probe for an upper bound, then a binary search
      size_t lo = s, hi = R - 1, step = 1;
      while (true) {
        const size_t r = std::min(s + step - 1, R - 1);
        if (distinct(s, r + 1) > max_kmer_count_) {
          hi = r;
          break;
        }
        lo = r + 1;
        step *= 2;
      }
      while (lo < hi) {
        const size_t mid = lo + (hi - lo) / 2;
        if (distinct(s, mid + 1) > max_kmer_count_) hi = mid; else lo = mid + 1;
      }
      count(s, lo + 1, &table);
      processor(table.begin(), table.end());
      s = lo + 1;
    }
    count(s, R, &table);
    processor(table.begin(), table.end());
    printf("Reads=%lu , Unique Kmers=%lu\n", (unsigned long)R, (unsigned long)table.size());
    symbol_begin_ = symbol_end_;
    return R;
  }

  // src/concurrent_kmer_counter.hpp:1932-2015 counts and prints but never calls the
  // processor; kept so.
  template <typename processor_t>
  size_t default_count_and_process_sort(processor_t&) {
    prepare();
    std::vector<kmer_count_t> table;
    count(0, read_off_.size(), &table);
    printf("Reads=%lu , Unique Kmers=%lu\n", (unsigned long)read_off_.size(), (unsigned long)table.size());
    symbol_begin_ = symbol_end_;
    return read_off_.size();
  }

  // The concurrent variants of the reference differ in their CPU threading only; with
  // the device building the whole table they all hand it to the processor in one call.
  template <typename P> size_t concurrent_count_and_process_omp(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_v0(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_v1(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_v3(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_good(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_explicit(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_implicit(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_implicit_v0(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_implicit_v1(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_implicit_map(P& p) { return whole(p); }
  template <typename P> size_t concurrent_count_and_process_omp_implicit_bit_vector(P& p) { return whole(p); }

 private:
  static constexpr size_t kBases = 4 * sizeof(kmer_t);  // bases one kmer_t register holds

  template <typename P>
  size_t whole(P& processor) {
    prepare();
    std::vector<kmer_count_t> table;
    count(0, read_off_.size(), &table);
    processor(table.begin(), table.end());
    symbol_begin_ = symbol_end_;
    return read_off_.size();
  }

  // Reads in the builder's sense, rewritten as records of the device path: each read
  // becomes ">\n" + (kBases - klen) 'A' + the read with every symbol other than
  // A/C/T/G written as 'A' + "\n", so the device's kBases-mers are exactly the
  // builder's unmasked registers.
  void prepare() {
    if (klen_ < 1 || klen_ > kBases)
      throw pakman_gb300::device_error(PK_ERR_INVALID, "klen must be in 1.." + std::to_string(kBases));
    buf_.clear();
    read_off_.clear();
    const char* p = symbol_begin_;
    const char* end = symbol_end_;
    while (p && p != end) {
      while (p != end && *p != skip_symbol_) ++p;
      if (p == end) break;
      ++p;
      while (p != end && *p != delimiter_) ++p;
      if (p == end) break;
      ++p;
      size_t rl = read_len_;
      if ((size_t)(end - p) < rl) rl = (size_t)(end - p);
      if (rl < klen_) continue;
      read_off_.push_back(buf_.size());
      buf_.push_back('>');
      buf_.push_back('\n');
      buf_.insert(buf_.end(), kBases - klen_, 'A');
      for (size_t i = 0; i < rl; i++) {
        const char c = p[i];
        buf_.push_back((c == 'A' || c == 'C' || c == 'T' || c == 'G') ? c : 'A');
      }
      buf_.push_back('\n');
    }
    end_off_ = buf_.size();
  }

  size_t off(size_t r) const { return r < read_off_.size() ? read_off_[r] : end_off_; }

  pk_params params() const {
    pk_params p;
    pk_params_default(&p);
    p.k = (int32_t)kBases;
    p.read_length = (int32_t)read_len_;
    return p;
  }

  // distinct k-mers of reads [a, b)
  size_t distinct(size_t a, size_t b) {
    if (a >= b) return 0;
    if (!job_) job_ = pakman_gb300::make_job(ctx_);
    pk_params p = params();
    pakman_gb300::check(pk_count(job_.get(), buf_.data() + off(a), off(b) - off(a), &p), "pk_count");
    uint64_t u = 0;
    pakman_gb300::check(pk_table_info(job_.get(), &u, nullptr, nullptr), "pk_table_info");
    return (size_t)u;
  }

  void count(size_t a, size_t b, std::vector<kmer_count_t>* out) {
    out->clear();
    if (a >= b) return;
    const size_t u = distinct(a, b);
    std::vector<uint64_t> keys(u * (kBases > 32 ? 2 : 1) + 2);
    std::vector<uint32_t> cnts(u + 1);
    pakman_gb300::check(pk_copy_table(job_.get(), keys.data(), cnts.data(), u), "pk_copy_table");
    out->reserve(u);
    for (size_t i = 0; i < u; i++) {
      kmer_t x;
      if (kBases > 32) {
        x = (kmer_t)(((unsigned __int128)keys[2 * i + 1] << 64) | keys[2 * i]);
      } else {
        x = (kmer_t)keys[i];
      }
      out->push_back(kmer_count_t(x, (size_t)cnts[i]));
    }
  }

  size_t klen_;
  const char* symbol_begin_;
  const char* symbol_end_;
  size_t read_len_;
  size_t max_kmer_count_;
  char delimiter_;
  char skip_symbol_;
  pk_ctx* ctx_;
  std::vector<char> buf_;
  std::vector<size_t> read_off_;
  size_t end_off_ = 0;
  pakman_gb300::job_ptr job_;
};

// The PaK-Graph builder.  build_graph keeps the k-mers with freq > threshold; the
// node of a k-mer's first k-1 bases gets a suffix entry (its last base), the node of
// its last k-1 bases a prefix entry (its first base), each with the count and
// visit = ceil(count / cov).  Nodes come out ascending by (k-1)-mer, entries within
// a node ascending by base code (the reference's order follows its thread-local
// hash maps and is unspecified).  The partitioned table is any container indexable
// by partition whose elements iterate over (kmer, freq) pairs; a k-mer must not
// occur in two partitions.
template <typename kmer_t>
class Pakman_Subgraph {
 public:
  struct extension_t {
    std::string ext;
    size_t count;
    int visit;
    bool terminal;
  };
  struct node_t {
    kmer_t k1mer;
    std::vector<extension_t> suffixes_;
    std::vector<extension_t> prefixes_;
  };

  explicit Pakman_Subgraph(size_t klen = 32, pk_ctx* ctx = nullptr) : klen_(klen), ctx_(ctx) {}

  template <typename partitioned_kmer_freq_table_t>
  void build_graph(const partitioned_kmer_freq_table_t& freq_table, size_t threshold, size_t cov = 100) {
    if (klen_ < 2 || klen_ > 64) throw pakman_gb300::device_error(PK_ERR_INVALID, "klen must be in 2..64");
    if (cov == 0) throw pakman_gb300::device_error(PK_ERR_INVALID, "cov must be >= 1");
    std::vector<std::pair<kmer_t, size_t>> rows;
    for (size_t t = 0; t < freq_table.size(); t++)
      for (auto it = freq_table[t].begin(); it != freq_table[t].end(); ++it)
        rows.push_back(std::pair<kmer_t, size_t>((kmer_t)it->first, (size_t)it->second));
    std::sort(rows.begin(), rows.end(),
              [](const std::pair<kmer_t, size_t>& a, const std::pair<kmer_t, size_t>& b) { return a.first < b.first; });
    const bool wide = klen_ > 32;
    std::vector<uint64_t> keys(rows.size() * (wide ? 2 : 1) + 2);
    std::vector<uint32_t> cnts(rows.size() + 1);
    size_t n = 0;
    for (size_t i = 0; i < rows.size(); i++) {
      if (i && rows[i].first == rows[i - 1].first)
        throw pakman_gb300::device_error(PK_ERR_INVALID, "a k-mer occurs in two partitions of the table");
      if (rows[i].second == 0) continue;  // never above a threshold
      const size_t c = rows[i].second > 0xffffffffull ? 0xffffffffull : rows[i].second;
      if (wide) {
        keys[2 * n] = (uint64_t)rows[i].first;
        keys[2 * n + 1] = (uint64_t)((unsigned __int128)rows[i].first >> 64);
      } else {
        keys[n] = (uint64_t)rows[i].first;
      }
      cnts[n] = (uint32_t)c;
      n++;
    }
    nodes_.clear();
    if (!job_) job_ = pakman_gb300::make_job(ctx_);
    pk_params p;
    pk_params_default(&p);
    p.k = (int32_t)klen_;
    p.coverage = (int32_t)cov;
    pakman_gb300::check(pk_table_load(job_.get(), keys.data(), cnts.data(), n, &p), "pk_table_load");
    if (n == 0) return;
    uint64_t m = 0;
    const uint64_t min_count = threshold + 1;
    if (min_count > 0xffffffffull) return;  // nothing can pass
    const pk_status st = pk_build_macro_nodes(job_.get(), (uint32_t)min_count, &m);
    if (st == PK_ERR_EMPTY) return;  // no k-mer above the threshold: an empty graph
    pakman_gb300::check(st, "pk_build_macro_nodes");
    read_nodes(m, cov);
  }

  const std::vector<node_t>& nodes() const { return nodes_; }
  size_t size() const { return nodes_.size(); }

 private:
  void read_nodes(uint64_t m, size_t cov) {
    const bool wide = klen_ > 32;
    std::vector<uint64_t> keys(m * (wide ? 2 : 1) + 2);
    std::vector<uint32_t> suf(4 * m + 4), pre(4 * m + 4);
    pakman_gb300::check(pk_copy_macro_nodes(job_.get(), keys.data(), suf.data(), pre.data(), m),
                        "pk_copy_macro_nodes");
    nodes_.resize(m);
    for (uint64_t i = 0; i < m; i++) {
      node_t& nd = nodes_[i];
      nd.k1mer = wide ? (kmer_t)(((unsigned __int128)keys[2 * i + 1] << 64) | keys[2 * i]) : (kmer_t)keys[i];
      for (unsigned e = 0; e < 4; e++) {
        if (suf[4 * i + e])
          nd.suffixes_.push_back(extension_t{std::string(1, pakman_gb300::base_char(e)), suf[4 * i + e],
                                             (int)((suf[4 * i + e] + cov - 1) / cov), false});
        if (pre[4 * i + e])
          nd.prefixes_.push_back(extension_t{std::string(1, pakman_gb300::base_char(e)), pre[4 * i + e],
                                             (int)((pre[4 * i + e] + cov - 1) / cov), false});
      }
    }
  }

  size_t klen_;
  pk_ctx* ctx_;
  pakman_gb300::job_ptr job_;
  std::vector<node_t> nodes_;
};

// FASTA file -> frequency table -> PaK-Graph (the driver the reference's
// default_pakgraph_builder calls with threshold - 1).  Counting follows the pkmer path
// (records of one header line and one sequence line); kmer_traits_t::kmer_length()
// gives k; node_traits_t (the reference's MPI rank traits) is accepted for signature
// compatibility: the graph is built on this process's GPU.
template <typename kmer_t, typename kmer_traits_t, typename node_traits_t = void>
class Distributed_Pak_Graph {
 public:
  explicit Distributed_Pak_Graph(pk_ctx* ctx = nullptr) : ctx_(ctx), graph_(kmer_traits_t::kmer_length(), ctx) {}

  void default_build(const char* fasta_file, size_t threshold, size_t cov = 100) {
    FILE* f = fopen(fasta_file, "rb");
    if (!f) throw std::logic_error("Unable to open file: " + std::string(fasta_file));
    fseek(f, 0, SEEK_END);
    const long len = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<char> data(len > 0 ? (size_t)len : 0);
    if (len > 0 && fread(data.data(), 1, (size_t)len, f) != (size_t)len) {
      fclose(f);
      throw std::logic_error("fread() failed");
    }
    fclose(f);
    const size_t k = kmer_traits_t::kmer_length();
    pakman_gb300::job_ptr job = pakman_gb300::make_job(ctx_);
    pk_params p;
    pk_params_default(&p);
    p.k = (int32_t)k;
    pakman_gb300::check(pk_count(job.get(), data.data(), data.size(), &p), "pk_count");
    uint64_t u = 0;
    pakman_gb300::check(pk_table_info(job.get(), &u, nullptr, nullptr), "pk_table_info");
    std::vector<uint64_t> keys(u * (k > 32 ? 2 : 1) + 2);
    std::vector<uint32_t> cnts(u + 1);
    pakman_gb300::check(pk_copy_table(job.get(), keys.data(), cnts.data(), u), "pk_copy_table");
    std::vector<std::vector<std::pair<kmer_t, size_t>>> table(1);
    table[0].reserve(u);
    for (uint64_t i = 0; i < u; i++)
      table[0].push_back(std::pair<kmer_t, size_t>(
          k > 32 ? (kmer_t)(((unsigned __int128)keys[2 * i + 1] << 64) | keys[2 * i]) : (kmer_t)keys[i],
          (size_t)cnts[i]));
    graph_.build_graph(table, threshold, cov);
  }

  const Pakman_Subgraph<kmer_t>& graph() const { return graph_; }

 private:
  pk_ctx* ctx_;
  Pakman_Subgraph<kmer_t> graph_;
};

}  // namespace esc
}  // namespace intel

#endif  // PAKMAN_GB300_HPP
