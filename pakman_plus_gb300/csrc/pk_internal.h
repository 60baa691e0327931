// Internal launcher interface between the C-ABI host runtime (pk_capi.cpp) and the
// sm_103a kernels (pk_kernels.cu).  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/pakman_gb300.h"

namespace pk {

// Records the calling thread's last-error text (pk_last_error) and returns s.
pk_status set_error(pk_status s, const std::string& msg);

// Counts one kernel launch made by this library (read by pk_kernel_launches); every
// launch site calls it as `note_launch(), kernel<<<...>>>(...)`.
void note_launch();

// Device error word bits (pk_job error flag).
enum : uint32_t {
  ERR_FORMAT = 1u,        // a record start is not '>' (reference asserts)
  ERR_LOOKBACK = 2u,      // a bounded look-back wait ran out
  ERR_BUCKET = 4u,        // a bucket could not be split small enough for on-chip counting
  ERR_MN_CAPACITY = 8u,   // a macro-node segment exceeded on-chip capacity
  ERR_TICKET = 16u,       // work ticket overrun (should not happen)
  ERR_BOUNDS = 32u,       // a computed index fell outside its buffer (write skipped)
};

constexpr int kTileBytes = 65536;   // line-scan tile; chunk boundaries are multiples of it
constexpr int kSegBytes = 64;       // bytes per thread per extraction step
constexpr int kBucketThreads = 512;
constexpr int kMnThreads = 128;
constexpr int kSmallCounts = 16;    // per-bucket histogram of the table kernel: counts 0..15
constexpr int kMnCap = 1536;        // items (k-mer records) per macro-node segment on chip
constexpr int kMnBinBits = 8;       // counting-sort bins of a macro-node segment
constexpr int kMnBins = 1 << kMnBinBits;
constexpr int kMnBinMax = 32;       // largest bin ranked within itself (else merge ranks)
constexpr int kHistSmem = 1024;     // count-histogram bins kept in shared memory
constexpr int kBucketStack = 256;   // pending sub-ranges of one bucket
constexpr int kSplitWays = 4;      // pieces an overflowing sub-range is cut into
constexpr int kMaxBucketAttempts = 1 << 16;  // sub-range attempts per bucket before giving up
constexpr int kCoarseBits = 7;     // pass-1 partition digits (coarse regions)
constexpr int kMaxPartBits = 18;   // partition digits (table buckets) at most
constexpr int kHistBits = 15;      // digits the counting pass histograms in shared memory
constexpr int kSortBinBits = 10;    // top remainder bits of the per-bucket counting sort
constexpr int kBinMax = 128;        // largest bin sorted by ranking (else radix sort)
// Giant buckets (skewed input: a homopolymer or tandem repeat and its error variants)
// are first reduced chunk by chunk, by many CTAs, to (key, count) pairs.
constexpr int kChunkKeys = 32768;                   // keys per chunk of a giant bucket
constexpr uint32_t kGiantKeys = 16u * kChunkKeys;   // a bucket this large is giant
constexpr uint32_t kChunkRaw = 0xffffffffu;         // chunk left as keys (too many distinct)

struct Scalars {                    // device-side scalars of one job
  unsigned long long s0;            // index of the first '>' (F if none)
  unsigned long long n_windows;     // number of k-mer instances
  unsigned long long n_reads;       // number of '>' bytes from s0 on
  uint32_t nl_before_s0;            // newlines in [0, s0)
  uint32_t err;                     // ERR_* bits
  uint32_t ticket_bucket;           // work tickets
  uint32_t ticket_mn;
  uint32_t cutoff;                  // histogram cutoff
  uint32_t ticket_filter;
  uint32_t ticket_fine;
  uint32_t ticket_fcount;
  uint32_t n_chunk_items;           // chunk items of giant buckets (table kernel)
  unsigned long long n_unique;      // U
  unsigned long long n_kept;        // V
  unsigned long long n_nodes;       // M
  unsigned long long n_kept_rows;   // V as counted by the filter
};

struct CountArgs {
  const uint8_t* fasta;
  unsigned long long F;
  int k;
  int lmer_m;        // min(k, LMER_LENGTH): record-start checks follow the l-mer pass
  int drop_n;
  int bbits;         // bucket bits (top bits of the 2k-bit key)
  int cbits;         // coarse bits of the pass-1 partition (<= bbits, <= kCoarseBits)
  int grid;          // extraction CTAs (chunks)
  unsigned long long chunk;  // bytes per chunk (multiple of kTileBytes)
  uint32_t* tile_nl;         // ceil(F / kTileBytes) + 1, exclusive newline prefix
  uint32_t* counts;          // grid x 2^bbits  (per-chunk bucket counts, then prefixes)
  uint32_t* bstart;          // 2^bbits + 1 bucket starts
  unsigned long long n_keys; // capacity of the bucketed key buffer (scatter pass)
  Scalars* sc;
  // Packed units written by the counting pass and rolled again by the coarse scatter.
  // Unit u (0..3) of kSegBytes-byte segment g (its bytes 16u..16u+15) sits at
  // [u * nseg + g] of the code and bit-2 planes; windows[g] has bit 16u + j set iff the
  // window whose newest byte is byte j of that unit was counted.
  uint32_t* unit_codes;      // 4 x nseg
  uint32_t* unit_nbits;      // 4 x nseg
  unsigned long long* unit_windows;  // nseg
  unsigned long long nseg;   // ceil(F / kSegBytes)
};

// The table is kept "sparse": the u rows of bucket b sit at [bstart[b], bstart[b] + u),
// inside the bucket's own key range, ascending.
struct BucketArgs {
  void* keys;                // bucketed keys (uint64 or u128), N entries; chunks of giant
                             // buckets are rewritten in place as (key, count) pairs
  const uint32_t* bstart;    // 2^bbits + 1
  void* tkeys;               // table keys out (N capacity)
  uint32_t* tcounts;         // table counts out (N capacity)
  uint32_t* tu;              // 2^bbits: rows per bucket
  unsigned long long* hist;  // t bins (zeroed)
  int t;
  int k;
  int bbits;
  unsigned long long cap;    // table capacity (rows)
  const uint32_t* gfirst;    // 2^bbits: first chunk item of each giant bucket (null: none)
  const uint32_t* gcount;    // 2^bbits: its chunk items (0: not giant)
  const uint32_t* chunk_bucket;  // per chunk item: its bucket
  uint32_t* gdone;           // 2^bbits: chunk items of the bucket finished
  uint32_t* chunk_u;         // per chunk item: pairs it left, or kChunkRaw
  uint32_t* bsmall;          // kSmallCounts x 2^bbits: rows of each bucket by count < kSmallCounts
  int spin_limit;            // polls of a bounded wait before it gives up (0: default)
  Scalars* sc;
};

// Kept rows (count >= cutoff), dense and ascending, with per-bucket extents.
struct FilterArgs {
  const void* tkeys;
  const uint32_t* tcounts;
  const uint32_t* bstart;
  const uint32_t* tu;
  unsigned long long* flags; // 2^bbits look-back words (zeroed)
  void* kkeys;               // kept keys out
  uint32_t* kcounts;         // kept counts out
  uint32_t* kstart;          // 2^bbits
  uint32_t* kcount;          // 2^bbits
  uint32_t* ksub;            // 3 * 2^bbits
  unsigned long long cap;    // kept-row capacity
  unsigned long long trows;  // rows the table count buffer holds (reads stay below)
  // the table kernel's rows per bucket by count below kSmallCounts (null: not known);
  // with a cutoff <= kSmallCounts a bucket's kept rows follow from them and its row count
  const uint32_t* bsmall;
  int k;
  int bbits;
  int spin_limit;            // polls of a bounded wait before it gives up (0: default)
  Scalars* sc;
};

struct MnArgs {
  const void* kkeys;
  const uint32_t* kcounts;
  const uint32_t* kstart;
  const uint32_t* kcount;
  const uint32_t* ksub;
  unsigned long long* flags; // 2^bbits look-back words (zeroed)
  void* nkeys;               // node keys out (capacity cap)
  uint32_t* nsuf;            // 4 * cap
  uint32_t* npre;            // 4 * cap
  unsigned long long cap;
  unsigned long long kcap;   // kept rows the kept buffers hold
  int k;
  int bbits;
  int level;                 // node units cover 4^level table buckets (0: one bucket, split)
  int spin_limit;            // polls of a bounded wait before it gives up (0: default)
  int withhold_unit;         // a unit that publishes no look-back word (-1: none; tests of
                             // the bounded waits)
  Scalars* sc;
};

// One macro-node's initial wiring (the pk_wiring layout of the C ABI).
struct WireRow {
  int32_t ns, np, term_suf, term_pre, nw;
  int32_t wire[9][3];
  int32_t begin[5][2];
};

// Launchers (all stream-ordered, no host synchronisation).
// SM count the calling thread's launches are sized for (a serving worker on an SM
// partition sets its partition's count; 0 restores the whole device)
void set_thread_sms(int n);
int thread_sms(int device_sms);

cudaError_t launch_line_scan(const CountArgs& a, cudaStream_t st);
// chunk items of the giant buckets (n_b >= kGiantKeys): floor(n_b / kChunkKeys)
// consecutive items each, from gfirst[b], gcount[b] of them; chunk_bucket maps an item
// to its bucket; sc->n_chunk_items = all items; gdone = 0
cudaError_t launch_giant_chunks(const uint32_t* bstart, int bbits, uint32_t* gfirst, uint32_t* gcount,
                                uint32_t* chunk_bucket, uint32_t* gdone, Scalars* sc, cudaStream_t st);
// the line scan in two halves: per-tile newline counts for tiles [tile0, tile0 + ntiles)
// (any order, any number of launches), then the prefix over all tiles
cudaError_t launch_line_tiles(const uint8_t* buf, unsigned long long F, uint32_t* tile_nl, Scalars* sc,
                              unsigned long long tile0, unsigned long long ntiles, cudaStream_t st);
cudaError_t launch_tile_prefix(const CountArgs& a, cudaStream_t st);
cudaError_t launch_bucket_count(const CountArgs& a, int wide, cudaStream_t st);
cudaError_t launch_fine_count(const void* in, const uint32_t* cstart, const uint32_t* slice_start,
                              uint32_t* bcount, int k, int bbits, int cbits, int wide, uint32_t* ticket,
                              cudaStream_t st);
cudaError_t launch_prefix(uint32_t* counts, int B, cudaStream_t st);
cudaError_t launch_wire(const void* nsuf, const void* npre, unsigned long long m, int coverage, WireRow* out,
                        cudaStream_t st);
// batch: reserve a set's rows in the batch macro-node table and copy them there
cudaError_t launch_batch_emit(const Scalars* sc, unsigned long long* counter, unsigned long long cap,
                              unsigned long long* res, const void* nkeys, const void* nsuf, const void* npre,
                              int wide, void* okeys, void* osuf, void* opre, cudaStream_t st);
cudaError_t launch_bucket_offsets(const CountArgs& a, cudaStream_t st);
// Two-pass partition: coarse regions (pass 1) then fine buckets inside each region.
// keys per pass-2 slice for a fan-out of 2^fb fine buckets per coarse region
int fine_slice_keys(int wide, int fb);
cudaError_t launch_coarse_offsets(const CountArgs& a, uint32_t* coff, uint32_t* cstart,
                                  uint32_t* slice_start, int slice_keys, cudaStream_t st);
cudaError_t launch_scatter_coarse(const CountArgs& a, const uint32_t* coff, void* out, int wide,
                                  cudaStream_t st);
cudaError_t launch_scatter_fine(const void* in, const uint32_t* cstart, const uint32_t* slice_start,
                                uint32_t* fcur, void* out, int k, int bbits, int cbits, int wide,
                                uint32_t* ticket, unsigned long long cap, uint32_t* err, cudaStream_t st);
cudaError_t launch_bucket_table(const BucketArgs& a, int wide, int grid, cudaStream_t st);
// bstart / tu of a dense ascending table (pk_table_load)
cudaError_t launch_table_bounds(const void* keys, unsigned long long n, int bbits, int k, uint32_t* bstart,
                                uint32_t* tu, int wide, cudaStream_t st);
cudaError_t launch_histogram(const uint32_t* tcounts, unsigned long long u, int t,
                             unsigned long long* hist, cudaStream_t st);
cudaError_t launch_cutoff(const unsigned long long* hist, int t, Scalars* sc, cudaStream_t st);
cudaError_t launch_filter_kept(const FilterArgs& a, int wide, int grid, cudaStream_t st);
cudaError_t launch_macro_nodes(const MnArgs& a, int wide, int grid, cudaStream_t st);
// Dense copy of the sparse table (doff: exclusive prefix of tu, computed by
// launch_row_offsets).  packed != null writes KmerPairs records instead of arrays.
cudaError_t launch_row_offsets(const uint32_t* tu, uint32_t* doff, int B, cudaStream_t st);
cudaError_t launch_compact_rows(const void* tkeys, const uint32_t* tcounts, const uint32_t* bstart,
                                const uint32_t* tu, const uint32_t* doff, int B, int wide,
                                void* dkeys, uint32_t* dcounts, void* packed, cudaStream_t st);

size_t bucket_smem_bytes(int wide);
size_t mn_smem_bytes(int wide);
int bucket_ctas_per_sm(int wide);
int mn_ctas_per_sm(int wide);

}  // namespace pk
