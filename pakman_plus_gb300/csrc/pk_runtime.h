// Host runtime state shared by the C-ABI translation units: contexts, jobs and the
// stream-ordered stages of one job (pk_capi.cu), used by the batch runner too.
#ifndef PK_RUNTIME_H
#define PK_RUNTIME_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/pakman_gb300.h"
#include "pk_internal.h"

#define PK_CUDA(call)                                                                     \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return pk::set_error(e_ == cudaErrorMemoryAllocation ? PK_ERR_NOMEM : PK_ERR_CUDA,           \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                     \
  } while (0)

#define PK_TRY(expr)              \
  do {                            \
    pk_status s_ = (expr);        \
    if (s_ != PK_OK) return s_;   \
  } while (0)

// ---------------------------------------------------------------- context -------
struct pk_ctx {
  int device = 0;
  uint64_t budget = 0;
  std::atomic<uint64_t> used{0};
  cudaMemPool_t pool = nullptr;
  int sms = 0;
};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

enum Stage {
  ST_H2D = 0,
  ST_LINES,
  ST_BUCKET_COUNT,
  ST_OFFSETS,
  ST_SCATTER,
  ST_SCATTER_FINE,
  ST_TABLE,
  ST_CUTOFF,
  ST_FILTER,
  ST_MN,
  ST_COMPACT,
  ST_WALK,
  ST_COUNT_
};
static const char* kStageNames[ST_COUNT_] = {"h2d",          "line_scan",      "bucket_count",
                                             "bucket_offsets", "scatter_coarse", "scatter_fine",
                                             "bucket_table", "cutoff",         "kept_filter",
                                             "macro_nodes",  "compaction",     "walk"};

namespace pk {
struct CpState;  // iterative compaction buffers (pk_compact.cu)
}

struct pk_job {
  pk_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  pk_params params{};
  int wide = 0;
  int bbits = 0;
  int grid = 0;
  unsigned long long chunk = 0;
  uint64_t F = 0, N = 0;
  int t_hist = 0;
  int stage = 0;  // 0 none, 1 counted, 2 cutoff, 3 macro-nodes
  uint64_t mn_cap = 0;
  pk::Scalars* d_sc = nullptr;
  pk::Scalars* h_sc = nullptr;  // pinned mirror
  DevBuf fasta, tile_nl, counts, bstart, hstart, keys, tkeys, tcounts, tu, flags_m, hist, hist2,
      nkeys, nsuf, npre, packed, doff, dkeys, dcounts, flags_f, kkeys, kcounts, kstart, kcount, ksub,
      coff, cstart, slice_start, fcur, wiring, gfirst, gcount, chunk_bucket, gdone, chunk_u,
      units,   // packed units of the counting pass, rolled again by the coarse scatter
      bsmall;  // rows of each table bucket by count below kSmallCounts (the table kernel's)
  bool bsmall_valid = false;  // bsmall describes the current table
  // counting in pieces (pk_chunked.cu): the accumulated table (ping-pong) and the merge
  DevBuf acc_keys[2], acc_counts[2], merge_keys, merge_counts, merge_part;
  uint32_t pieces = 0;  // pieces the last count used (1: the whole input at once)
  bool dense_valid = false;
  bool wired = false;  // wiring matches the current macro-nodes
  pk::CpState* cp = nullptr;
  bool compacted = false;  // the compaction state matches the current macro-nodes
  bool timing = false;
  // launch shapes chosen by the batch autotuner (0: the defaults): counting/scatter chunks
  // of chunk_mult times the one-chunk-per-SM size, and table CTAs per SM
  int chunk_mult = 0;
  int table_ctas = 0;
  // bounded device waits: polls before a wait gives up (0: the default, about 1-2 s), and
  // a macro-node unit that withholds its look-back word (-1: none); see pk_job_set_wait_limit
  uint32_t wait_limit = 0;
  int32_t withhold_unit = -1;
  // graph mode (batch capture): no host synchronisation and no allocation; the
  // window count is bounded by ncap and scalars were initialised by the caller
  bool graph_mode = false;
  uint64_t ncap = 0;
  // file ingest (pk_count_file): the tiles were line-scanned and the scalars set up
  // as the pieces landed, so counting starts at the tile prefix
  bool lines_ready = false;
  static constexpr int kIngestBufs = 8;  // pinned staging pieces (two per reader thread)
  void* ing_host[kIngestBufs] = {};
  cudaEvent_t ing_ev[kIngestBufs] = {};
  cudaEvent_t ev0[ST_COUNT_] = {}, ev1[ST_COUNT_] = {};
  bool ev_rec[ST_COUNT_] = {};
};


namespace pk {
pk_status set_device(pk_ctx* c);
pk_status job_alloc(pk_job* j, DevBuf& b, size_t bytes);
void job_free_all(pk_job* j);
void cp_free(pk_job* j);  // the compaction state, if any
pk_status check_params(const pk_params* p);
int auto_bucket_bits(uint64_t F, int k, int wide);
// device FASTA -> resident table; in graph mode no host synchronisation happens and
// the window count is taken as j->ncap
pk_status count_impl(pk_job* j, const void* d_fasta, uint64_t n, const pk_params* p);
// pk_count's body: a host buffer counted at once, or in -b pieces (pk_params.chunking)
pk_status count_host(pk_job* j, const char* fasta, uint64_t n, const pk_params* p);
pk_status sync_scalars(pk_job* j);
pk_status cutoff_enqueue(pk_job* j, int t);
pk_status mn_enqueue(pk_job* j, uint32_t min_count, uint64_t kept_bound);
// the resident table as dense ascending rows in j->dkeys / j->dcounts (built on demand)
pk_status dense_table(pk_job* j);
// counting a host buffer in record-aligned pieces of at most `piece` bytes, merged into
// one table (pk_chunked.cu)
pk_status count_pieces(pk_job* j, const char* host, uint64_t n, const pk_params* p, uint64_t piece);
// frees every buffer of the counting stages except the table (tkeys, tcounts)
void release_piece_buffers(pk_job* j);
// every device buffer of a job, for freeing and accounting
int job_buffers(pk_job* j, DevBuf** out, int cap);
// per-stage CUDA events on the job's stream (when timing is on)
void mark_begin(pk_job* j, int st);
void mark_end(pk_job* j, int st);
}  // namespace pk

#endif  // PK_RUNTIME_H
