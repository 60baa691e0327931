/*
 * pakman_gb300.h -- C ABI of the GB300 k-mer counting / histogram cutoff /
 * macro-node construction path of PaKman.
 *
 * Plain C types only (pointers, sizes, fixed-width integers); no CUDA or torch
 * types appear in any signature (a CUDA stream is passed as `void*`).  Every
 * call returns a pk_status; the text of the last failure on the calling thread
 * is available from pk_last_error().  There is no CPU fallback: without a CUDA
 * device pk_ctx_create() fails with PK_ERR_NO_DEVICE.
 *
 * Which reference interface each entry point replaces (paths inside the PaKman
 * tree):
 *   pk_count / pk_count_device   perform_kmer_counting(const char*, size_t)
 *                                 src/kmer_counting.cpp:3351 (fills kmer_proc_buf,
 *                                 src/distribute_kmers.cpp:87, sorted and unique)
 *   pk_copy_table_packed          the kmer_proc_buf contents as packed KmerPairs
 *                                 (includes/distribute_kmers.h:702-714)
 *   pk_cutoff                     construct_kmer_histogram, src/kmer_histogram.cpp:72-115
 *                                 (histogram of counts < t, first-minimum cutoff)
 *   pk_build_macro_nodes          construct_macro_nodes / begin_mnode_construction,
 *                                 src/mn_construct.cpp:212-532
 *   pk_copy_macro_nodes           the MN_map contents (MacroNode suffix/prefix counts,
 *                                 includes/distribute_kmers.h:533-658)
 *   pk_run / pk_run_device        the driver sequence src/distribute_kmers.cpp:147-168
 *   pk_fasta_slice / pk_count_file
 *                                 perform_input_reading + DivideReads,
 *                                 src/input_reading.cpp:68-243, 246-303 (a rank's
 *                                 record-aligned slice of the FASTA file), streamed
 *                                 to the device and counted
 *   pk_wire_macro_nodes           initiate_mnode_wiring, src/wire.cpp:66-121
 *   pk_compact / pk_copy_compacted / pk_copy_partial_contigs
 *                                 begin_iterative_compaction (MN_map after the rounds,
 *                                 partial_contig_list), src/iterative_compaction.cpp:131-464
 *   pk_walk / pk_copy_walk_contigs
 *                                 identify_begin_kmers + traverse_pakgraph,
 *                                 src/iterative_compaction.cpp:65-93, src/walk.cpp:268-533
 */
#ifndef PAKMAN_GB300_H
#define PAKMAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pk_status {
  PK_OK = 0,
  PK_ERR_INVALID = 1,   /* bad argument (k outside 2..64, t < 1, null pointer, ...) */
  PK_ERR_FORMAT = 2,    /* a record start is not '>' (the reference asserts in its
                           l-mer and k-mer passes, src/kmer_counting.cpp:407, 2920) */
  PK_ERR_EMPTY = 3,     /* no k-mer reaches the cutoff (the reference calls
                           MPI_Abort, src/kmer_histogram.cpp:189-200) */
  PK_ERR_NOMEM = 4,     /* HBM budget of the context exceeded or allocation failed */
  PK_ERR_CUDA = 5,      /* CUDA runtime error */
  PK_ERR_STATE = 6,     /* call out of order (e.g. macro-nodes before counting) */
  PK_ERR_LIMIT = 7,     /* input beyond a documented limit (>= 2^32 k-mer windows) */
  PK_ERR_DEVICE = 8,    /* a kernel reported failure (bounded wait expired,
                           on-chip capacity exceeded); results are not valid */
  PK_ERR_BUSY = 9,      /* serving: no capacity right now, retry later */
  PK_ERR_NO_DEVICE = 10, /* no usable CUDA device */
  PK_ERR_IO = 11,        /* the input file cannot be opened or read (the reference
                            prints "Couldn't open the input FASTA file" and exits 2,
                            src/input_reading.cpp:260-265) */
  PK_ERR_CANCELLED = 12  /* serving: the request was cancelled (pk_cancel) */
} pk_status;

typedef struct pk_ctx pk_ctx;
typedef struct pk_job pk_job;

/* Run parameters.  Field meanings follow the reference's command line
 * (src/distribute_kmers.cpp:217-313) and build knobs (Makefile:1-20). */
typedef struct pk_params {
  int32_t k;            /* k-mer length (ksize; WINDW_SIZE = k-1), 2..64 */
  int32_t lmer_length;  /* LMER_LENGTH, default 8 */
  int32_t num_buckets;  /* -t: histogram bins, default 21 */
  int32_t coverage;     /* -c: visit count = ceil(count / coverage); non-zero */
  int32_t read_length;  /* -r: accepted and passed through; the counter does not use it */
  int32_t drop_n;       /* 0: reference behaviour (an 'N' is code 7 OR-ed into the
                           window); 1: windows containing 'N'/'n' are skipped */
  uint64_t batch_kmers; /* -b: MAX_KMER_COUNT, the piece size of counting in pieces (see
                           chunking); the table is the same for any value */
  int32_t bucket_bits;  /* partition digits (leading key bits), 2..18; 0 = automatic */
  int32_t mn_units;     /* macro-node work units: 0 = automatic (about 1000 kept rows
                           each); n > 0 = units of 4^(n-1) partition buckets */
  int32_t chunking;     /* -b pieces for host input (pk_count, pk_run, pk_count_file):
                           0 = automatic -- the whole input at once when it fits the
                           context's HBM budget and the 2^32-window limit, else in
                           record-aligned pieces of at most batch_kmers bytes (so at most
                           batch_kmers k-mer windows each) whose tables are merged on the
                           device; 1 = always in such pieces; 2 = never.  The table is the
                           same for any piece size, as the reference's is for any -b. */
  int32_t reserved[5];
} pk_params;

/* Counts reported by a run. */
typedef struct pk_summary {
  uint64_t n_reads;     /* '>' bytes in the buffer (the reference's "Total number of reads") */
  uint64_t n_windows;   /* k-mer instances counted (sum of the table's counts) */
  uint64_t n_unique;    /* distinct k-mers (table rows) */
  uint64_t n_kept;      /* rows with count >= cutoff */
  uint64_t n_nodes;     /* macro-nodes */
  uint32_t cutoff;      /* histogram cutoff (first minimum over [1, t)) */
  int32_t key_bytes;    /* 8 for k <= 32, 16 for k <= 64 */
} pk_summary;

void pk_params_default(pk_params* p);
const char* pk_status_string(pk_status s);
/* Text of the last failure on the calling thread ("" if none). */
const char* pk_last_error(void);

/* ---- context: one device, one HBM budget ------------------------------------- */
pk_status pk_ctx_create(int device, uint64_t hbm_budget_bytes, pk_ctx** out);
void pk_ctx_destroy(pk_ctx* ctx);
pk_status pk_ctx_memory(pk_ctx* ctx, uint64_t* used_bytes, uint64_t* budget_bytes);

/* ---- job: one read set; device buffers are held until reset/destroy ------------ */
/* stream: a cudaStream_t to run on, or NULL for a stream owned by the job. */
pk_status pk_job_create(pk_ctx* ctx, void* stream, pk_job** out);
void pk_job_destroy(pk_job* job);
pk_status pk_job_reset(pk_job* job);
pk_status pk_job_sync(pk_job* job);
/* Bytes of device memory the job holds now. */
pk_status pk_job_memory(pk_job* job, uint64_t* bytes);

/* ---- counting: replaces perform_kmer_counting -------------------------------------
 * fasta/d_fasta: one or more records, each a '>' header line followed by exactly one
 * sequence line (the reference's layout).  d_fasta must be 16-byte aligned device
 * memory; it is read, never written, and must stay valid until the job is synced.
 * Returns once the table is enqueued; the table stays resident on the device. */
pk_status pk_count(pk_job* job, const char* fasta, uint64_t n, const pk_params* p);
pk_status pk_count_device(pk_job* job, const void* d_fasta, uint64_t n, const pk_params* p);
pk_status pk_table_info(pk_job* job, uint64_t* n_unique, uint64_t* n_windows, uint64_t* n_reads);
/* Pieces the last count used: 1 when the whole input was counted at once, more when it
 * was counted in -b pieces (the reference's batch flush, src/kmer_counting.cpp:3022-3139)
 * and their tables merged. */
pk_status pk_count_pieces(pk_job* job, uint32_t* pieces);

/* ---- file ingest: replaces perform_input_reading ----------------------------------
 * The slice of a FASTA file that MPI rank `rank` of `n_ranks` reads in the reference
 * (DivideReads): rank r nominally owns bytes [r*(S/n), (r+1)*(S/n)) of the S-byte
 * file (the last rank to the end); its data start at the first '>' at or after its
 * nominal start (rank 0: byte 0) and end at the first '>' at or after the next rank's
 * nominal start (the last rank: end of file).  The reference looks for that '>'
 * inside an overlap of read_length + 100 bytes; here the search runs on to the end
 * of the file, which gives the same slice whenever the reference's search ends inside
 * its overlap.  The slices of ranks 0..n-1 tile the file.  Host only (no device). */
pk_status pk_fasta_slice(const char* path, int32_t rank, int32_t n_ranks, int32_t read_length,
                         uint64_t* offset, uint64_t* length);
/* pk_count on rank `rank`'s slice of the file, streamed: reader threads fill pinned
 * staging pieces from the file while earlier pieces are copied to the device and
 * line-scanned, so reading, copying and scanning overlap.  n_ranks = 1 counts the
 * whole file.  PK_ERR_IO when the file cannot be opened or read. */
pk_status pk_count_file(pk_job* job, const char* path, int32_t rank, int32_t n_ranks, const pk_params* p);

/* Load an existing frequency table instead of counting (the input of the PaK-Graph
 * builder, Pakman_Subgraph::build_graph, src/pakman_graph.hpp:592-673, whose table
 * comes from elsewhere).  Rows ascending and unique, keys below 4^k in the layout of
 * pk_copy_table, counts >= 1.  Afterwards pk_cutoff / pk_build_macro_nodes run as
 * after pk_count (n_windows = sum of counts, n_reads = 0). */
pk_status pk_table_load(pk_job* job, const void* keys, const uint32_t* counts, uint64_t n_rows,
                        const pk_params* params);
/* Table rows ascending by k-mer: keys as uint64 (k <= 32) or {uint64 lo, hi}
 * (k > 32), counts as uint32.  capacity = rows the buffers hold. */
pk_status pk_copy_table(pk_job* job, void* keys, uint32_t* counts, uint64_t capacity);
/* Same rows as packed KmerPairs {kmer_t seq; int k_count;} (12 or 20 bytes). */
pk_status pk_copy_table_packed(pk_job* job, void* pairs, uint64_t capacity);
/* Device pointers of the resident table (valid until reset/destroy). */
pk_status pk_table_device(pk_job* job, const void** d_keys, const uint32_t** d_counts);

/* ---- histogram cutoff: replaces construct_kmer_histogram ----------------------------
 * hist (optional) receives num_buckets bins.  Returns PK_ERR_EMPTY when no row
 * reaches the cutoff (cutoff, hist and n_kept are still filled in). */
pk_status pk_cutoff(pk_job* job, int32_t num_buckets, uint32_t* cutoff, uint64_t* hist,
                    uint64_t* n_kept);

/* ---- macro-nodes: replaces construct_macro_nodes ----------------------------------
 * min_count = 0 uses the cutoff from pk_cutoff; otherwise rows with count >=
 * min_count are kept.  Node keys are the (k-1)-mers ascending; per node four suffix
 * counts and four prefix counts indexed by extension base code (A=0 C=1 T=2 G=3),
 * 0 meaning absent.  Visit values are ceil(count / coverage). */
pk_status pk_build_macro_nodes(pk_job* job, uint32_t min_count, uint64_t* n_nodes);
pk_status pk_copy_macro_nodes(pk_job* job, void* keys, uint32_t* suffix_counts,
                              uint32_t* prefix_counts, uint64_t capacity);
pk_status pk_macro_nodes_device(pk_job* job, const void** d_keys, const uint32_t** d_suffix,
                                const uint32_t** d_prefix);

/* ---- whole path --------------------------------------------------------------------
 * count -> cutoff (p->num_buckets) -> macro-nodes, synchronised at the end. */
pk_status pk_run(pk_job* job, const char* fasta, uint64_t n, const pk_params* p, pk_summary* out);
pk_status pk_run_device(pk_job* job, const void* d_fasta, uint64_t n, const pk_params* p,
                        pk_summary* out);
/* ---- initial wiring: replaces initiate_mnode_wiring (src/wire.cpp:66-121) ---------
 * Per macro-node, MacroNode::setup_wiring (includes/distribute_kmers.h:549-655) after a
 * terminal entry is appended to both lists.  List entries: the present extensions in
 * ascending base code, then the terminal one (visit max(other side's visit sum - own
 * side's, 0)).  wire[w] = {suffix list index, offset in that suffix's visits, visits};
 * prefix_begin[p] = {first wire of prefix p, its wires}; unused entries are 0, as in
 * the reference.  The reference leaves the order of equal-ranked prefixes to an
 * unstable sort; here equal entries keep list order. */
typedef struct pk_wiring {
  int32_t n_suffixes;             /* list sizes including the terminal entry */
  int32_t n_prefixes;
  int32_t terminal_suffix_visit;
  int32_t terminal_prefix_visit;
  int32_t n_wires;
  int32_t wire[9][3];
  int32_t prefix_begin[5][2];
} pk_wiring;

/* After pk_build_macro_nodes; coverage 0 uses the job's params.coverage. */
pk_status pk_wire_macro_nodes(pk_job* job, int32_t coverage);
pk_status pk_copy_wiring(pk_job* job, pk_wiring* out, uint64_t capacity);
pk_status pk_wiring_device(pk_job* job, const pk_wiring** d_wiring);

/* ---- iterative compaction: replaces begin_iterative_compaction
 * (src/iterative_compaction.cpp:131-464) -------------------------------------------
 * Rounds of independent-set merging on the device until at most node_threshold
 * macro-nodes remain (the reference's -n; its command line turns 0 into 100000,
 * src/distribute_kmers.cpp:300-302).  A round merges every node whose non-terminal
 * neighbours all have smaller (k-1)-mers (generate_id_set, src/merge_mn.cpp:289-432):
 * each of its wires hands the predecessor a longer suffix and the successor a longer
 * prefix (iterate_and_pack_mn :433-550, push_to_pred / push_to_succ :1325-1411), or
 * becomes a partial contig when both ends are terminal; touched nodes are re-wired
 * (MacroNode::setup_wiring, includes/distribute_kmers.h:550-657).  The start is the
 * wired map of pk_wire_macro_nodes (lists in ascending base order).  Needs
 * pk_build_macro_nodes; coverage 0 uses the job's params.coverage.  Lists are held on
 * chip up to 32 entries a side (PK_ERR_DEVICE beyond, as for a node whose visits do
 * not balance or a transfer whose target is missing, where the reference asserts or
 * exits). */
typedef struct pk_compaction_info {
  uint64_t n_nodes;       /* nodes left (<= node_threshold) */
  uint64_t n_entries;     /* prefix + suffix entries over those nodes */
  uint64_t n_contigs;     /* partial contigs emitted by the rounds, in emission order */
  uint64_t ext_bases;     /* total extension length over the entries */
  uint64_t contig_bases;  /* total partial-contig length */
  int32_t rounds;
  int32_t key_bytes;      /* 8, or 16 for k > 32 */
} pk_compaction_info;

/* One prefix or suffix entry of a remaining node (MacroNode's per-entry vectors). */
typedef struct pk_compact_entry {
  uint64_t ext_offset;  /* into ext_bases: the extension's bases, one code per byte */
  uint32_t ext_length;  /* 0 for the terminal null entry */
  int32_t count;        /* first of the (count, visit) pair */
  int32_t visit;
  int32_t terminal;
  int32_t prefix_pos;   /* prefix_begin_info (prefix entries; 0 on suffix entries) */
  int32_t num_wires;
} pk_compact_entry;

pk_status pk_compact(pk_job* job, uint64_t node_threshold, int32_t coverage, pk_compaction_info* info);
pk_status pk_compaction_get_info(pk_job* job, pk_compaction_info* info);
/* Remaining nodes, ascending by key.  Node i's entries are entries[entry_offsets[i] ..
 * entry_offsets[i+1]): n_prefixes[i] prefixes, then its suffixes, each list in the
 * reference's order; its wiring_info is wires[3 * (entry_offsets[i] + i) ..] with
 * (n_entries of the node + 1) slots of {suffix_id, offset_in_suffix, count}.  Sizes
 * come from pk_compaction_info (keys n_nodes * key_bytes, entry_offsets n_nodes + 1,
 * wires 3 * (n_entries + n_nodes) int32, ext_bases ext_bases bytes); any pointer may
 * be NULL. */
pk_status pk_copy_compacted(pk_job* job, void* keys, uint64_t* entry_offsets, uint32_t* n_prefixes,
                            pk_compact_entry* entries, int32_t* wires, uint8_t* ext_bases);
/* Partial contigs in emission order: contig c is bases[offsets[c] .. offsets[c+1])
 * (base codes A=0 C=1 T=2 G=3); offsets has n_contigs + 1 slots. */
pk_status pk_copy_partial_contigs(pk_job* job, uint64_t* offsets, uint8_t* bases);

/* ---- walk: replaces identify_begin_kmers + traverse_pakgraph
 * (src/iterative_compaction.cpp:65-93, src/walk.cpp:268-533) -------------------------
 * On the map left by pk_compact: from every terminal prefix with visits (map order,
 * then prefix-list order) a depth-first walk over the wires, each wire taking its share
 * of the prefix's visits, emits a contig at every terminal suffix.  Contigs come in
 * begin order, then depth-first order -- the reference's order with one thread; all
 * contigs are returned (the reference writes those longer than 400 bases).  A missing
 * successor or prefix, an empty share, a contig of 500000 bases (the reference exits
 * or asserts) or a path deeper than max_depth nodes gives PK_ERR_DEVICE. */
typedef struct pk_walk_info {
  uint64_t n_begins;
  uint64_t n_contigs;
  uint64_t contig_bases;
  uint32_t max_depth;  /* frames on each walk's stack */
  uint32_t reserved;
} pk_walk_info;

pk_status pk_walk(pk_job* job, pk_walk_info* info);
/* contig c is bases[offsets[c] .. offsets[c+1]) (codes A=0 C=1 T=2 G=3); offsets has
 * n_contigs + 1 slots, bases contig_bases bytes. */
pk_status pk_copy_walk_contigs(pk_job* job, uint64_t* offsets, uint8_t* bases);

pk_status pk_summary_get(pk_job* job, pk_summary* out);

/* ---- bounded device waits -----------------------------------------------------------
 * Kernels that wait on other CTAs (the decoupled look-back of the kept-row filter and of
 * the macro-node kernel, a giant bucket waiting for its chunks) poll a bounded number of
 * times with a short sleep between polls, then set an error bit and return, so the call
 * fails with PK_ERR_DEVICE and the context stays usable.  spins = polls before a wait
 * gives up (0 = the default, about 1-2 s).  withhold_unit >= 0 makes that macro-node work
 * unit publish nothing, so the waits of the units after it run out: a fault injected on
 * the host side, for testing this error path; -1 turns it off.  Both apply to this
 * job's later calls. */
pk_status pk_job_set_wait_limit(pk_job* job, uint32_t spins, int32_t withhold_unit);

/* ---- per-kernel timing (CUDA events on the job's stream) ---------------------------- */
pk_status pk_job_enable_timing(pk_job* job, int on);
/* Milliseconds per stage of the last run; n_stages receives the stage count. */
pk_status pk_job_stage_times(pk_job* job, float* ms, int capacity, int* n_stages);
const char* pk_stage_name(int stage);

/* ---- histogram cutoff that allocates nothing ---------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory at
 * call time (an application whose own allocator owns every device allocation, a
 * latency-critical loop where an allocation may block, a process whose device-memory
 * budget is already committed): the histogram of counts < num_buckets, the first-
 * minimum cutoff over [1, num_buckets) and the number of rows >= cutoff -- the same
 * values as pk_cutoff -- over a count column already in device memory (for example the
 * counts from pk_table_device).  The results stay on the device, so no row reaching the
 * cutoff is not an error here: where pk_cutoff returns PK_ERR_EMPTY this call returns
 * PK_OK with *d_kept == 0, and the caller tests *d_kept before building macro-nodes.
 *   d_counts  device array of n_rows row counts (read only)
 *   d_cutoff  device output, 1 uint32 (required)
 *   d_hist    device output, num_buckets uint64, or NULL
 *   d_kept    device output, 1 uint64, or NULL
 *   stream    cudaStream_t to run on (NULL = the legacy default stream)
 * Scratch is one static device array of PK_NOALLOC_MAX_BUCKETS uint64 bins that every
 * GPU loading this library holds until the process exits; num_buckets above that
 * maximum returns PK_ERR_INVALID.  The function calls no cudaMalloc, cudaFree or other
 * allocating routine.  Its first call on a device, made with that device current, looks
 * up the scratch array's device address; make that first call before any stream
 * capture.  The address is kept for the rest of the process: after cudaDeviceReset on
 * that device this function must not be called again in the same process.  All calls share the one array and each call clears it first: calls whose
 * work overlaps on the GPU race and give wrong results.  Returns once the work is
 * enqueued on `stream`. */
#define PK_NOALLOC_MAX_BUCKETS 4096
pk_status pk_cutoff_noalloc(const uint32_t* d_counts, uint64_t n_rows, int32_t num_buckets,
                            uint32_t* d_cutoff, uint64_t* d_hist, uint64_t* d_kept, void* stream);

/* Pinned host memory for fast transfers (cudaHostAlloc). */
pk_status pk_host_alloc(uint64_t bytes, void** out);
void pk_host_free(void* p);

/* Library version string. */
const char* pk_version(void);
/* Kernel launches this library has made in this process so far (all jobs, contexts and
 * threads; a launch recorded into a CUDA graph counts once, when it is captured). */
uint64_t pk_kernel_launches(void);

/* ---- Serving: many independent count -> cutoff -> macro-node jobs on one GPU ----
 *
 * The submit / poll interface of the serving design (there is no reference
 * counterpart: the reference runs one read set per MPI job).  A server owns `workers`
 * worker threads on one context; a worker takes the next request as soon as its last
 * one has finished (continuous batching), so one request's host<->device copies and
 * host synchronisations overlap other requests' kernels.
 * Scheduling: the queued request with the least estimated work (FASTA bytes, doubled
 * for k > 32) starts first, so small requests are not queued behind large ones; a
 * request that has waited longer than aging_ms starts first regardless of size (while
 * it does not fit the budget, others start only in the memory it leaves).
 * Requests of at most small_bytes are small: reserved_small workers take only small
 * requests, and small requests run on high-priority CUDA streams.
 * Admission: a request starts only when the estimate of its device footprint, added to
 * the running requests' estimates and the device memory of kept results, fits the
 * context's HBM budget; a request that still runs out of device memory goes back to
 * the queue and starts again after another request has finished.  Results are
 * bit-identical to a job run alone. */
typedef struct pk_server pk_server;

typedef struct pk_request {
  const char* fasta;          /* host FASTA (pinned memory copies fastest); must stay
                                 valid until the request has completed */
  uint64_t fasta_bytes;
  pk_params params;
  /* Macro-node output, filled on completion.  Either caller buffers with room for
   * mn_capacity rows (keys: 8 or 16 bytes per row, suffix / prefix: 4 uint32 per
   * row; more nodes than that gives PK_ERR_LIMIT with n_nodes in the summary), or
   * all three NULL: the server keeps the table in pinned host memory, read with
   * pk_result_get(). */
  void* mn_keys;
  uint32_t* mn_suffix;
  uint32_t* mn_prefix;
  uint64_t mn_capacity;
  /* 1: the finished request's job -- its k-mer table and macro-nodes resident in HBM --
   * is kept for the caller (pk_result_job) until pk_result_release, and its device
   * memory counts against the budget meanwhile; the macro-node buffers above are then
   * optional (NULL: nothing is copied to the host). */
  int32_t keep_on_device;
  int32_t reserved[3];
} pk_request;

typedef struct pk_request_info {
  pk_status status;           /* the job's own status (PK_OK, PK_ERR_FORMAT, ...) */
  int32_t done;               /* 1 once the job has finished (ok or failed) */
  pk_summary summary;
  uint64_t submit_ns;         /* CLOCK_MONOTONIC timestamps */
  uint64_t start_ns;
  uint64_t end_ns;
  uint32_t attempts;          /* > 1 when the job was re-queued after running out of HBM */
  uint32_t reserved;
} pk_request_info;

typedef struct pk_server_stats {
  uint64_t submitted, completed, failed, queued, running;
  uint64_t admitted_bytes;       /* sum of the running jobs' footprint estimates */
  uint64_t peak_admitted_bytes;  /* peak of admitted_bytes + resident_bytes */
  uint64_t requeued;             /* jobs re-queued after running out of HBM */
  uint64_t cancelled;
  uint64_t resident_bytes;       /* device memory of results kept on the device */
  uint64_t resident_jobs;
  /* worker wall time summed over finished requests, by phase: counting (input copy
   * included), histogram cutoff, macro-nodes, copying the result out, releasing the
   * job's device buffers */
  uint64_t count_ns, cutoff_ns, mn_ns, copyout_ns, release_ns;
  uint64_t pin_ns;               /* of copyout_ns: page-locking new host blocks for results */
} pk_server_stats;

typedef struct pk_server_config {
  uint64_t small_bytes;    /* requests of at most this estimated work are small (32 MiB) */
  int32_t reserved_small;  /* workers that take only small requests (one in eight) */
  int32_t aging_ms;        /* a request waiting longer starts first (2000) */
  /* SMs set aside for small requests (0: none).  When > 0 the device is split into two
   * SM partitions (green contexts): small requests run on their own SMs (rounded up to
   * the device's partition granularity) and the rest on the others, so a small request
   * never waits for a large one's kernels; pk_server_create_config fails with
   * PK_ERR_CUDA when the driver cannot partition the device. */
  int32_t small_sms;
  int32_t reserved[3];
} pk_server_config;

void pk_server_config_default(pk_server_config* cfg, int32_t workers);
pk_status pk_server_create(pk_ctx* ctx, int32_t workers, pk_server** out);
/* cfg NULL: the defaults of pk_server_config_default. */
pk_status pk_server_create_config(pk_ctx* ctx, int32_t workers, const pk_server_config* cfg,
                                  pk_server** out);
/* The SMs of the server's partitions: small requests' and the others' (both the whole
 * device's count when the server has no partition). */
pk_status pk_server_partition(pk_server* s, int32_t* small_sms, int32_t* large_sms);
/* Cancels queued requests and ends running ones at their next stage boundary, waits for
 * the workers, frees every result. */
void pk_server_destroy(pk_server* s);
pk_status pk_submit(pk_server* s, const pk_request* req, uint64_t* ticket);
/* A queued request ends at once, a running one at its next stage boundary (after
 * counting or after the cutoff), with status PK_ERR_CANCELLED; PK_ERR_STATE once the
 * request has finished. */
pk_status pk_cancel(pk_server* s, uint64_t ticket);
/* Non-blocking: fills *info (info->done == 0 while queued or running). */
pk_status pk_poll(pk_server* s, uint64_t ticket, pk_request_info* info);
/* Completion order: the next finished (or cancelled) request not handed out before, its
 * ticket and state; blocks up to timeout_ms (< 0: no limit), PK_ERR_BUSY on timeout.  A
 * caller that consumes results as they finish releases each one promptly, whatever
 * order the scheduler ran them in. */
pk_status pk_next_done(pk_server* s, int64_t timeout_ms, uint64_t* ticket, pk_request_info* info);
/* Blocks until the job is done or timeout_ms (< 0: no limit) passes; PK_ERR_BUSY on timeout. */
pk_status pk_wait(pk_server* s, uint64_t ticket, int64_t timeout_ms, pk_request_info* info);
/* Server-kept macro-node table of a finished request (valid until pk_result_release). */
pk_status pk_result_get(pk_server* s, uint64_t ticket, const void** keys, const uint32_t** suffix,
                        const uint32_t** prefix, uint64_t* n_nodes);
/* The job of a finished keep_on_device request: its table and macro-nodes stay resident
 * and every pk_* call on a job works on it (pk_copy_table, pk_wire_macro_nodes,
 * pk_compact, pk_walk, ...).  The server owns it: valid until pk_result_release. */
pk_status pk_result_job(pk_server* s, uint64_t ticket, pk_job** job);
/* Forgets a finished request and frees what the server kept for it (host tables and a
 * kept job's device memory).  The pinned host blocks of server-kept tables are recycled
 * by every server of the process (up to 32 GiB of free blocks are kept). */
pk_status pk_result_release(pk_server* s, uint64_t ticket);
/* Frees the recycled pinned host blocks no request holds. */
void pk_server_cache_release(void);
pk_status pk_server_get_stats(pk_server* s, pk_server_stats* out);
/* Device footprint the admission control assumes for a request (bytes): the FASTA,
 * keys and counts over the k-mer windows estimated from the first 256 KiB of the input,
 * kept rows and macro-nodes for one kept k-mer in twelve windows. */
uint64_t pk_request_footprint(const pk_request* req);

/* ---- Batching: many independent read sets in one CUDA-graph launch ----------------
 *
 * (No reference counterpart: the reference runs one read set per MPI job.)  The whole
 * count -> cutoff -> macro-node path of every set is captured once into one CUDA graph
 * (sets spread over `branches` concurrent graph branches, each with buffers sized for
 * its largest set) and replayed with a single launch while the batch's shape (set
 * sizes and parameters) stays the same.  The partition digits of each size class are
 * autotuned once (the fastest of the automatic choice and its neighbours, timed on
 * the class's largest set) unless params.bucket_bits is set.  Inside the graph a set's
 * window count is bounded by its size, its kept k-mers by 1/8 of that and all sets'
 * macro-nodes by the batch output capacity; a set that exceeds a bound (or fails) is
 * run again on its own, so every result equals the set run alone. */
typedef struct pk_batch pk_batch;

typedef struct pk_batch_set {
  const char* fasta;          /* host FASTA of the set (pinned memory copies fastest) */
  uint64_t fasta_bytes;
  pk_params params;
} pk_batch_set;

typedef struct pk_batch_result {
  pk_status status;           /* PK_OK, PK_ERR_EMPTY, PK_ERR_FORMAT, ... of this set */
  int32_t rerun;              /* 1 if the set was run again outside the graph */
  pk_summary summary;
  uint64_t mn_first;          /* first row of this set in the batch's macro-node table */
} pk_batch_result;

typedef struct pk_batch_stats {
  uint64_t graph_launches;    /* graph launches so far (one per pk_batch_run) */
  uint64_t graph_captures;    /* captures (the shape changed) */
  uint64_t kernels_per_launch;/* kernel nodes in the current graph */
  uint64_t reruns;            /* sets run again on their own */
  uint64_t tuned_classes;     /* size classes with autotuned partition digits */
  uint64_t total_nodes;       /* rows of the last run's macro-node table */
  double last_graph_ms;       /* device time of the last graph launch */
  double tune_ms;             /* host time spent autotuning */
} pk_batch_stats;

pk_status pk_batch_create(pk_ctx* ctx, int32_t branches, pk_batch** out);
void pk_batch_destroy(pk_batch* b);
/* Runs all sets; results[i] describes set i, whose macro-node rows are
 * [mn_first, mn_first + summary.n_nodes) of the batch table. */
pk_status pk_batch_run(pk_batch* b, const pk_batch_set* sets, int32_t n_sets, pk_batch_result* results);
/* The batch's macro-node table: every set's rows contiguous, at its mn_first (sets
 * are not in set order); capacity in rows. */
pk_status pk_batch_copy_macro_nodes(pk_batch* b, void* keys, uint32_t* suffix_counts,
                                    uint32_t* prefix_counts, uint64_t capacity);
pk_status pk_batch_get_stats(pk_batch* b, pk_batch_stats* out);
/* Where the sets' inputs are copied to the device.  PK_BATCH_INPUT_IN_GRAPH (the
 * default): when every set's FASTA is in page-locked host memory, the graph copies each
 * set itself, on the set's branch ahead of its kernels, so the copies overlap the other
 * branches' work (the graph reads the host buffers at every launch; new buffers
 * recapture it); otherwise, as with PK_BATCH_INPUT_BEFORE, all sets are copied before
 * the graph is launched. */
#define PK_BATCH_INPUT_IN_GRAPH 0
#define PK_BATCH_INPUT_BEFORE 1
pk_status pk_batch_set_input_mode(pk_batch* b, int32_t mode);
/* Autotuned partition digits for a set of this size and k (0 if not tuned yet). */
int32_t pk_batch_tuned_bits(pk_batch* b, uint64_t fasta_bytes, int32_t k);
/* The whole tuned launch shape of that size class: partition digits, counting/scatter
 * chunks as a multiple of the one-chunk-per-SM size, table CTAs per SM; PK_ERR_STATE
 * if the class has not been tuned. */
pk_status pk_batch_tuned_shape(pk_batch* b, uint64_t fasta_bytes, int32_t k, int32_t* digits,
                               int32_t* chunk_mult, int32_t* table_ctas);

#ifdef __cplusplus
}
#endif
#endif /* PAKMAN_GB300_H */
