// Host runtime behind the C ABI (include/pakman_gb300.h): contexts with an HBM
// budget, jobs that own their device buffers, and the stream-ordered launch
// sequence of the counting -> cutoff -> macro-node path.  No CPU fallback: every
// result comes from the kernels in pk_kernels.cu.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pakman_gb300.h"
#include "pk_internal.h"
#include "pk_runtime.h"

using namespace pk;

static const int kMaxPartitionBits = kMaxPartBits;

// ------------------------------------------------------------------ errors ------
static thread_local std::string t_last_error;

static pk_status fail(pk_status s, const std::string& msg) {
  t_last_error = msg;
  return s;
}

pk_status pk::set_error(pk_status s, const std::string& msg) { return fail(s, msg); }


pk_status pk::set_device(pk_ctx* c) {
  PK_CUDA(cudaSetDevice(c->device));
  return PK_OK;
}

pk_status pk::job_alloc(pk_job* j, DevBuf& b, size_t bytes) {
  if (b.p && b.bytes >= bytes) return PK_OK;
  if (j->graph_mode) return fail(PK_ERR_STATE, "batch buffers are smaller than a set needs");
  if (b.p) {
    PK_CUDA(cudaFreeAsync(b.p, j->stream));
    j->ctx->used -= b.bytes;
    b.p = nullptr;
    b.bytes = 0;
  }
  if (bytes == 0) bytes = 16;
  bytes = (bytes + 255) & ~(size_t)255;
  uint64_t now = j->ctx->used.fetch_add(bytes) + bytes;
  if (j->ctx->budget && now > j->ctx->budget) {
    j->ctx->used -= bytes;
    return fail(PK_ERR_NOMEM, "HBM budget exceeded: need " + std::to_string(bytes) + " more bytes, " +
                                  std::to_string(now - bytes) + " of " + std::to_string(j->ctx->budget) +
                                  " in use");
  }
  cudaError_t e = cudaMallocFromPoolAsync(&b.p, bytes, j->ctx->pool, j->stream);
  if (e != cudaSuccess) {
    j->ctx->used -= bytes;
    b.p = nullptr;
    return fail(PK_ERR_NOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
  }
  b.bytes = bytes;
  return PK_OK;
}

static void job_free(pk_job* j, DevBuf& b) {
  if (b.p) {
    cudaFreeAsync(b.p, j->stream);
    j->ctx->used -= b.bytes;
  }
  b.p = nullptr;
  b.bytes = 0;
}

int pk::job_buffers(pk_job* j, DevBuf** out, int cap) {
  DevBuf* all[] = {&j->fasta, &j->tile_nl, &j->counts, &j->bstart, &j->hstart, &j->keys,  &j->tkeys,
                   &j->tcounts, &j->tu,    &j->flags_m, &j->hist,  &j->hist2,
                   &j->nkeys,  &j->nsuf,   &j->npre,    &j->packed,  &j->doff,  &j->dkeys,
                   &j->dcounts, &j->flags_f, &j->kkeys, &j->kcounts, &j->kstart, &j->kcount,
                   &j->ksub,  &j->coff,    &j->cstart,  &j->slice_start, &j->fcur, &j->wiring,
                   &j->gfirst, &j->gcount, &j->chunk_bucket, &j->gdone,
                   &j->chunk_u, &j->acc_keys[0], &j->acc_keys[1], &j->acc_counts[0], &j->acc_counts[1],
                   &j->merge_keys, &j->merge_counts, &j->merge_part, &j->units, &j->bsmall};
  const int n = (int)(sizeof(all) / sizeof(all[0]));
  for (int i = 0; i < n && i < cap; i++) out[i] = all[i];
  return n;
}

void pk::job_free_all(pk_job* j) {
  DevBuf* all[64];
  const int n = job_buffers(j, all, 64);
  for (int i = 0; i < n; i++) job_free(j, *all[i]);
  j->bsmall_valid = false;
  cp_free(j);
  j->compacted = false;
  j->dense_valid = false;
}

void pk::release_piece_buffers(pk_job* j) {
  DevBuf* all[64];
  const int n = job_buffers(j, all, 64);
  for (int i = 0; i < n; i++)
    if (all[i] != &j->tkeys && all[i] != &j->tcounts) job_free(j, *all[i]);
  j->dense_valid = false;
}

// per-stage CUDA events on the job's stream (begin/end pairs, so host-side gaps
// between stages are not charged to a kernel)
void pk::mark_begin(pk_job* j, int st) {
  if (j->timing) cudaEventRecord(j->ev0[st], j->stream);
}
void pk::mark_end(pk_job* j, int st) {
  if (j->timing) {
    cudaEventRecord(j->ev1[st], j->stream);
    j->ev_rec[st] = true;
  }
}

// ---------------------------------------------------------------- C ABI ---------
void pk_params_default(pk_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->k = 32;
  p->lmer_length = 8;
  p->num_buckets = 21;
  p->coverage = 1;
  p->read_length = 100;
  p->drop_n = 0;
  p->batch_kmers = 100000000ull;
  p->bucket_bits = 0;
}

const char* pk_status_string(pk_status s) {
  switch (s) {
    case PK_OK: return "ok";
    case PK_ERR_INVALID: return "invalid argument";
    case PK_ERR_FORMAT: return "FASTA record does not start with '>'";
    case PK_ERR_EMPTY: return "no k-mer reaches the histogram cutoff";
    case PK_ERR_NOMEM: return "out of device memory or HBM budget";
    case PK_ERR_CUDA: return "CUDA error";
    case PK_ERR_STATE: return "call out of order";
    case PK_ERR_LIMIT: return "input beyond supported size";
    case PK_ERR_DEVICE: return "device-side failure";
    case PK_ERR_BUSY: return "busy";
    case PK_ERR_NO_DEVICE: return "no CUDA device";
    case PK_ERR_IO: return "input file cannot be read";
    case PK_ERR_CANCELLED: return "cancelled";
  }
  return "unknown status";
}

const char* pk_last_error(void) { return t_last_error.c_str(); }

const char* pk_version(void) { return "pakman-gb300 0.1 (sm_103a)"; }

pk_status pk_ctx_create(int device, uint64_t budget, pk_ctx** out) {
  if (!out) return fail(PK_ERR_INVALID, "out is null");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n <= 0)
    return fail(PK_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (device < 0 || device >= n) return fail(PK_ERR_INVALID, "device index out of range");
  PK_CUDA(cudaSetDevice(device));
  pk_ctx* c = new pk_ctx();
  c->device = device;
  c->budget = budget;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  e = cudaMemPoolCreate(&c->pool, &props);
  if (e != cudaSuccess) {
    delete c;
    return fail(PK_ERR_CUDA, std::string("cudaMemPoolCreate: ") + cudaGetErrorString(e));
  }
  uint64_t thr = ~0ull;
  cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &thr);
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return PK_OK;
}

void pk_ctx_destroy(pk_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaDeviceSynchronize();
  if (c->pool) cudaMemPoolDestroy(c->pool);
  delete c;
}

pk_status pk_ctx_memory(pk_ctx* c, uint64_t* used, uint64_t* budget) {
  if (!c) return fail(PK_ERR_INVALID, "ctx is null");
  if (used) *used = c->used.load();
  if (budget) *budget = c->budget;
  return PK_OK;
}

pk_status pk_job_create(pk_ctx* c, void* stream, pk_job** out) {
  if (!c || !out) return fail(PK_ERR_INVALID, "null argument");
  PK_TRY(set_device(c));
  pk_job* j = new pk_job();
  j->ctx = c;
  if (stream) {
    j->stream = (cudaStream_t)stream;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete j;
      return fail(PK_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    j->own_stream = true;
  }
  cudaError_t e = cudaMalloc(&j->d_sc, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaHostAlloc(&j->h_sc, sizeof(Scalars), cudaHostAllocDefault);
  if (e != cudaSuccess) {
    if (j->d_sc) cudaFree(j->d_sc);
    if (j->own_stream) cudaStreamDestroy(j->stream);
    delete j;
    return fail(PK_ERR_NOMEM, std::string("job scalars: ") + cudaGetErrorString(e));
  }
  memset(j->h_sc, 0, sizeof(Scalars));
  for (int i = 0; i < ST_COUNT_; i++) {
    cudaEventCreate(&j->ev0[i]);
    cudaEventCreate(&j->ev1[i]);
  }
  *out = j;
  return PK_OK;
}

void pk_job_destroy(pk_job* j) {
  if (!j) return;
  cudaSetDevice(j->ctx->device);
  cudaStreamSynchronize(j->stream);
  job_free_all(j);
  cudaStreamSynchronize(j->stream);
  for (int i = 0; i < ST_COUNT_; i++) {
    if (j->ev0[i]) cudaEventDestroy(j->ev0[i]);
    if (j->ev1[i]) cudaEventDestroy(j->ev1[i]);
  }
  if (j->d_sc) cudaFree(j->d_sc);
  if (j->h_sc) cudaFreeHost(j->h_sc);
  for (int i = 0; i < pk_job::kIngestBufs; i++) {
    if (j->ing_host[i]) cudaFreeHost(j->ing_host[i]);
    if (j->ing_ev[i]) cudaEventDestroy(j->ing_ev[i]);
  }
  if (j->own_stream) cudaStreamDestroy(j->stream);
  delete j;
}

pk_status pk_job_reset(pk_job* j) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  PK_TRY(set_device(j->ctx));
  job_free_all(j);
  j->stage = 0;
  j->wired = false;
  PK_CUDA(cudaStreamSynchronize(j->stream));
  return PK_OK;
}

pk_status pk_job_sync(pk_job* j) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  PK_TRY(set_device(j->ctx));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  return PK_OK;
}

pk_status pk_job_memory(pk_job* j, uint64_t* bytes) {
  if (!j || !bytes) return fail(PK_ERR_INVALID, "null argument");
  DevBuf* all[64];
  const int n = job_buffers(j, all, 64);
  uint64_t s = 0;
  for (int i = 0; i < n; i++) s += all[i]->bytes;
  *bytes = s;
  return PK_OK;
}

pk_status pk_job_set_wait_limit(pk_job* j, uint32_t spins, int32_t withhold_unit) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (spins > (1u << 30)) return fail(PK_ERR_INVALID, "spins must be at most 2^30");
  j->wait_limit = spins;
  j->withhold_unit = withhold_unit < 0 ? -1 : withhold_unit;
  return PK_OK;
}

pk_status pk_job_enable_timing(pk_job* j, int on) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  j->timing = on != 0;
  return PK_OK;
}

pk_status pk_job_stage_times(pk_job* j, float* ms, int cap, int* n) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  PK_TRY(set_device(j->ctx));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  if (n) *n = ST_COUNT_;
  for (int s = 0; s < ST_COUNT_ && s < cap; s++) {
    float v = 0.f;
    if (j->ev_rec[s]) cudaEventElapsedTime(&v, j->ev0[s], j->ev1[s]);
    ms[s] = v;
  }
  return PK_OK;
}

const char* pk_stage_name(int s) { return (s >= 0 && s < ST_COUNT_) ? kStageNames[s] : ""; }

pk_status pk_host_alloc(uint64_t bytes, void** out) {
  if (!out) return fail(PK_ERR_INVALID, "out is null");
  PK_CUDA(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault));
  return PK_OK;
}

void pk_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

pk_status pk::check_params(const pk_params* p) {
  if (!p) return fail(PK_ERR_INVALID, "params is null");
  if (p->k < 2 || p->k > 64) return fail(PK_ERR_INVALID, "k must be in 2..64");
  if (p->lmer_length < 1 || p->lmer_length > 32) return fail(PK_ERR_INVALID, "lmer_length must be in 1..32");
  if (p->num_buckets < 1) return fail(PK_ERR_INVALID, "num_buckets (-t) must be >= 1");
  if (p->mn_units < 0 || p->mn_units > 16) return fail(PK_ERR_INVALID, "mn_units must be in 0..16");
  if (p->chunking < 0 || p->chunking > 2) return fail(PK_ERR_INVALID, "chunking must be 0, 1 or 2");
  if (p->bucket_bits < 0 || p->bucket_bits > kMaxPartitionBits)
    return fail(PK_ERR_INVALID, "bucket_bits must be in 0.." + std::to_string(kMaxPartitionBits));
  return PK_OK;
}

// Partition digits: the leading key bits that pick a bucket, sized so an average
// bucket holds a few thousand keys (the per-bucket kernel counts a bucket on chip).
// The keys reach their buckets in two passes (kCoarseBits coarse regions, then fine
// buckets inside each region), so the digit count is not tied to L2 capacity.
int pk::auto_bucket_bits(uint64_t F, int k, int wide) {
  // keys per bucket aimed at: large enough to amortise the per-bucket work of the
  // table and macro-node kernels, small enough that a bucket's distinct keys usually
  // fit one on-chip hash table (8192 64-bit or 4096 128-bit slots at load <= 1/2)
  const double per_bucket = wide ? 3000.0 : 16000.0;
  const double est = 0.62 * (double)F;               // k-mer windows per byte, 100 bp reads, k=32
  int b = 2;
  while (b < kMaxPartitionBits && est / (double)(1u << b) > per_bucket) b++;
  return std::max(2, std::min(b, 2 * k - 2));
}

static pk_status table_impl(pk_job* j, uint64_t N, int t);

// Stages 1-5: device FASTA -> sorted (k-mer, count) table, resident.
pk_status pk::count_impl(pk_job* j, const void* d_fasta, uint64_t n, const pk_params* p) {
  const int k = p->k;
  j->params = *p;
  j->wide = k > 32;
  j->F = n;
  j->stage = 0;
  j->wired = false;
  j->compacted = false;
  const int W = j->wide ? 16 : 8;
  const int bb = p->bucket_bits ? std::min(p->bucket_bits, std::min(kMaxPartitionBits, 2 * k - 2))
                                : auto_bucket_bits(n, k, j->wide);
  j->bbits = std::max(2, bb);
  const int B = 1 << j->bbits;
  // the counting pass histograms at most kHistBits digits; deeper partitions get their
  // fine bucket sizes from a count over the coarse regions (k_fine_count)
  const int hb = std::min(j->bbits, kHistBits);
  const int HB = 1 << hb;
  const uint64_t ntiles = (n + kTileBytes - 1) / kTileBytes;
  int grid = (int)std::min<uint64_t>((uint64_t)thread_sms(j->ctx->sms), std::max<uint64_t>(ntiles, 1));
  unsigned long long chunk = (ntiles + grid - 1) / grid * (unsigned long long)kTileBytes;
  if (chunk == 0) chunk = kTileBytes;
  if (j->chunk_mult > 1) chunk *= (unsigned long long)j->chunk_mult;  // fewer, longer chunks
  grid = (int)std::max<uint64_t>(1, (n + chunk - 1) / chunk);
  j->grid = grid;
  j->chunk = chunk;

  PK_TRY(job_alloc(j, j->tile_nl, sizeof(uint32_t) * (ntiles + 1)));
  PK_TRY(job_alloc(j, j->counts, sizeof(uint32_t) * (size_t)grid * HB));
  // packed units: 4 x nseg codes, 4 x nseg bit-2 planes, nseg window masks (10 bytes per
  // 16 input bytes)
  const uint64_t nseg = (n + kSegBytes - 1) / kSegBytes;
  PK_TRY(job_alloc(j, j->units, (size_t)40 * nseg));
  PK_TRY(job_alloc(j, j->bstart, sizeof(uint32_t) * (B + 1)));
  if (hb < j->bbits) PK_TRY(job_alloc(j, j->hstart, sizeof(uint32_t) * (HB + 1)));
  uint32_t* hstart = (uint32_t*)(hb < j->bbits ? j->hstart.p : j->bstart.p);
  if (!j->graph_mode && !j->lines_ready) {
    Scalars init{};
    memset(&init, 0, sizeof(init));
    init.s0 = ~0ull;
    *j->h_sc = init;
    PK_CUDA(cudaMemcpyAsync(j->d_sc, j->h_sc, sizeof(Scalars), cudaMemcpyHostToDevice, j->stream));
  }

  CountArgs a{};
  a.fasta = (const uint8_t*)d_fasta;
  a.F = n;
  a.k = k;
  a.lmer_m = std::min(k, p->lmer_length);
  a.drop_n = p->drop_n ? 1 : 0;
  a.bbits = hb;
  a.cbits = std::min(j->bbits, kCoarseBits);
  a.grid = grid;
  a.chunk = chunk;
  a.tile_nl = (uint32_t*)j->tile_nl.p;
  a.counts = (uint32_t*)j->counts.p;
  a.bstart = hstart;
  a.sc = j->d_sc;
  a.nseg = nseg;
  a.unit_codes = (uint32_t*)j->units.p;
  a.unit_nbits = a.unit_codes + 4 * nseg;
  a.unit_windows = (unsigned long long*)(a.unit_nbits + 4 * nseg);

  mark_begin(j, ST_LINES);
  if (j->lines_ready) PK_CUDA(launch_tile_prefix(a, j->stream));
  else PK_CUDA(launch_line_scan(a, j->stream));
  mark_end(j, ST_LINES);
  mark_begin(j, ST_BUCKET_COUNT);
  PK_CUDA(launch_bucket_count(a, j->wide, j->stream));
  mark_end(j, ST_BUCKET_COUNT);
  mark_begin(j, ST_OFFSETS);
  PK_CUDA(launch_bucket_offsets(a, j->stream));
  mark_end(j, ST_OFFSETS);
  // the key buffer is sized by the exact window count (graph mode: by the bound the
  // caller sized its buffers for)
  uint64_t N = j->ncap;
  if (!j->graph_mode) {
    PK_CUDA(cudaMemcpyAsync(j->h_sc, j->d_sc, sizeof(Scalars), cudaMemcpyDeviceToHost, j->stream));
    PK_CUDA(cudaStreamSynchronize(j->stream));
    if (j->h_sc->err & ERR_FORMAT)
      return fail(PK_ERR_FORMAT, "a FASTA record start is not '>' (one '>' header line and one "
                                 "sequence line per record expected)");
    N = j->h_sc->n_windows;
  }
  if (N >= (1ull << 32) - 1)
    return fail(PK_ERR_LIMIT, "more than 2^32-2 k-mer windows in one job; split the input");
  j->N = N;
  PK_TRY(job_alloc(j, j->keys, (size_t)W * N));
  a.n_keys = N;
  PK_TRY(job_alloc(j, j->tkeys, (size_t)W * N));
  PK_TRY(job_alloc(j, j->tcounts, sizeof(uint32_t) * N));
  PK_TRY(job_alloc(j, j->tu, sizeof(uint32_t) * (size_t)B));
  const int t = p->num_buckets;
  PK_TRY(job_alloc(j, j->hist, sizeof(unsigned long long) * (size_t)t));
  PK_CUDA(cudaMemsetAsync(j->hist.p, 0, sizeof(unsigned long long) * (size_t)t, j->stream));
  j->t_hist = t;
  j->dense_valid = false;

  // two-pass partition: coarse regions (pass 1), then fine buckets (pass 2).  The
  // coarse copy lives in the table buffer, which is written only after pass 2.
  const int Cn = 1 << a.cbits;
  PK_TRY(job_alloc(j, j->coff, sizeof(uint32_t) * (size_t)grid * Cn));
  PK_TRY(job_alloc(j, j->cstart, sizeof(uint32_t) * (Cn + 1)));
  PK_TRY(job_alloc(j, j->slice_start, sizeof(uint32_t) * (Cn + 1)));
  PK_TRY(job_alloc(j, j->fcur, sizeof(uint32_t) * (size_t)B));
  const bool two_pass = a.cbits < a.bbits;
  mark_begin(j, ST_SCATTER);
  PK_CUDA(launch_coarse_offsets(a, (uint32_t*)j->coff.p, (uint32_t*)j->cstart.p,
                                (uint32_t*)j->slice_start.p, fine_slice_keys(j->wide, j->bbits - a.cbits),
                                j->stream));
  PK_CUDA(launch_scatter_coarse(a, (const uint32_t*)j->coff.p, two_pass ? j->tkeys.p : j->keys.p,
                                j->wide, j->stream));
  mark_end(j, ST_SCATTER);
  mark_begin(j, ST_SCATTER_FINE);
  if (two_pass) {
    if (hb < j->bbits) {
      PK_CUDA(cudaMemsetAsync(j->bstart.p, 0, sizeof(uint32_t) * (size_t)(B + 1), j->stream));
      PK_CUDA(cudaMemsetAsync(&j->d_sc->ticket_fcount, 0, sizeof(uint32_t), j->stream));
      PK_CUDA(launch_fine_count(j->tkeys.p, (const uint32_t*)j->cstart.p, (const uint32_t*)j->slice_start.p,
                                (uint32_t*)j->bstart.p, k, j->bbits, a.cbits, j->wide, &j->d_sc->ticket_fcount,
                                j->stream));
      PK_CUDA(launch_prefix((uint32_t*)j->bstart.p, B, j->stream));
    }
    PK_CUDA(cudaMemcpyAsync(j->fcur.p, j->bstart.p, sizeof(uint32_t) * (size_t)B, cudaMemcpyDeviceToDevice,
                            j->stream));
    PK_CUDA(cudaMemsetAsync(&j->d_sc->ticket_fine, 0, sizeof(uint32_t), j->stream));
    PK_CUDA(launch_scatter_fine(j->tkeys.p, (const uint32_t*)j->cstart.p, (const uint32_t*)j->slice_start.p,
                                (uint32_t*)j->fcur.p, j->keys.p, k, j->bbits, a.cbits, j->wide,
                                &j->d_sc->ticket_fine, N, &j->d_sc->err, j->stream));
  }
  mark_end(j, ST_SCATTER_FINE);
  return table_impl(j, N, t);
}

// Stage 5: bucketed keys -> (k-mer, count) table, resident.
static pk_status table_impl(pk_job* j, uint64_t N, int t) {
  const int k = j->params.k;
  const int B = 1 << j->bbits;
  mark_begin(j, ST_TABLE);
  // giant buckets are reduced chunk by chunk first (chunk items ahead of the buckets)
  PK_TRY(job_alloc(j, j->gfirst, sizeof(uint32_t) * (size_t)B));
  PK_TRY(job_alloc(j, j->gcount, sizeof(uint32_t) * (size_t)B));
  PK_TRY(job_alloc(j, j->gdone, sizeof(uint32_t) * (size_t)B));
  PK_TRY(job_alloc(j, j->chunk_bucket, sizeof(uint32_t) * (size_t)(N / kChunkKeys + 1)));
  PK_TRY(job_alloc(j, j->chunk_u, sizeof(uint32_t) * (size_t)(N / kChunkKeys + 1)));
  PK_CUDA(launch_giant_chunks((const uint32_t*)j->bstart.p, j->bbits, (uint32_t*)j->gfirst.p,
                              (uint32_t*)j->gcount.p, (uint32_t*)j->chunk_bucket.p, (uint32_t*)j->gdone.p,
                              j->d_sc, j->stream));
  PK_TRY(job_alloc(j, j->bsmall, sizeof(uint32_t) * kSmallCounts * (size_t)B));
  BucketArgs b{};
  b.keys = j->keys.p;
  b.bsmall = (uint32_t*)j->bsmall.p;
  b.gfirst = (const uint32_t*)j->gfirst.p;
  b.gcount = (const uint32_t*)j->gcount.p;
  b.chunk_bucket = (const uint32_t*)j->chunk_bucket.p;
  b.gdone = (uint32_t*)j->gdone.p;
  b.chunk_u = (uint32_t*)j->chunk_u.p;
  b.bstart = (const uint32_t*)j->bstart.p;
  b.tkeys = j->tkeys.p;
  b.tcounts = (uint32_t*)j->tcounts.p;
  b.tu = (uint32_t*)j->tu.p;
  b.hist = (unsigned long long*)j->hist.p;
  b.t = t;
  b.k = k;
  b.bbits = j->bbits;
  b.cap = N;
  b.spin_limit = (int)j->wait_limit;
  b.sc = j->d_sc;
  PK_CUDA(launch_bucket_table(b, j->wide, j->table_ctas > 0 ? j->table_ctas * thread_sms(j->ctx->sms) : 0, j->stream));
  mark_end(j, ST_TABLE);
  j->bsmall_valid = true;
  j->pieces = 1;
  j->stage = 1;
  return PK_OK;
}

pk_status pk_count_device(pk_job* j, const void* d_fasta, uint64_t n, const pk_params* p) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  PK_TRY(check_params(p));
  if (n && !d_fasta) return fail(PK_ERR_INVALID, "d_fasta is null");
  if (((uintptr_t)d_fasta & 15) != 0) return fail(PK_ERR_INVALID, "d_fasta must be 16-byte aligned");
  PK_TRY(set_device(j->ctx));
  for (int i = 0; i < ST_COUNT_; i++) j->ev_rec[i] = false;
  return count_impl(j, d_fasta, n, p);
}

pk_status pk::count_host(pk_job* j, const char* fasta, uint64_t n, const pk_params* p) {
  for (int i = 0; i < ST_COUNT_; i++) j->ev_rec[i] = false;
  // -b pieces: always (chunking 1), or when the whole input at once does not fit the
  // HBM budget or the 2^32-window limit (chunking 0)
  if (p->chunking == 1) return count_pieces(j, fasta, n, p, p->batch_kmers);
  pk_status s = job_alloc(j, j->fasta, (size_t)n + 16);
  if (s == PK_OK) {
    mark_begin(j, ST_H2D);
    if (n) PK_CUDA(cudaMemcpyAsync(j->fasta.p, fasta, n, cudaMemcpyHostToDevice, j->stream));
    mark_end(j, ST_H2D);
    s = count_impl(j, j->fasta.p, n, p);
  }
  if ((s == PK_ERR_NOMEM || s == PK_ERR_LIMIT) && p->chunking == 0 && n > 1) {
    PK_CUDA(cudaStreamSynchronize(j->stream));
    job_free_all(j);
    const uint64_t b = p->batch_kmers ? p->batch_kmers : 100000000ull;
    return count_pieces(j, fasta, n, p, std::min<uint64_t>(b, (n + 1) / 2));
  }
  return s;
}

pk_status pk_count(pk_job* j, const char* fasta, uint64_t n, const pk_params* p) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  PK_TRY(check_params(p));
  if (n && !fasta) return fail(PK_ERR_INVALID, "fasta is null");
  PK_TRY(set_device(j->ctx));
  return count_host(j, fasta, n, p);
}

// An existing (k-mer, count) table in place of counting: host rows ascending and
// unique, k-mers below 4^k.  The rows are laid out as the counting stages leave them
// (every bucket's rows contiguous), so cutoff and macro-nodes run unchanged.
pk_status pk_table_load(pk_job* j, const void* keys, const uint32_t* counts, uint64_t n, const pk_params* p) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  PK_TRY(check_params(p));
  if (n && (!keys || !counts)) return fail(PK_ERR_INVALID, "keys and counts must not be null");
  if (n >= 0xffffffffull) return fail(PK_ERR_LIMIT, "tables of 2^32-1 rows or more are not supported");
  j->bsmall_valid = false;  // the loaded table did not come from the table kernel
  const int k = p->k;
  const bool wide = k > 32;
  const uint64_t* kw = (const uint64_t*)keys;
  unsigned long long total = 0;
  for (uint64_t i = 0; i < n; i++) {
    const unsigned __int128 x = wide ? ((unsigned __int128)kw[2 * i + 1] << 64) | kw[2 * i]
                                     : (unsigned __int128)kw[i];
    if (k < 64 && (x >> (2 * k)) != 0) return fail(PK_ERR_INVALID, "row " + std::to_string(i) + " is not a k-mer");
    if (i) {
      const unsigned __int128 y = wide ? ((unsigned __int128)kw[2 * i - 1] << 64) | kw[2 * i - 2]
                                       : (unsigned __int128)kw[i - 1];
      if (!(y < x)) return fail(PK_ERR_INVALID, "rows must be ascending and unique (row " + std::to_string(i) + ")");
    }
    if (counts[i] == 0) return fail(PK_ERR_INVALID, "row " + std::to_string(i) + " has count 0");
    total += counts[i];
  }
  PK_TRY(set_device(j->ctx));
  for (int i = 0; i < ST_COUNT_; i++) j->ev_rec[i] = false;
  j->params = *p;
  j->wide = wide;
  j->F = 0;
  j->N = n;
  j->stage = 0;
  int bb = p->bucket_bits;
  if (!bb) {  // about 4000 rows per bucket
    bb = 2;
    while (bb < kMaxPartitionBits && (double)n / (double)(1u << bb) > 4000.0) bb++;
  }
  j->bbits = std::max(2, std::min(bb, std::min(kMaxPartitionBits, 2 * k - 2)));
  const int B = 1 << j->bbits;
  const size_t W = wide ? 16 : 8;
  PK_TRY(job_alloc(j, j->tkeys, W * (n ? n : 1)));
  PK_TRY(job_alloc(j, j->tcounts, 4 * (n ? n : 1)));
  PK_TRY(job_alloc(j, j->bstart, sizeof(uint32_t) * (B + 1)));
  PK_TRY(job_alloc(j, j->tu, sizeof(uint32_t) * (size_t)B));
  if (n) {
    PK_CUDA(cudaMemcpyAsync(j->tkeys.p, keys, W * n, cudaMemcpyHostToDevice, j->stream));
    PK_CUDA(cudaMemcpyAsync(j->tcounts.p, counts, 4 * n, cudaMemcpyHostToDevice, j->stream));
  }
  PK_CUDA(launch_table_bounds(j->tkeys.p, n, j->bbits, k, (uint32_t*)j->bstart.p, (uint32_t*)j->tu.p,
                              wide, j->stream));
  Scalars init{};
  memset(&init, 0, sizeof(init));
  init.n_unique = n;
  init.n_windows = total;
  *j->h_sc = init;
  PK_CUDA(cudaMemcpyAsync(j->d_sc, j->h_sc, sizeof(Scalars), cudaMemcpyHostToDevice, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  j->t_hist = 0;  // no histogram was fused into a counting pass
  j->dense_valid = false;
  j->stage = 1;
  return PK_OK;
}

pk_status pk::sync_scalars(pk_job* j) {
  PK_CUDA(cudaMemcpyAsync(j->h_sc, j->d_sc, sizeof(Scalars), cudaMemcpyDeviceToHost, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  const uint32_t err = j->h_sc->err;
  if (err & ERR_FORMAT) return fail(PK_ERR_FORMAT, "a FASTA record start is not '>'");
  if (err & ERR_LOOKBACK) return fail(PK_ERR_DEVICE, "a bounded look-back wait expired");
  if (err & ERR_BUCKET) return fail(PK_ERR_DEVICE, "a bucket could not be split to fit on chip");
  if (err & ERR_MN_CAPACITY) return fail(PK_ERR_DEVICE, "a macro-node segment exceeded on-chip capacity");
  if (err & ERR_BOUNDS) return fail(PK_ERR_DEVICE, "an index fell outside its buffer (write skipped)");
  return PK_OK;
}

pk_status pk_table_info(pk_job* j, uint64_t* u, uint64_t* w, uint64_t* r) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (j->stage < 1) return fail(PK_ERR_STATE, "no table: call pk_count first");
  PK_TRY(set_device(j->ctx));
  PK_TRY(sync_scalars(j));
  if (u) *u = j->h_sc->n_unique;
  if (w) *w = j->h_sc->n_windows;
  if (r) *r = j->h_sc->n_reads;
  return PK_OK;
}

// Dense (contiguous, ascending) copy of the resident sparse table, built on demand.
pk_status pk::dense_table(pk_job* j) {
  if (j->dense_valid) return PK_OK;
  const uint64_t u = j->h_sc->n_unique;
  const int B = 1 << j->bbits;
  const size_t W = j->wide ? 16 : 8;
  PK_TRY(job_alloc(j, j->doff, sizeof(uint32_t) * (B + 1)));
  PK_TRY(job_alloc(j, j->dkeys, W * (u ? u : 1)));
  PK_TRY(job_alloc(j, j->dcounts, 4 * (u ? u : 1)));
  PK_CUDA(launch_row_offsets((const uint32_t*)j->tu.p, (uint32_t*)j->doff.p, B, j->stream));
  PK_CUDA(launch_compact_rows(j->tkeys.p, (const uint32_t*)j->tcounts.p, (const uint32_t*)j->bstart.p,
                              (const uint32_t*)j->tu.p, (const uint32_t*)j->doff.p, B, j->wide,
                              j->dkeys.p, (uint32_t*)j->dcounts.p, nullptr, j->stream));
  j->dense_valid = true;
  return PK_OK;
}

pk_status pk_copy_table(pk_job* j, void* keys, uint32_t* counts, uint64_t cap) {
  uint64_t u = 0;
  PK_TRY(pk_table_info(j, &u, nullptr, nullptr));
  if (cap < u) return fail(PK_ERR_INVALID, "capacity smaller than the table");
  const size_t W = j->wide ? 16 : 8;
  PK_TRY(dense_table(j));
  if (u && keys) PK_CUDA(cudaMemcpyAsync(keys, j->dkeys.p, W * u, cudaMemcpyDeviceToHost, j->stream));
  if (u && counts)
    PK_CUDA(cudaMemcpyAsync(counts, j->dcounts.p, 4 * u, cudaMemcpyDeviceToHost, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  return PK_OK;
}

pk_status pk_copy_table_packed(pk_job* j, void* pairs, uint64_t cap) {
  uint64_t u = 0;
  PK_TRY(pk_table_info(j, &u, nullptr, nullptr));
  if (cap < u) return fail(PK_ERR_INVALID, "capacity smaller than the table");
  if (!u) return PK_OK;
  const size_t rec = j->wide ? 20 : 12;
  const int B = 1 << j->bbits;
  PK_TRY(job_alloc(j, j->doff, sizeof(uint32_t) * (B + 1)));
  PK_TRY(job_alloc(j, j->packed, rec * u));
  PK_CUDA(launch_row_offsets((const uint32_t*)j->tu.p, (uint32_t*)j->doff.p, B, j->stream));
  PK_CUDA(launch_compact_rows(j->tkeys.p, (const uint32_t*)j->tcounts.p, (const uint32_t*)j->bstart.p,
                              (const uint32_t*)j->tu.p, (const uint32_t*)j->doff.p, B, j->wide, nullptr,
                              nullptr, j->packed.p, j->stream));
  PK_CUDA(cudaMemcpyAsync(pairs, j->packed.p, rec * u, cudaMemcpyDeviceToHost, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  job_free(j, j->packed);
  return PK_OK;
}

pk_status pk_table_device(pk_job* j, const void** k, const uint32_t** c) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (j->stage < 1) return fail(PK_ERR_STATE, "no table: call pk_count first");
  PK_TRY(set_device(j->ctx));
  PK_TRY(sync_scalars(j));
  PK_TRY(dense_table(j));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  if (k) *k = j->dkeys.p;
  if (c) *c = (const uint32_t*)j->dcounts.p;
  return PK_OK;
}

// cutoff on the device; no host synchronisation
pk_status pk::cutoff_enqueue(pk_job* j, int t) {
  const unsigned long long* hist = (const unsigned long long*)j->hist.p;
  if (t != j->t_hist) {
    // histogram for a different -t than the one fused into counting
    PK_TRY(sync_scalars(j));
    PK_TRY(job_alloc(j, j->hist2, sizeof(unsigned long long) * (size_t)t));
    PK_CUDA(cudaMemsetAsync(j->hist2.p, 0, sizeof(unsigned long long) * (size_t)t, j->stream));
    PK_TRY(dense_table(j));
    PK_CUDA(launch_histogram((const uint32_t*)j->dcounts.p, j->h_sc->n_unique, t,
                             (unsigned long long*)j->hist2.p, j->stream));
    hist = (const unsigned long long*)j->hist2.p;
  }
  mark_begin(j, ST_CUTOFF);
  PK_CUDA(launch_cutoff(hist, t, j->d_sc, j->stream));
  mark_end(j, ST_CUTOFF);
  j->stage = 2;
  return PK_OK;
}

pk_status pk_cutoff(pk_job* j, int32_t t, uint32_t* cutoff, uint64_t* hist, uint64_t* kept) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (t < 1) return fail(PK_ERR_INVALID, "num_buckets must be >= 1");
  if (j->stage < 1) return fail(PK_ERR_STATE, "no table: call pk_count first");
  PK_TRY(set_device(j->ctx));
  PK_TRY(cutoff_enqueue(j, t));
  const void* hsrc = t == j->t_hist ? j->hist.p : j->hist2.p;
  if (hist) PK_CUDA(cudaMemcpyAsync(hist, hsrc, sizeof(uint64_t) * (size_t)t, cudaMemcpyDeviceToHost, j->stream));
  PK_TRY(sync_scalars(j));
  if (cutoff) *cutoff = j->h_sc->cutoff;
  if (kept) *kept = j->h_sc->n_kept;
  if (j->h_sc->n_kept == 0)
    return fail(PK_ERR_EMPTY, "no k-mer reaches the cutoff " + std::to_string(j->h_sc->cutoff) +
                                  "; macro-node construction cannot proceed");
  return PK_OK;
}

pk_status pk::mn_enqueue(pk_job* j, uint32_t min_count, uint64_t kept_bound) {
  const int B = 1 << j->bbits;
  const size_t W = j->wide ? 16 : 8;
  const uint64_t kcap = kept_bound ? kept_bound : 1;
  uint64_t cap = 2 * kept_bound;
  if (cap == 0) cap = 1;
  PK_TRY(job_alloc(j, j->kkeys, W * kcap));
  PK_TRY(job_alloc(j, j->kcounts, 4 * kcap));
  PK_TRY(job_alloc(j, j->kstart, sizeof(uint32_t) * B));
  PK_TRY(job_alloc(j, j->kcount, sizeof(uint32_t) * B));
  PK_TRY(job_alloc(j, j->ksub, sizeof(uint32_t) * 3 * (size_t)B));
  PK_TRY(job_alloc(j, j->flags_f, sizeof(unsigned long long) * B));
  PK_TRY(job_alloc(j, j->nkeys, W * cap));
  PK_TRY(job_alloc(j, j->nsuf, 16 * cap));
  PK_TRY(job_alloc(j, j->npre, 16 * cap));
  PK_TRY(job_alloc(j, j->flags_m, sizeof(unsigned long long) * B));
  PK_CUDA(cudaMemsetAsync(j->flags_f.p, 0, sizeof(unsigned long long) * B, j->stream));
  PK_CUDA(cudaMemsetAsync(j->flags_m.p, 0, sizeof(unsigned long long) * B, j->stream));
  PK_CUDA(cudaMemsetAsync(&j->d_sc->ticket_mn, 0, sizeof(uint32_t), j->stream));
  PK_CUDA(cudaMemsetAsync(&j->d_sc->ticket_filter, 0, sizeof(uint32_t), j->stream));
  PK_CUDA(cudaMemsetAsync(&j->d_sc->n_nodes, 0, sizeof(unsigned long long), j->stream));
  PK_CUDA(cudaMemsetAsync(&j->d_sc->n_kept_rows, 0, sizeof(unsigned long long), j->stream));
  if (min_count) PK_CUDA(cudaMemcpyAsync(&j->d_sc->cutoff, &min_count, sizeof(uint32_t), cudaMemcpyHostToDevice, j->stream));
  j->mn_cap = cap;
  FilterArgs f{};
  f.tkeys = j->tkeys.p;
  f.tcounts = (const uint32_t*)j->tcounts.p;
  f.bstart = (const uint32_t*)j->bstart.p;
  f.tu = (const uint32_t*)j->tu.p;
  f.flags = (unsigned long long*)j->flags_f.p;
  f.kkeys = j->kkeys.p;
  f.kcounts = (uint32_t*)j->kcounts.p;
  f.kstart = (uint32_t*)j->kstart.p;
  f.kcount = (uint32_t*)j->kcount.p;
  f.ksub = (uint32_t*)j->ksub.p;
  f.cap = kcap;
  f.trows = j->tcounts.bytes / sizeof(uint32_t);
  f.bsmall = j->bsmall_valid ? (const uint32_t*)j->bsmall.p : nullptr;
  f.k = j->params.k;
  f.bbits = j->bbits;
  f.spin_limit = (int)j->wait_limit;
  f.sc = j->d_sc;
  mark_begin(j, ST_FILTER);
  PK_CUDA(launch_filter_kept(f, j->wide, 0, j->stream));
  mark_end(j, ST_FILTER);
  MnArgs m{};
  m.kkeys = j->kkeys.p;
  m.kcounts = (const uint32_t*)j->kcounts.p;
  m.kstart = (const uint32_t*)j->kstart.p;
  m.kcount = (const uint32_t*)j->kcount.p;
  m.ksub = (const uint32_t*)j->ksub.p;
  m.flags = (unsigned long long*)j->flags_m.p;
  m.nkeys = j->nkeys.p;
  m.nsuf = (uint32_t*)j->nsuf.p;
  m.npre = (uint32_t*)j->npre.p;
  m.cap = cap;
  m.kcap = kcap;
  m.k = j->params.k;
  m.bbits = j->bbits;
  // node units of about 1000 kept rows: each unit merges up to 2V / units rows
  {
    const double units = std::max(1.0, 2.0 * (double)kept_bound / 1000.0);
    int ub = 0;
    while ((double)(1u << ub) < units && ub < 30) ub++;
    int level = (j->bbits - ub) / 2;
    if (level < 1) level = 0;
    if (j->params.mn_units > 0) level = j->params.mn_units - 1;
    if (2 * level > j->bbits) level = j->bbits / 2;
    m.level = level;
  }
  m.spin_limit = (int)j->wait_limit;
  m.withhold_unit = j->withhold_unit;
  m.sc = j->d_sc;
  mark_begin(j, ST_MN);
  PK_CUDA(launch_macro_nodes(m, j->wide, 0, j->stream));
  mark_end(j, ST_MN);
  j->stage = 3;
  j->wired = false;
  j->compacted = false;
  return PK_OK;
}

pk_status pk_build_macro_nodes(pk_job* j, uint32_t min_count, uint64_t* n_nodes) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (j->stage < 1 || (min_count == 0 && j->stage < 2))
    return fail(PK_ERR_STATE, "call pk_count and pk_cutoff (or pass min_count) first");
  PK_TRY(set_device(j->ctx));
  PK_TRY(sync_scalars(j));
  uint64_t bound = min_count ? j->h_sc->n_unique : j->h_sc->n_kept;
  if (bound == 0)
    return fail(PK_ERR_EMPTY, "no k-mer reaches the cutoff; macro-node construction cannot proceed");
  PK_TRY(mn_enqueue(j, min_count, bound));
  PK_TRY(sync_scalars(j));
  if (n_nodes) *n_nodes = j->h_sc->n_nodes;
  return PK_OK;
}

pk_status pk_copy_macro_nodes(pk_job* j, void* keys, uint32_t* suf, uint32_t* pre, uint64_t cap) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (j->stage < 3) return fail(PK_ERR_STATE, "no macro-nodes: call pk_build_macro_nodes first");
  PK_TRY(set_device(j->ctx));
  PK_TRY(sync_scalars(j));
  const uint64_t m = j->h_sc->n_nodes;
  if (cap < m) return fail(PK_ERR_INVALID, "capacity smaller than the node count");
  const size_t W = j->wide ? 16 : 8;
  if (m && keys) PK_CUDA(cudaMemcpyAsync(keys, j->nkeys.p, W * m, cudaMemcpyDeviceToHost, j->stream));
  if (m && suf) PK_CUDA(cudaMemcpyAsync(suf, j->nsuf.p, 16 * m, cudaMemcpyDeviceToHost, j->stream));
  if (m && pre) PK_CUDA(cudaMemcpyAsync(pre, j->npre.p, 16 * m, cudaMemcpyDeviceToHost, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  return PK_OK;
}

pk_status pk_macro_nodes_device(pk_job* j, const void** k, const uint32_t** s, const uint32_t** p) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (j->stage < 3) return fail(PK_ERR_STATE, "no macro-nodes: call pk_build_macro_nodes first");
  if (k) *k = j->nkeys.p;
  if (s) *s = (const uint32_t*)j->nsuf.p;
  if (p) *p = (const uint32_t*)j->npre.p;
  return PK_OK;
}

pk_status pk_wire_macro_nodes(pk_job* j, int32_t coverage) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (j->stage < 3) return fail(PK_ERR_STATE, "no macro-nodes: call pk_build_macro_nodes first");
  const int cov = coverage ? coverage : j->params.coverage;
  if (cov <= 0) return fail(PK_ERR_INVALID, "coverage must be >= 1");
  PK_TRY(set_device(j->ctx));
  PK_TRY(sync_scalars(j));
  const uint64_t m = j->h_sc->n_nodes;
  PK_TRY(job_alloc(j, j->wiring, sizeof(WireRow) * (m ? m : 1)));
  PK_CUDA(launch_wire(j->nsuf.p, j->npre.p, m, cov, (WireRow*)j->wiring.p, j->stream));
  j->wired = true;
  return PK_OK;
}

pk_status pk_copy_wiring(pk_job* j, pk_wiring* out, uint64_t cap) {
  if (!j) return fail(PK_ERR_INVALID, "job is null");
  if (!j->wired) return fail(PK_ERR_STATE, "no wiring: call pk_wire_macro_nodes first");
  PK_TRY(set_device(j->ctx));
  PK_TRY(sync_scalars(j));
  const uint64_t m = j->h_sc->n_nodes;
  if (cap < m) return fail(PK_ERR_INVALID, "capacity smaller than the node count");
  if (m && out) PK_CUDA(cudaMemcpyAsync(out, j->wiring.p, sizeof(pk_wiring) * m, cudaMemcpyDeviceToHost, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  return PK_OK;
}

pk_status pk_wiring_device(pk_job* j, const pk_wiring** d) {
  if (!j || !d) return fail(PK_ERR_INVALID, "null argument");
  if (!j->wired) return fail(PK_ERR_STATE, "no wiring: call pk_wire_macro_nodes first");
  *d = (const pk_wiring*)j->wiring.p;
  return PK_OK;
}

pk_status pk_summary_get(pk_job* j, pk_summary* o) {
  if (!j || !o) return fail(PK_ERR_INVALID, "null argument");
  PK_TRY(set_device(j->ctx));
  PK_TRY(sync_scalars(j));
  o->n_reads = j->h_sc->n_reads;
  o->n_windows = j->h_sc->n_windows;
  o->n_unique = j->stage >= 1 ? j->h_sc->n_unique : 0;
  o->n_kept = j->stage >= 2 ? j->h_sc->n_kept : 0;
  o->n_nodes = j->stage >= 3 ? j->h_sc->n_nodes : 0;
  o->cutoff = j->stage >= 2 ? j->h_sc->cutoff : 0;
  o->key_bytes = j->wide ? 16 : 8;
  return PK_OK;
}

static pk_status run_rest(pk_job* j, const pk_params* p, pk_summary* out) {
  PK_TRY(cutoff_enqueue(j, p->num_buckets));
  PK_TRY(sync_scalars(j));
  if (j->h_sc->n_kept == 0) {
    if (out) pk_summary_get(j, out);
    return fail(PK_ERR_EMPTY, "no k-mer reaches the cutoff " + std::to_string(j->h_sc->cutoff) +
                                  "; macro-node construction cannot proceed");
  }
  PK_TRY(mn_enqueue(j, 0, j->h_sc->n_kept));
  if (out) return pk_summary_get(j, out);
  return sync_scalars(j);
}

pk_status pk_run(pk_job* j, const char* fasta, uint64_t n, const pk_params* p, pk_summary* out) {
  PK_TRY(pk_count(j, fasta, n, p));
  return run_rest(j, p, out);
}

pk_status pk_run_device(pk_job* j, const void* d_fasta, uint64_t n, const pk_params* p, pk_summary* out) {
  PK_TRY(pk_count_device(j, d_fasta, n, p));
  return run_rest(j, p, out);
}

