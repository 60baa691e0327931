// Serving: independent count -> cutoff -> macro-node requests run by worker threads on
// one context, with continuous batching, size-aware scheduling and HBM-budget
// admission.
//
// Continuous batching: a worker takes the next request as soon as its previous one
// has finished, so requests of different sizes and k overlap on the GPU (one request's
// host-to-device copy and host synchronisations run while others' kernels execute).
//
// Scheduling.  Queued requests are not served first come, first served: a worker takes
// the request with the least estimated work (FASTA bytes, doubled for 128-bit keys), so
// a small request is never queued behind a large one.  A request that has waited longer
// than the aging bound goes first regardless of size, and while it does not fit the
// HBM budget others start only in the memory it leaves, so memory drains for it and
// large requests cannot starve.  Requests up to `small_bytes` are small: some workers
// (`reserved_small`) take only small requests, so a burst of large ones never occupies
// every worker, and small requests run on high-priority CUDA streams (the GPU's block
// scheduler starts their blocks ahead of the large requests' pending blocks).
//
// Admission keeps the sum of the running requests' footprint estimates plus the device
// memory of results kept on the device within the context's HBM budget; the budget is
// enforced exactly by the context's allocator, and a request that hits it anyway goes
// back to the queue and starts again after another request has finished.
//
// A request can be cancelled while queued (it ends at once) or while running (it ends
// at its next stage boundary).  A request submitted with keep_on_device hands its job
// -- the k-mer table and macro-nodes resident in HBM -- to the caller, who can run
// further stages on it (pk_copy_table, pk_compact, pk_walk, ...) until releasing it.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/pakman_gb300.h"
#include "pk_internal.h"
#include "pk_runtime.h"

namespace {

uint64_t now_ns() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

struct Request {
  uint64_t ticket = 0;
  pk_request req{};
  uint64_t footprint = 0;
  uint64_t cost = 0;         // estimated work: FASTA bytes, doubled for 128-bit keys
  bool small = false;
  uint64_t retry_after = 0;  // re-queued: start again only after this many completions
  bool cancel = false;       // cancellation asked while running
  pk_request_info info{};
  std::string error;
  // server-kept macro-node table (pinned host memory)
  void* own_keys = nullptr;
  uint32_t* own_suf = nullptr;
  uint32_t* own_pre = nullptr;
  // keep_on_device: the finished job, handed to the caller, and its device bytes
  pk_job* job = nullptr;
  uint64_t resident = 0;
  // worker wall time by phase: counting, cutoff, macro-nodes, copy-out, releasing the
  // job's buffers (added to the server's stats when the request finishes)
  uint64_t phase_ns[5] = {0, 0, 0, 0, 0};
};

}  // namespace

struct pk_server {
  pk_ctx* ctx = nullptr;
  uint64_t budget = 0;  // 0: no budget
  int workers = 0;
  pk_server_config cfg{};
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work;  // queue changed / admission freed / stop
  std::condition_variable cv_done;  // a request finished
  std::vector<Request*> queue;      // waiting requests, in submission order
  std::unordered_map<uint64_t, Request*> reqs;
  std::deque<uint64_t> done_q;      // finished requests not yet handed out by pk_next_done
  uint64_t next_ticket = 1;
  bool stop = false;
  int running = 0;
  uint64_t events = 0;  // requests finished and results released (re-queued requests wait for one)
  pk_server_stats st{};
  std::atomic<uint64_t> pin_ns{0};  // time spent page-locking new result blocks
  // idle jobs with streams of their own: a request kept on the device takes its
  // worker's job and the worker continues with one of these; a released resident
  // job is reset and comes back here (creating and destroying jobs page-locks and
  // frees memory, which can wait for the whole device)
  std::vector<pk_job*> spare;
  // SM partition (cfg.small_sms > 0): small requests on green context g_small's SMs,
  // the others on g_large's; the driver calls come through the runtime's entry-point
  // query, so the library does not link the driver library itself
  CUgreenCtx g_small = nullptr, g_large = nullptr;
  int sms_small = 0, sms_large = 0;
  PFN_cuGreenCtxStreamCreate_v12050 green_stream = nullptr;
  PFN_cuGreenCtxDestroy_v12040 green_destroy = nullptr;
};

namespace {

// k-mer windows in a FASTA buffer, estimated from its first 256 KiB: lines alternate
// header / sequence from the first '>', and a sequence line of L bytes holds L - k + 1
// windows.  The count is scaled to the whole buffer with 5 % to spare; a buffer whose
// later records are denser than its first ones still runs exactly, through the
// allocator's own budget check and a retry.  Without a complete record in the sample
// the bound N <= F (a window needs at least one byte) is used.
uint64_t estimate_windows(const pk_request& r) {
  const uint64_t F = r.fasta_bytes;
  const uint64_t S = std::min<uint64_t>(F, 256ull << 10);
  const char* b = r.fasta;
  uint64_t p = 0, w = 0, end = 0;
  while (p < S && b[p] != '>') p++;
  bool seq = false;
  while (p < S) {
    const void* q = memchr(b + p, '\n', (size_t)(S - p));
    if (!q) break;
    const uint64_t e = (uint64_t)(static_cast<const char*>(q) - b);
    if (seq && e - p >= (uint64_t)r.params.k) w += e - p - (uint64_t)r.params.k + 1;
    seq = !seq;
    p = e + 1;
    if (!seq) end = p;  // a record ends here
  }
  if (end == 0 || S == F) return end == 0 ? F : w;
  return std::min<uint64_t>(F, (uint64_t)((double)w / (double)end * (double)F * 1.05) + 1);
}

// Device bytes a request may need: the FASTA, two key arrays and the count array over
// N windows, kept rows and the macro-node arrays over V kept k-mers.  V, the k-mers at
// or above the cutoff, is taken as N / 12: read sets at 20x coverage or more keep about
// one k-mer per genome position, one in 14 to 55 windows at 30-80x.
uint64_t footprint(const pk_request& r) {
  const uint64_t F = r.fasta_bytes;
  const uint64_t W = r.params.k > 32 ? 16 : 8;
  const uint64_t N = r.fasta ? estimate_windows(r) : F;
  const uint64_t V = N / 12;
  const uint64_t fixed = 64ull << 20;  // per-bucket tables, histograms, look-back flags
  // FASTA, its packed units (10 bytes per 16), two key arrays and the counts, kept rows,
  // macro-nodes
  return F + F / 16 * 10 + N * (2 * W + 4) + V * (W + 4) + 2 * V * (W + 32) + fixed;
}

uint64_t cost_of(const pk_request& r) { return r.fasta_bytes * (r.params.k > 32 ? 2 : 1); }

// Pinned host blocks for server-kept results, recycled between requests and between
// servers of the process (page-locking new memory costs far more than the copy into it).
// Block sizes are rounded up to a power of two so blocks fit later requests of similar
// size; at most kPinnedCache bytes of free blocks are kept.
constexpr uint64_t kPinnedCache = 32ull << 30;
std::mutex g_block_mu;
std::unordered_map<void*, size_t> g_block_size;
std::vector<std::pair<size_t, void*>> g_pinned_free;
uint64_t g_pinned_free_bytes = 0;

void* pinned_get(pk_server* s, size_t bytes) {
  size_t sz = 4096;
  while (sz < bytes) sz <<= 1;
  {
    std::lock_guard<std::mutex> lk(g_block_mu);
    for (size_t i = 0; i < g_pinned_free.size(); i++)
      if (g_pinned_free[i].first == sz) {
        void* p = g_pinned_free[i].second;
        g_pinned_free[i] = g_pinned_free.back();
        g_pinned_free.pop_back();
        g_pinned_free_bytes -= sz;
        return p;
      }
  }
  const uint64_t t0 = now_ns();
  void* p = nullptr;
  if (cudaMallocHost(&p, sz) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_block_mu);
  g_block_size[p] = sz;
  s->pin_ns += now_ns() - t0;  // read under s->mu by the stats; a relaxed count is enough
  return p;
}

void pinned_put(pk_server*, void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_block_mu);
  const size_t sz = g_block_size[p];
  if (g_pinned_free_bytes + sz > kPinnedCache) {
    cudaFreeHost(p);
    g_block_size.erase(p);
    return;
  }
  g_pinned_free.emplace_back(sz, p);
  g_pinned_free_bytes += sz;
}

// called with s->mu held
bool fits(const pk_server* s, const Request* q, uint64_t reserve) {
  if (s->budget == 0) return true;
  return s->st.admitted_bytes + s->st.resident_bytes + reserve + q->footprint <= s->budget;
}

// The request a worker starts next, or null (called with s->mu held).  small_only:
// a worker reserved for small requests.
Request* pick(pk_server* s, bool small_only) {
  const uint64_t now = now_ns();
  const uint64_t done = s->events;
  const uint64_t aging = (uint64_t)s->cfg.aging_ms * 1000000ull;
  Request* aged = nullptr;
  for (Request* q : s->queue)
    if (now - q->info.submit_ns > aging && done >= q->retry_after) {
      aged = q;  // the queue is in submission order: the first is the oldest
      break;
    }
  uint64_t reserve = 0;
  if (aged) {
    const bool mine = !small_only || aged->small;
    if (mine && (s->running == 0 || fits(s, aged, 0))) return aged;
    // memory drains for it: meanwhile others start only in the memory it leaves
    if (!fits(s, aged, 0)) reserve = aged->footprint;
  }
  Request* best = nullptr;
  for (Request* q : s->queue) {
    if (small_only && !q->small) continue;
    if (done < q->retry_after) continue;
    if (!(s->running == 0 && !aged) && !fits(s, q, reserve)) continue;
    if (!best || q->cost < best->cost || (q->cost == best->cost && q->ticket < best->ticket)) best = q;
  }
  return best;
}

void remove_queued(pk_server* s, Request* q) {
  s->queue.erase(std::find(s->queue.begin(), s->queue.end(), q));
  s->st.queued = s->queue.size();
}

void finish(pk_server* s, Request* q, pk_status status, const pk_summary& sum, const std::string& err) {
  std::lock_guard<std::mutex> lk(s->mu);
  q->info.status = status;
  q->info.summary = sum;
  q->info.end_ns = now_ns();
  q->info.done = 1;
  q->error = err;
  s->running--;
  s->st.running = (uint64_t)s->running;
  s->st.admitted_bytes -= q->footprint;
  if (q->job) {
    s->st.resident_bytes += q->resident;
    s->st.resident_jobs++;
  }
  s->st.count_ns += q->phase_ns[0];
  s->st.cutoff_ns += q->phase_ns[1];
  s->st.mn_ns += q->phase_ns[2];
  s->st.copyout_ns += q->phase_ns[3];
  s->st.release_ns += q->phase_ns[4];
  if (status == PK_OK) s->st.completed++;
  else if (status == PK_ERR_CANCELLED) s->st.cancelled++;
  else s->st.failed++;
  s->events++;
  s->done_q.push_back(q->ticket);
  s->cv_done.notify_all();
  s->cv_work.notify_all();
}

bool cancelled(pk_server* s, Request* q) {
  std::lock_guard<std::mutex> lk(s->mu);
  return q->cancel;
}

void summary_of(const pk_job* j, pk_summary* o) {
  const pk::Scalars& h = *j->h_sc;
  o->n_reads = h.n_reads;
  o->n_windows = h.n_windows;
  o->n_unique = j->stage >= 1 ? h.n_unique : 0;
  o->n_kept = j->stage >= 2 ? h.n_kept : 0;
  o->n_nodes = j->stage >= 3 ? h.n_nodes : 0;
  o->cutoff = j->stage >= 2 ? h.cutoff : 0;
  o->key_bytes = j->wide ? 16 : 8;
}

// count -> cutoff -> macro-nodes of one request on `job` (the stages of pk_run, with one
// host synchronisation after the cutoff and one at the end), ending early when it is
// cancelled at a stage boundary
pk_status run_request(pk_server* s, Request* q, pk_job* job, pk_summary* sum) {
  const pk_params& p = q->req.params;
  const uint64_t t0 = now_ns();
  pk_status r = pk_count(job, q->req.fasta, q->req.fasta_bytes, &p);
  const uint64_t t1 = now_ns();
  q->phase_ns[0] += t1 - t0;
  if (r != PK_OK) return r;
  if (cancelled(s, q)) return pk::set_error(PK_ERR_CANCELLED, "cancelled after counting");
  PK_TRY(pk::cutoff_enqueue(job, p.num_buckets));
  PK_TRY(pk::sync_scalars(job));
  const uint64_t t2 = now_ns();
  q->phase_ns[1] += t2 - t1;
  summary_of(job, sum);
  if (job->h_sc->n_kept == 0)
    return pk::set_error(PK_ERR_EMPTY, "no k-mer reaches the cutoff " + std::to_string(job->h_sc->cutoff) +
                                           "; macro-node construction cannot proceed");
  if (cancelled(s, q)) return pk::set_error(PK_ERR_CANCELLED, "cancelled after the histogram cutoff");
  PK_TRY(pk::mn_enqueue(job, 0, job->h_sc->n_kept));
  PK_TRY(pk::sync_scalars(job));
  q->phase_ns[2] += now_ns() - t2;
  summary_of(job, sum);
  return PK_OK;
}

void worker_main(pk_server* s, bool small_only) {
  // two jobs: small requests on a high-priority stream, the rest on a low-priority one
  int least = 0, greatest = 0;
  cudaSetDevice(s->ctx->device);
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  cudaStream_t st_hi = nullptr, st_lo = nullptr;
  pk_status cs = PK_OK;
  std::string cs_msg;
  if (s->g_small) {
    // small requests on the small partition's SMs, the others on the rest
    if (s->green_stream(&st_hi, s->g_small, CU_STREAM_NON_BLOCKING, greatest) != CUDA_SUCCESS ||
        s->green_stream(&st_lo, s->g_large, CU_STREAM_NON_BLOCKING, least) != CUDA_SUCCESS) {
      cs = PK_ERR_CUDA;
      cs_msg = "a stream on an SM partition";
    }
  } else {
    cudaStreamCreateWithPriority(&st_hi, cudaStreamNonBlocking, greatest);
    cudaStreamCreateWithPriority(&st_lo, cudaStreamNonBlocking, least);
  }
  pk_job* job_hi = nullptr;
  pk_job* job_lo = nullptr;
  if (cs == PK_OK) cs = pk_job_create(s->ctx, st_hi, &job_hi);
  if (cs == PK_OK) cs = pk_job_create(s->ctx, st_lo, &job_lo);
  if (cs != PK_OK && cs_msg.empty()) cs_msg = pk_last_error();
  while (true) {
    Request* q = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] {
        if (s->stop) return true;
        q = s->queue.empty() ? nullptr : pick(s, small_only);
        return q != nullptr;
      });
      if (s->stop) break;
      remove_queued(s, q);
      s->running++;
      s->st.running = (uint64_t)s->running;
      s->st.admitted_bytes += q->footprint;
      const uint64_t occ = s->st.admitted_bytes + s->st.resident_bytes;
      if (occ > s->st.peak_admitted_bytes) s->st.peak_admitted_bytes = occ;
      if (q->info.start_ns == 0) q->info.start_ns = now_ns();
      q->info.attempts++;
    }
    pk_summary sum{};
    if (cs != PK_OK) {
      finish(s, q, cs, sum, "worker could not create its jobs: " + cs_msg);
      continue;
    }
    pk_job*& job = q->small ? job_hi : job_lo;
    // grids sized for the partition the request runs on
    pk::set_thread_sms(s->g_small ? (q->small ? s->sms_small : s->sms_large) : 0);
    pk_status r = run_request(s, q, job, &sum);
    std::string err = r == PK_OK ? std::string() : std::string(pk_last_error());
    if (r == PK_ERR_NOMEM) {
      pk_job_reset(job);
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->running > 1 || s->st.resident_jobs > 0) {
        // others hold memory: back to the queue, started again once another request
        // has finished
        s->running--;
        s->st.running = (uint64_t)s->running;
        s->st.admitted_bytes -= q->footprint;
        s->st.requeued++;
        q->retry_after = s->events + 1;
        // back in submission order, so it keeps its age
        auto at = std::lower_bound(s->queue.begin(), s->queue.end(), q,
                                   [](const Request* a, const Request* b) { return a->ticket < b->ticket; });
        s->queue.insert(at, q);
        s->st.queued = s->queue.size();
        continue;
      }
    }
    const uint64_t t_copy = now_ns();
    if (r == PK_OK) {
      const uint64_t m = sum.n_nodes;
      const uint64_t W = q->req.params.k > 32 ? 16 : 8;
      if (q->req.mn_keys || q->req.mn_suffix || q->req.mn_prefix) {
        if (!q->req.mn_keys || !q->req.mn_suffix || !q->req.mn_prefix) {
          r = PK_ERR_INVALID;
          err = "mn_keys, mn_suffix and mn_prefix must all be set or all be NULL";
        } else if (m > q->req.mn_capacity) {
          r = PK_ERR_LIMIT;
          err = "macro-node table has " + std::to_string(m) + " rows, capacity " +
                std::to_string(q->req.mn_capacity);
        } else {
          r = pk_copy_macro_nodes(job, q->req.mn_keys, q->req.mn_suffix, q->req.mn_prefix, m);
          if (r != PK_OK) err = pk_last_error();
        }
      } else if (!q->req.keep_on_device) {
        const size_t rows = m ? m : 1;
        q->own_keys = pinned_get(s, rows * W);
        q->own_suf = (uint32_t*)pinned_get(s, rows * 16);
        q->own_pre = (uint32_t*)pinned_get(s, rows * 16);
        if (!q->own_keys || !q->own_suf || !q->own_pre) {
          cudaGetLastError();
          r = PK_ERR_NOMEM;
          err = "pinned host memory for the macro-node table";
        } else {
          r = pk_copy_macro_nodes(job, q->own_keys, q->own_suf, q->own_pre, m);
          if (r != PK_OK) err = pk_last_error();
        }
      }
    }
    if (r == PK_OK && q->req.keep_on_device) {
      // the finished job goes to the request (its work is complete) on the stream of
      // a spare job, which takes the worker's stream and the worker's place
      pk_job* fresh = nullptr;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        if (!s->spare.empty()) {
          fresh = s->spare.back();
          s->spare.pop_back();
        }
      }
      if (fresh || pk_job_create(s->ctx, nullptr, &fresh) == PK_OK) {
        std::swap(job->stream, fresh->stream);
        std::swap(job->own_stream, fresh->own_stream);
        pk_job_memory(job, &q->resident);
        q->job = job;
        job = fresh;
      } else {
        cudaGetLastError();
        r = PK_ERR_NOMEM;
        err = "a job for the next request";
      }
    }
    const uint64_t t_reset = now_ns();
    q->phase_ns[3] += t_reset - t_copy;
    // the job's device buffers go back to the context's pool, so the budget
    // accounting follows the running jobs (and the results kept on the device) only
    if (job != q->job) pk_job_reset(job);
    q->phase_ns[4] += now_ns() - t_reset;
    finish(s, q, r, sum, err);
  }
  if (job_hi) pk_job_destroy(job_hi);
  if (job_lo) pk_job_destroy(job_lo);
  if (st_hi) cudaStreamDestroy(st_hi);
  if (st_lo) cudaStreamDestroy(st_lo);
}

// called with s->mu held
void free_request(pk_server* s, Request* q) {
  pinned_put(s, q->own_keys);
  pinned_put(s, q->own_suf);
  pinned_put(s, q->own_pre);
  if (q->job) {
    // its device buffers go back to the context's pool; the job itself is kept for
    // the next request kept on the device
    if (!s->stop && s->spare.size() < (size_t)(2 * s->workers) && pk_job_reset(q->job) == PK_OK)
      s->spare.push_back(q->job);
    else
      pk_job_destroy(q->job);
    s->st.resident_bytes -= q->resident;
    s->st.resident_jobs--;
  }
  delete q;
}

Request* find(pk_server* s, uint64_t ticket) {
  auto it = s->reqs.find(ticket);
  return it == s->reqs.end() ? nullptr : it->second;
}

}  // namespace

namespace {

template <typename F>
bool driver_fn(const char* name, F* fn) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12050, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !p) {
    cudaGetLastError();
    return false;
  }
  *fn = reinterpret_cast<F>(p);
  return true;
}

// Splits the device into `small_sms` SMs (rounded up by the driver) for small requests
// and the rest for the others, one green context each.
pk_status make_partition(pk_server* s, int small_sms) {
  PFN_cuDeviceGet_v2000 device_get = nullptr;
  PFN_cuDeviceGetDevResource_v12040 get_resource = nullptr;
  PFN_cuDevSmResourceSplitByCount_v12040 split = nullptr;
  PFN_cuDevResourceGenerateDesc_v12040 make_desc = nullptr;
  PFN_cuGreenCtxCreate_v12040 green_create = nullptr;
  if (!driver_fn("cuDeviceGet", &device_get) || !driver_fn("cuDeviceGetDevResource", &get_resource) ||
      !driver_fn("cuDevSmResourceSplitByCount", &split) || !driver_fn("cuDevResourceGenerateDesc", &make_desc) ||
      !driver_fn("cuGreenCtxCreate", &green_create) || !driver_fn("cuGreenCtxDestroy", &s->green_destroy) ||
      !driver_fn("cuGreenCtxStreamCreate", &s->green_stream))
    return pk::set_error(PK_ERR_CUDA, "SM partitions: the driver has no green-context entry points");
  CUdevice dev = 0;
  CUdevResource all{}, part{}, rest{};
  unsigned int groups = 1;
  CUdevResourceDesc d_small = nullptr, d_large = nullptr;
  CUresult r = device_get(&dev, s->ctx->device);
  if (r == CUDA_SUCCESS) r = get_resource(dev, &all, CU_DEV_RESOURCE_TYPE_SM);
  if (r == CUDA_SUCCESS && (unsigned)small_sms >= all.sm.smCount)
    return pk::set_error(PK_ERR_INVALID, "small_sms must be below the device's " +
                                             std::to_string(all.sm.smCount) + " SMs");
  if (r == CUDA_SUCCESS) r = split(&part, &groups, &all, &rest, 0, (unsigned)small_sms);
  if (r == CUDA_SUCCESS && (groups != 1 || rest.sm.smCount == 0)) r = CUDA_ERROR_INVALID_VALUE;
  if (r == CUDA_SUCCESS) r = make_desc(&d_small, &part, 1);
  if (r == CUDA_SUCCESS) r = make_desc(&d_large, &rest, 1);
  if (r == CUDA_SUCCESS) r = green_create(&s->g_small, d_small, dev, CU_GREEN_CTX_DEFAULT_STREAM);
  if (r == CUDA_SUCCESS) r = green_create(&s->g_large, d_large, dev, CU_GREEN_CTX_DEFAULT_STREAM);
  if (r != CUDA_SUCCESS) {
    if (s->g_small) s->green_destroy(s->g_small);
    if (s->g_large) s->green_destroy(s->g_large);
    s->g_small = s->g_large = nullptr;
    return pk::set_error(PK_ERR_CUDA, "SM partitions: driver error " + std::to_string((int)r));
  }
  s->sms_small = (int)part.sm.smCount;
  s->sms_large = (int)rest.sm.smCount;
  return PK_OK;
}

}  // namespace

extern "C" {

uint64_t pk_request_footprint(const pk_request* req) { return req ? footprint(*req) : 0; }

void pk_server_config_default(pk_server_config* c, int32_t workers) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->small_bytes = 32ull << 20;
  c->reserved_small = workers >= 2 ? (workers + 7) / 8 : 0;
  c->aging_ms = 2000;
}

pk_status pk_server_create_config(pk_ctx* ctx, int32_t workers, const pk_server_config* cfg, pk_server** out) {
  if (!ctx || !out) return pk::set_error(PK_ERR_INVALID, "ctx and out must not be null");
  if (workers < 1 || workers > 64) return pk::set_error(PK_ERR_INVALID, "workers must be in 1..64");
  pk_server_config c;
  pk_server_config_default(&c, workers);
  if (cfg) c = *cfg;
  if (c.reserved_small < 0 || c.reserved_small >= workers)
    return pk::set_error(PK_ERR_INVALID, "reserved_small must be in 0..workers-1");
  if (c.small_sms < 0) return pk::set_error(PK_ERR_INVALID, "small_sms must be >= 0");
  uint64_t used = 0, budget = 0;
  pk_status st = pk_ctx_memory(ctx, &used, &budget);
  if (st != PK_OK) return st;
  pk_server* s = new pk_server();
  s->ctx = ctx;
  s->budget = budget;
  s->workers = workers;
  s->cfg = c;
  if (c.small_sms > 0) {
    pk::set_device(ctx);
    const pk_status ps = make_partition(s, c.small_sms);
    if (ps != PK_OK) {
      delete s;
      return ps;
    }
  }
  for (int i = 0; i < workers; i++) s->threads.emplace_back(worker_main, s, i < c.reserved_small);
  *out = s;
  return PK_OK;
}

pk_status pk_server_create(pk_ctx* ctx, int32_t workers, pk_server** out) {
  return pk_server_create_config(ctx, workers, nullptr, out);
}

void pk_server_destroy(pk_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (auto& kv : s->reqs) kv.second->cancel = true;
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
  for (auto& t : s->threads) t.join();
  for (auto& kv : s->reqs) free_request(s, kv.second);
  for (pk_job* j : s->spare) pk_job_destroy(j);
  if (s->g_small) s->green_destroy(s->g_small);
  if (s->g_large) s->green_destroy(s->g_large);
  delete s;
}

pk_status pk_submit(pk_server* s, const pk_request* req, uint64_t* ticket) {
  if (!s || !req || !ticket) return pk::set_error(PK_ERR_INVALID, "server, request and ticket must not be null");
  if (!req->fasta && req->fasta_bytes) return pk::set_error(PK_ERR_INVALID, "fasta is null");
  Request* q = new Request();
  q->req = *req;
  q->footprint = footprint(*req);
  q->cost = cost_of(*req);
  q->info.submit_ns = now_ns();
  q->info.status = PK_ERR_BUSY;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) {
    delete q;
    return pk::set_error(PK_ERR_STATE, "server is shutting down");
  }
  q->small = q->cost <= s->cfg.small_bytes;
  q->ticket = s->next_ticket++;
  s->reqs[q->ticket] = q;
  s->queue.push_back(q);
  s->st.submitted++;
  s->st.queued = s->queue.size();
  *ticket = q->ticket;
  s->cv_work.notify_all();
  return PK_OK;
}

pk_status pk_cancel(pk_server* s, uint64_t ticket) {
  if (!s) return pk::set_error(PK_ERR_INVALID, "server is null");
  std::lock_guard<std::mutex> lk(s->mu);
  Request* q = find(s, ticket);
  if (!q) return pk::set_error(PK_ERR_INVALID, "unknown ticket");
  if (q->info.done) return pk::set_error(PK_ERR_STATE, "the request has finished");
  if (std::find(s->queue.begin(), s->queue.end(), q) != s->queue.end()) {
    remove_queued(s, q);
    q->info.status = PK_ERR_CANCELLED;
    q->info.done = 1;
    q->info.end_ns = now_ns();
    q->error = "cancelled while queued";
    s->st.cancelled++;
    s->done_q.push_back(q->ticket);
    s->cv_done.notify_all();
    s->cv_work.notify_all();
    return PK_OK;
  }
  q->cancel = true;  // running: it ends at its next stage boundary
  return PK_OK;
}

static pk_status report(const Request* q, pk_request_info* info) {
  if (info) *info = q->info;
  if (q->info.done && q->info.status != PK_OK) pk::set_error(q->info.status, q->error);
  return PK_OK;
}

pk_status pk_poll(pk_server* s, uint64_t ticket, pk_request_info* info) {
  if (!s) return pk::set_error(PK_ERR_INVALID, "server is null");
  std::lock_guard<std::mutex> lk(s->mu);
  Request* q = find(s, ticket);
  if (!q) return pk::set_error(PK_ERR_INVALID, "unknown ticket");
  return report(q, info);
}

pk_status pk_next_done(pk_server* s, int64_t timeout_ms, uint64_t* ticket, pk_request_info* info) {
  if (!s || !ticket) return pk::set_error(PK_ERR_INVALID, "server and ticket must not be null");
  std::unique_lock<std::mutex> lk(s->mu);
  auto ready = [&] {
    while (!s->done_q.empty() && !s->reqs.count(s->done_q.front())) s->done_q.pop_front();  // released
    return !s->done_q.empty() || s->stop;
  };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, ready);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    return pk::set_error(PK_ERR_BUSY, "no request finished in time");
  }
  if (s->done_q.empty()) return pk::set_error(PK_ERR_STATE, "server is shutting down");
  *ticket = s->done_q.front();
  s->done_q.pop_front();
  Request* q = find(s, *ticket);
  if (info) *info = q->info;
  return PK_OK;
}

pk_status pk_wait(pk_server* s, uint64_t ticket, int64_t timeout_ms, pk_request_info* info) {
  if (!s) return pk::set_error(PK_ERR_INVALID, "server is null");
  std::unique_lock<std::mutex> lk(s->mu);
  Request* q = find(s, ticket);
  if (!q) return pk::set_error(PK_ERR_INVALID, "unknown ticket");
  auto ready = [&] { return q->info.done != 0 || s->stop; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, ready);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    if (info) *info = q->info;
    return pk::set_error(PK_ERR_BUSY, "request still queued or running");
  }
  return report(q, info);
}

pk_status pk_result_get(pk_server* s, uint64_t ticket, const void** keys, const uint32_t** suffix,
                        const uint32_t** prefix, uint64_t* n_nodes) {
  if (!s) return pk::set_error(PK_ERR_INVALID, "server is null");
  std::lock_guard<std::mutex> lk(s->mu);
  Request* q = find(s, ticket);
  if (!q) return pk::set_error(PK_ERR_INVALID, "unknown ticket");
  if (!q->info.done) return pk::set_error(PK_ERR_BUSY, "request still queued or running");
  if (q->info.status != PK_OK) return pk::set_error(q->info.status, q->error);
  if (!q->own_keys) return pk::set_error(PK_ERR_STATE, "the result is not kept in host memory by the server");
  if (keys) *keys = q->own_keys;
  if (suffix) *suffix = q->own_suf;
  if (prefix) *prefix = q->own_pre;
  if (n_nodes) *n_nodes = q->info.summary.n_nodes;
  return PK_OK;
}

pk_status pk_result_job(pk_server* s, uint64_t ticket, pk_job** job) {
  if (!s || !job) return pk::set_error(PK_ERR_INVALID, "server and job must not be null");
  std::lock_guard<std::mutex> lk(s->mu);
  Request* q = find(s, ticket);
  if (!q) return pk::set_error(PK_ERR_INVALID, "unknown ticket");
  if (!q->info.done) return pk::set_error(PK_ERR_BUSY, "request still queued or running");
  if (q->info.status != PK_OK) return pk::set_error(q->info.status, q->error);
  if (!q->job) return pk::set_error(PK_ERR_STATE, "the request was not submitted with keep_on_device");
  *job = q->job;
  return PK_OK;
}

pk_status pk_result_release(pk_server* s, uint64_t ticket) {
  if (!s) return pk::set_error(PK_ERR_INVALID, "server is null");
  std::lock_guard<std::mutex> lk(s->mu);
  Request* q = find(s, ticket);
  if (!q) return pk::set_error(PK_ERR_INVALID, "unknown ticket");
  if (!q->info.done) return pk::set_error(PK_ERR_BUSY, "request still queued or running");
  s->reqs.erase(ticket);
  const bool had_job = q->job != nullptr;
  free_request(s, q);
  if (had_job) s->events++;
  s->cv_work.notify_all();  // released device memory may admit a waiting request
  return PK_OK;
}

pk_status pk_server_get_stats(pk_server* s, pk_server_stats* out) {
  if (!s || !out) return pk::set_error(PK_ERR_INVALID, "server and out must not be null");
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->st;
  out->pin_ns = s->pin_ns.load();
  return PK_OK;
}

pk_status pk_server_partition(pk_server* s, int32_t* small_sms, int32_t* large_sms) {
  if (!s || !small_sms || !large_sms) return pk::set_error(PK_ERR_INVALID, "null argument");
  *small_sms = s->g_small ? s->sms_small : s->ctx->sms;
  *large_sms = s->g_small ? s->sms_large : s->ctx->sms;
  return PK_OK;
}

void pk_server_cache_release(void) {
  std::lock_guard<std::mutex> lk(g_block_mu);
  for (auto& b : g_pinned_free) {
    cudaFreeHost(b.second);
    g_block_size.erase(b.second);
  }
  g_pinned_free.clear();
  g_pinned_free_bytes = 0;
}

}  // extern "C"
