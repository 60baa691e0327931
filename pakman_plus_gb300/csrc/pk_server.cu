// Serving: a FIFO of independent count -> cutoff -> macro-node requests executed by
// worker threads, each owning one pk_job (and its CUDA stream) on a shared context.
//
// Continuous batching: a worker takes the next request as soon as its previous one
// has finished, so jobs of different sizes and k overlap on the GPU (one job's host
// to device copy and host synchronisations run while another job's kernels execute).
// Admission control keeps the sum of the running jobs' footprint estimates within the
// context's HBM budget; the budget itself is enforced exactly by the context's
// allocator, and a job that hits it anyway goes back to the head of the queue.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <time.h>

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
  uint64_t retry_after = 0;  // re-queued: start again only after this many completions
  pk_request_info info{};
  std::string error;
  // server-kept macro-node table (pinned host memory)
  void* own_keys = nullptr;
  uint32_t* own_suf = nullptr;
  uint32_t* own_pre = nullptr;
};

}  // namespace

struct pk_server {
  pk_ctx* ctx = nullptr;
  uint64_t budget = 0;  // 0: no budget
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work;  // queue changed / admission freed / stop
  std::condition_variable cv_done;  // a request finished
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, Request*> reqs;
  uint64_t next_ticket = 1;
  bool stop = false;
  int running = 0;
  pk_server_stats st{};
  std::vector<std::pair<size_t, void*>> pinned_free;  // pinned host blocks for kept results
};

namespace {

// Device bytes a request may need: the FASTA, two key arrays and the count array
// over N windows, kept rows and the macro-node arrays over V kept k-mers.  N is
// bounded by the FASTA size (a window needs at least one byte); V, the k-mers at or
// above the cutoff, is taken as N / 8 (a read set whose kept k-mers exceed that still
// runs exactly, through the allocator's own budget check and a retry).
uint64_t footprint(const pk_request& r) {
  const uint64_t F = r.fasta_bytes;
  const uint64_t W = r.params.k > 32 ? 16 : 8;
  const uint64_t N = F;
  const uint64_t V = N / 8;
  const uint64_t fixed = 64ull << 20;  // per-bucket tables, histograms, look-back flags
  return F + N * (2 * W + 4) + V * (W + 4) + 2 * V * (W + 32) + fixed;
}

// Pinned host blocks for server-kept results, recycled between requests (page-locking
// new memory costs far more than the copy into it).  Block sizes are rounded up to a
// power of two so blocks fit later requests of similar size.
std::mutex g_block_mu;
std::unordered_map<void*, size_t> g_block_size;

void* pinned_get(pk_server* s, size_t bytes) {
  size_t sz = 4096;
  while (sz < bytes) sz <<= 1;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (size_t i = 0; i < s->pinned_free.size(); i++)
      if (s->pinned_free[i].first == sz) {
        void* p = s->pinned_free[i].second;
        s->pinned_free[i] = s->pinned_free.back();
        s->pinned_free.pop_back();
        return p;
      }
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, sz) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_block_mu);
  g_block_size[p] = sz;
  return p;
}

// called with s->mu held
void pinned_put(pk_server* s, void* p) {
  if (!p) return;
  size_t sz;
  {
    std::lock_guard<std::mutex> lk(g_block_mu);
    sz = g_block_size[p];
  }
  s->pinned_free.emplace_back(sz, p);
}

void pinned_release_all(pk_server* s) {
  for (auto& b : s->pinned_free) {
    cudaFreeHost(b.second);
    std::lock_guard<std::mutex> lk(g_block_mu);
    g_block_size.erase(b.second);
  }
  s->pinned_free.clear();
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
  if (status == PK_OK) s->st.completed++; else s->st.failed++;
  s->cv_done.notify_all();
  s->cv_work.notify_all();
}

void worker_main(pk_server* s) {
  pk_job* job = nullptr;
  pk_status cs = pk_job_create(s->ctx, nullptr, &job);
  while (true) {
    Request* q = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // FIFO: only the head may start, and only when its estimate fits the budget
      // (or nothing else is running, so an oversized job still gets its chance)
      s->cv_work.wait(lk, [&] {
        if (s->stop) return true;
        if (s->queue.empty()) return false;
        const Request* h = s->queue.front();
        if (s->running == 0) return true;
        if (s->st.completed + s->st.failed < h->retry_after) return false;
        return s->budget == 0 || s->st.admitted_bytes + h->footprint <= s->budget;
      });
      if (s->stop) break;
      q = s->queue.front();
      s->queue.pop_front();
      s->running++;
      s->st.running = (uint64_t)s->running;
      s->st.queued = s->queue.size();
      s->st.admitted_bytes += q->footprint;
      if (s->st.admitted_bytes > s->st.peak_admitted_bytes) s->st.peak_admitted_bytes = s->st.admitted_bytes;
      if (q->info.start_ns == 0) q->info.start_ns = now_ns();
      q->info.attempts++;
    }
    pk_summary sum{};
    if (cs != PK_OK) {
      finish(s, q, cs, sum, "worker could not create its job: " + std::string(pk_last_error()));
      continue;
    }
    pk_status r = pk_run(job, q->req.fasta, q->req.fasta_bytes, &q->req.params, &sum);
    std::string err = r == PK_OK ? std::string() : std::string(pk_last_error());
    if (r == PK_ERR_NOMEM) {
      pk_job_reset(job);
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->running > 1) {
        // others hold memory: back to the head of the queue, started again once
        // another job has finished
        s->running--;
        s->st.running = (uint64_t)s->running;
        s->st.admitted_bytes -= q->footprint;
        s->st.requeued++;
        q->retry_after = s->st.completed + s->st.failed + 1;
        s->queue.push_front(q);
        s->st.queued = s->queue.size();
        continue;
      }
    }
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
      } else {
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
    // the job's device buffers go back to the context's pool, so the budget
    // accounting follows the running jobs only
    pk_job_reset(job);
    finish(s, q, r, sum, err);
  }
  if (job) pk_job_destroy(job);
}

// called with s->mu held
void free_request(pk_server* s, Request* q) {
  pinned_put(s, q->own_keys);
  pinned_put(s, q->own_suf);
  pinned_put(s, q->own_pre);
  delete q;
}

Request* find(pk_server* s, uint64_t ticket) {
  auto it = s->reqs.find(ticket);
  return it == s->reqs.end() ? nullptr : it->second;
}

}  // namespace

extern "C" {

uint64_t pk_request_footprint(const pk_request* req) { return req ? footprint(*req) : 0; }

pk_status pk_server_create(pk_ctx* ctx, int32_t workers, pk_server** out) {
  if (!ctx || !out) return pk::set_error(PK_ERR_INVALID, "ctx and out must not be null");
  if (workers < 1 || workers > 64) return pk::set_error(PK_ERR_INVALID, "workers must be in 1..64");
  uint64_t used = 0, budget = 0;
  pk_status st = pk_ctx_memory(ctx, &used, &budget);
  if (st != PK_OK) return st;
  pk_server* s = new pk_server();
  s->ctx = ctx;
  s->budget = budget;
  for (int i = 0; i < workers; i++) s->threads.emplace_back(worker_main, s);
  *out = s;
  return PK_OK;
}

void pk_server_destroy(pk_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
  for (auto& t : s->threads) t.join();
  for (auto& kv : s->reqs) free_request(s, kv.second);
  pinned_release_all(s);
  delete s;
}

pk_status pk_submit(pk_server* s, const pk_request* req, uint64_t* ticket) {
  if (!s || !req || !ticket) return pk::set_error(PK_ERR_INVALID, "server, request and ticket must not be null");
  if (!req->fasta && req->fasta_bytes) return pk::set_error(PK_ERR_INVALID, "fasta is null");
  Request* q = new Request();
  q->req = *req;
  q->footprint = footprint(*req);
  q->info.submit_ns = now_ns();
  q->info.status = PK_ERR_BUSY;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) {
    delete q;
    return pk::set_error(PK_ERR_STATE, "server is shutting down");
  }
  q->ticket = s->next_ticket++;
  s->reqs[q->ticket] = q;
  s->queue.push_back(q);
  s->st.submitted++;
  s->st.queued = s->queue.size();
  *ticket = q->ticket;
  s->cv_work.notify_all();
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
  if (!q->own_keys) return pk::set_error(PK_ERR_STATE, "the result was written to the caller's buffers");
  if (keys) *keys = q->own_keys;
  if (suffix) *suffix = q->own_suf;
  if (prefix) *prefix = q->own_pre;
  if (n_nodes) *n_nodes = q->info.summary.n_nodes;
  return PK_OK;
}

pk_status pk_result_release(pk_server* s, uint64_t ticket) {
  if (!s) return pk::set_error(PK_ERR_INVALID, "server is null");
  std::lock_guard<std::mutex> lk(s->mu);
  Request* q = find(s, ticket);
  if (!q) return pk::set_error(PK_ERR_INVALID, "unknown ticket");
  if (!q->info.done) return pk::set_error(PK_ERR_BUSY, "request still queued or running");
  s->reqs.erase(ticket);
  free_request(s, q);
  return PK_OK;
}

pk_status pk_server_get_stats(pk_server* s, pk_server_stats* out) {
  if (!s || !out) return pk::set_error(PK_ERR_INVALID, "server and out must not be null");
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->st;
  return PK_OK;
}

}  // extern "C"
