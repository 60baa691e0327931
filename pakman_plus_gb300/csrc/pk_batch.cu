// Batching: the count -> cutoff -> macro-node path of many independent read sets
// captured into one CUDA graph and replayed with one launch.
//
// Sets are dealt to `branches` graph branches (largest first, each to the branch with
// the least bytes so far); a branch owns one job whose buffers are sized for its
// largest set, so the branch's sets run one after another in the same memory, while
// the branches run side by side.  Inside the graph nothing waits for the host: a
// set's window count is bounded by its byte count and its kept k-mers by 1/8 of that,
// and every kernel checks those bounds (an overrun raises the set's error bits and
// skips the write).  A short pair of kernels after each set reserves its rows in the
// batch's macro-node table and copies them there.  Sets whose run failed inside the
// graph, or did not fit a bound, are run again on their own afterwards, so every
// result is the set's own.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <string>
#include <vector>

#include "../../include/pakman_gb300.h"
#include "pk_internal.h"
#include "pk_runtime.h"

using namespace pk;

namespace {

constexpr uint64_t kAlign = 256;  // set offsets in the device input buffer

struct SetPlan {
  uint64_t off = 0;      // byte offset of the set in the device input
  uint64_t bytes = 0;
  pk_params params{};
  int branch = 0;
  bool in_graph = true;  // false: too large for the graph bounds, run on its own
  const void* host = nullptr;  // the set's FASTA in host memory
};

struct HostTable {      // rows of sets run on their own
  std::vector<uint64_t> keys;  // key words
  std::vector<uint32_t> suf, pre;
  uint64_t rows = 0;
};

int size_class(uint64_t bytes) { return bytes ? 63 - __builtin_clzll(bytes) : 0; }

// What the autotuner picks for a size class: the partition digits (radix width), the
// counting/scatter chunk size (a multiple of one chunk per SM: fewer, longer chunks leave
// SMs to the other graph branches) and the table kernel's CTAs per SM (how the buckets are
// dealt to CTAs).
struct Shape {
  int digits = 0;
  int chunk_mult = 1;
  int table_ctas = 2;
};

}  // namespace

struct pk_batch {
  pk_ctx* ctx = nullptr;
  int branches = 1;
  cudaStream_t origin = nullptr;
  std::vector<pk_job*> jobs;            // one per branch (own stream)
  std::vector<uint64_t> vcap;           // kept-row capacity of each branch's buffers
  pk_job* solo = nullptr;               // tuning and sets run on their own
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
  DevBuf input, scal, res, counter, okeys, osuf, opre;
  uint64_t out_cap = 0;
  int key_words = 1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> signature;      // shape of the captured batch
  bool copy_in_graph = false;           // the graph copies each set's input itself
  int input_mode = PK_BATCH_INPUT_IN_GRAPH;
  std::vector<SetPlan> plan;
  std::vector<Scalars> h_scal;
  std::vector<unsigned long long> h_res;
  std::map<std::pair<int, int>, Shape> tuned;  // (size class, k) -> launch shape
  std::vector<HostTable> extra;         // per set run on its own (empty otherwise)
  uint64_t device_rows = 0;
  pk_batch_stats st{};
};

namespace {

pk_status dev_alloc(pk_ctx* ctx, DevBuf& b, size_t bytes, cudaStream_t s) {
  if (b.p && b.bytes >= bytes) return PK_OK;
  if (b.p) {
    cudaFreeAsync(b.p, s);
    ctx->used -= b.bytes;
    b = DevBuf{};
  }
  bytes = std::max<size_t>(256, (bytes + 255) & ~(size_t)255);
  const uint64_t now = ctx->used.fetch_add(bytes) + bytes;
  if (ctx->budget && now > ctx->budget) {
    ctx->used -= bytes;
    return set_error(PK_ERR_NOMEM, "HBM budget exceeded by the batch buffers");
  }
  cudaError_t e = cudaMallocFromPoolAsync(&b.p, bytes, ctx->pool, s);
  if (e != cudaSuccess) {
    ctx->used -= bytes;
    b.p = nullptr;
    return set_error(PK_ERR_NOMEM, std::string("batch buffer: ") + cudaGetErrorString(e));
  }
  b.bytes = bytes;
  return PK_OK;
}

void dev_free(pk_ctx* ctx, DevBuf& b, cudaStream_t s) {
  if (b.p) {
    cudaFreeAsync(b.p, s);
    ctx->used -= b.bytes;
  }
  b = DevBuf{};
}

uint64_t kept_cap(uint64_t bytes) { return std::max<uint64_t>(1ull << 16, bytes / 8); }

// Sizes every buffer of a branch job for the largest set it will run (the requests
// count_impl and mn_enqueue make, at their bounds), so the capture allocates nothing.
pk_status presize(pk_job* j, uint64_t fmax, int k, int bbits, int t, int sms) {
  const size_t W = k > 32 ? 16 : 8;
  const int B = 1 << bbits;
  const int hb = std::min(bbits, kHistBits);
  const int HB = 1 << hb;
  const int Cn = 1 << std::min(bbits, kCoarseBits);
  const uint64_t ntiles = (fmax + kTileBytes - 1) / kTileBytes;
  const uint64_t vcap = kept_cap(fmax);
  PK_TRY(job_alloc(j, j->tile_nl, 4 * (ntiles + 1)));
  PK_TRY(job_alloc(j, j->counts, 4 * (size_t)sms * HB));
  PK_TRY(job_alloc(j, j->units, 40 * ((fmax + kSegBytes - 1) / kSegBytes)));
  PK_TRY(job_alloc(j, j->bsmall, 4 * kSmallCounts * (size_t)B));
  PK_TRY(job_alloc(j, j->bstart, 4 * (size_t)(B + 1)));
  PK_TRY(job_alloc(j, j->hstart, 4 * (size_t)(HB + 1)));
  PK_TRY(job_alloc(j, j->keys, W * fmax));
  PK_TRY(job_alloc(j, j->tkeys, W * fmax));
  PK_TRY(job_alloc(j, j->tcounts, 4 * fmax));
  PK_TRY(job_alloc(j, j->tu, 4 * (size_t)B));
  PK_TRY(job_alloc(j, j->hist, 8 * (size_t)t));
  PK_TRY(job_alloc(j, j->coff, 4 * (size_t)sms * Cn));
  PK_TRY(job_alloc(j, j->cstart, 4 * (size_t)(Cn + 1)));
  PK_TRY(job_alloc(j, j->slice_start, 4 * (size_t)(Cn + 1)));
  PK_TRY(job_alloc(j, j->fcur, 4 * (size_t)B));
  PK_TRY(job_alloc(j, j->kkeys, W * vcap));
  PK_TRY(job_alloc(j, j->kcounts, 4 * vcap));
  PK_TRY(job_alloc(j, j->kstart, 4 * (size_t)B));
  PK_TRY(job_alloc(j, j->kcount, 4 * (size_t)B));
  PK_TRY(job_alloc(j, j->ksub, 12 * (size_t)B));
  PK_TRY(job_alloc(j, j->flags_f, 8 * (size_t)B));
  PK_TRY(job_alloc(j, j->nkeys, W * 2 * vcap));
  PK_TRY(job_alloc(j, j->nsuf, 16 * 2 * vcap));
  PK_TRY(job_alloc(j, j->npre, 16 * 2 * vcap));
  PK_TRY(job_alloc(j, j->flags_m, 8 * (size_t)B));
  PK_TRY(job_alloc(j, j->gfirst, 4 * (size_t)B));
  PK_TRY(job_alloc(j, j->gcount, 4 * (size_t)B));
  PK_TRY(job_alloc(j, j->chunk_bucket, 4 * (fmax / kChunkKeys + 1)));
  PK_TRY(job_alloc(j, j->gdone, 4 * (size_t)B));
  PK_TRY(job_alloc(j, j->chunk_u, 4 * (fmax / kChunkKeys + 1)));
  return PK_OK;
}

int digits_for(pk_batch* b, const pk_params& p, uint64_t bytes) {
  if (p.bucket_bits) return std::min(p.bucket_bits, std::min(kMaxPartBits, 2 * p.k - 2));
  auto it = b->tuned.find({size_class(bytes), p.k});
  if (it != b->tuned.end()) return it->second.digits;
  return auto_bucket_bits(bytes, p.k, p.k > 32);
}

Shape shape_for(pk_batch* b, const pk_params& p, uint64_t bytes) {
  auto it = b->tuned.find({size_class(bytes), p.k});
  Shape s = it != b->tuned.end() ? it->second : Shape{};
  s.digits = digits_for(b, p, bytes);
  return s;
}

void apply(pk_job* j, const Shape& s) {
  j->chunk_mult = s.chunk_mult;
  j->table_ctas = s.table_ctas;
}

// Time the whole path of one set on a branch job (outside any capture).
pk_status time_set(pk_job* j, const void* d_fasta, uint64_t bytes, const pk_params& p, double* ms) {
  cudaEvent_t a, z;
  cudaEventCreate(&a);
  cudaEventCreate(&z);
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(a, j->stream);
    pk_summary s;
    pk_status r = pk_run_device(j, d_fasta, bytes, &p, &s);
    cudaEventRecord(z, j->stream);
    cudaEventSynchronize(z);
    if (r != PK_OK && r != PK_ERR_EMPTY) {
      cudaEventDestroy(a);
      cudaEventDestroy(z);
      return r;
    }
    float t = 0;
    cudaEventElapsedTime(&t, a, z);
    if (rep > 0) best = std::min(best, t);  // the first run also sizes the buffers
  }
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  *ms = best;
  return PK_OK;
}

// Autotune the launch shape of every (size class, k) of the batch that has automatic
// digits, on the class's largest set: first the partition digits (the fastest of the
// automatic choice and its two neighbours), then with those the chunk size (one or two
// times the one-chunk-per-SM size) and the table CTAs per SM (one or two).
// size classes not tuned yet -> their largest set
std::map<std::pair<int, int>, int> untuned(const pk_batch* b, const std::vector<SetPlan>& plan) {
  std::map<std::pair<int, int>, int> largest;  // class -> set index
  for (size_t i = 0; i < plan.size(); i++) {
    if (plan[i].params.bucket_bits || !plan[i].in_graph) continue;
    const std::pair<int, int> key{size_class(plan[i].bytes), plan[i].params.k};
    if (b->tuned.count(key)) continue;
    auto it = largest.find(key);
    if (it == largest.end() || plan[it->second].bytes < plan[i].bytes) largest[key] = (int)i;
  }
  return largest;
}

pk_status autotune(pk_batch* b, const std::vector<SetPlan>& plan) {
  const std::map<std::pair<int, int>, int> largest = untuned(b, plan);
  if (largest.empty()) return PK_OK;
  const auto t0 = std::chrono::steady_clock::now();
  pk_job* j = b->solo;
  for (auto& kv : largest) {
    const SetPlan& sp = plan[kv.second];
    const int base = auto_bucket_bits(sp.bytes, sp.params.k, sp.params.k > 32);
    int best_bits = base;
    double best_ms = 1e30;
    for (int d = -1; d <= 1; d++) {
      const int bits = base + d;
      if (bits < 2 || bits > std::min(kMaxPartBits, 2 * sp.params.k - 2)) continue;
      pk_params p = sp.params;
      p.bucket_bits = bits;
      double ms = 0;
      PK_TRY(time_set(j, (const char*)b->input.p + sp.off, sp.bytes, p, &ms));
      if (ms < best_ms) {
        best_ms = ms;
        best_bits = bits;
      }
    }
    Shape best{best_bits, 1, 2};
    for (int cm = 1; cm <= 2; cm++)
      for (int tc = 1; tc <= 2; tc++) {
        if (cm == 1 && tc == 2) continue;  // timed above
        pk_params p = sp.params;
        p.bucket_bits = best_bits;
        apply(j, Shape{best_bits, cm, tc});
        double ms = 0;
        const pk_status r = time_set(j, (const char*)b->input.p + sp.off, sp.bytes, p, &ms);
        apply(j, Shape{});
        PK_TRY(r);
        if (ms < best_ms) {
          best_ms = ms;
          best = Shape{best_bits, cm, tc};
        }
      }
    b->tuned[kv.first] = best;
  }
  pk_job_reset(j);
  b->st.tuned_classes = b->tuned.size();
  b->st.tune_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return PK_OK;
}

pk_status capture(pk_batch* b) {
  const int n = (int)b->plan.size();
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  // size each branch's buffers for its largest set (all jobs idle: reset first)
  b->vcap.assign(b->branches, 1);
  for (int r = 0; r < b->branches; r++) {
    pk_job* j = b->jobs[r];
    pk_job_reset(j);
    uint64_t fmax = 0;
    int kmax = 2, bmax = 2, tmax = 1;
    for (const SetPlan& sp : b->plan) {
      if (sp.branch != r || !sp.in_graph) continue;
      fmax = std::max(fmax, sp.bytes);
      kmax = std::max(kmax, (int)sp.params.k);
      bmax = std::max(bmax, sp.params.bucket_bits);
      tmax = std::max(tmax, (int)sp.params.num_buckets);
    }
    if (fmax == 0) continue;
    PK_TRY(presize(j, fmax + kAlign, kmax, bmax, tmax, b->ctx->sms));
    b->vcap[r] = kept_cap(fmax + kAlign);
    PK_CUDA(cudaStreamSynchronize(j->stream));
  }
  PK_CUDA(cudaStreamSynchronize(b->origin));
  PK_CUDA(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
  pk_status st = PK_OK;
  cudaEventRecord(b->fork, b->origin);
  for (int r = 0; r < b->branches; r++) cudaStreamWaitEvent(b->jobs[r]->stream, b->fork, 0);
  Scalars* scal = (Scalars*)b->scal.p;
  unsigned long long* res = (unsigned long long*)b->res.p;
  for (int i = 0; i < n && st == PK_OK; i++) {
    const SetPlan& sp = b->plan[i];
    if (!sp.in_graph) continue;
    pk_job* j = b->jobs[sp.branch];
    Scalars* own = j->d_sc;
    j->graph_mode = true;
    j->ncap = sp.bytes;
    j->d_sc = scal + i;
    apply(j, shape_for(b, sp.params, sp.bytes));
    if (b->copy_in_graph && sp.bytes) {
      // the set's input, on its branch ahead of its kernels: other branches compute
      // meanwhile
      cudaError_t e = cudaMemcpyAsync((char*)b->input.p + sp.off, sp.host, sp.bytes, cudaMemcpyHostToDevice,
                                      j->stream);
      if (e != cudaSuccess) st = set_error(PK_ERR_CUDA, std::string("batch input copy: ") + cudaGetErrorString(e));
    }
    if (st == PK_OK) st = count_impl(j, (const char*)b->input.p + sp.off, sp.bytes, &sp.params);
    if (st == PK_OK) st = cutoff_enqueue(j, sp.params.num_buckets);
    if (st == PK_OK) st = mn_enqueue(j, 0, b->vcap[sp.branch]);
    if (st == PK_OK) {
      cudaError_t e = launch_batch_emit(scal + i, (unsigned long long*)b->counter.p, b->out_cap, res + 3 * i,
                                        j->nkeys.p, j->nsuf.p, j->npre.p, j->wide, b->okeys.p, b->osuf.p,
                                        b->opre.p, j->stream);
      if (e != cudaSuccess) st = set_error(PK_ERR_CUDA, std::string("batch emit: ") + cudaGetErrorString(e));
    }
    j->graph_mode = false;
    j->d_sc = own;
    apply(j, Shape{});
  }
  for (int r = 0; r < b->branches; r++) {
    cudaEventRecord(b->join[r], b->jobs[r]->stream);
    cudaStreamWaitEvent(b->origin, b->join[r], 0);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->origin, &g);
  if (st != PK_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return set_error(PK_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  b->graph = g;
  e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) return set_error(PK_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  size_t nodes = 0;
  cudaGraphGetNodes(g, nullptr, &nodes);
  std::vector<cudaGraphNode_t> all(nodes);
  if (nodes) cudaGraphGetNodes(g, all.data(), &nodes);
  uint64_t kernels = 0;
  for (cudaGraphNode_t nd : all) {
    cudaGraphNodeType ty;
    if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) kernels++;
  }
  b->st.kernels_per_launch = kernels;
  b->st.graph_captures++;
  return PK_OK;
}

// A set run on its own (outside the graph), its rows kept on the host.
pk_status run_alone(pk_batch* b, int i, const pk_batch_set& s, pk_batch_result* out) {
  pk_job* j = b->solo;
  pk_summary sum{};
  pk_status r = pk_run(j, s.fasta, s.fasta_bytes, &s.params, &sum);
  out->status = r;
  out->rerun = 1;
  out->summary = sum;
  HostTable& ht = b->extra[i];
  ht = HostTable{};
  if (r == PK_OK && sum.n_nodes) {
    const uint64_t m = sum.n_nodes;
    const int kw = s.params.k > 32 ? 2 : 1;
    ht.keys.resize(m * kw);
    ht.suf.resize(4 * m);
    ht.pre.resize(4 * m);
    r = pk_copy_macro_nodes(j, ht.keys.data(), ht.suf.data(), ht.pre.data(), m);
    if (r != PK_OK) out->status = r;
    ht.rows = m;
  }
  pk_job_reset(j);
  b->st.reruns++;
  return PK_OK;
}

}  // namespace

pk_status pk_batch_create(pk_ctx* ctx, int32_t branches, pk_batch** out) {
  if (!ctx || !out) return set_error(PK_ERR_INVALID, "ctx and out must not be null");
  if (branches < 1 || branches > 32) return set_error(PK_ERR_INVALID, "branches must be in 1..32");
  PK_TRY(set_device(ctx));
  pk_batch* b = new pk_batch();
  b->ctx = ctx;
  b->branches = branches;
  cudaError_t e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
  if (e == cudaSuccess && pk_job_create(ctx, nullptr, &b->solo) != PK_OK) e = cudaErrorMemoryAllocation;
  for (int r = 0; r < branches && e == cudaSuccess; r++) {
    pk_job* j = nullptr;
    if (pk_job_create(ctx, nullptr, &j) != PK_OK) {
      e = cudaErrorMemoryAllocation;
      break;
    }
    b->jobs.push_back(j);
    cudaEvent_t ev;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) b->join.push_back(ev);
  }
  if (e != cudaSuccess) {
    pk_batch_destroy(b);
    return set_error(PK_ERR_CUDA, std::string("pk_batch_create: ") + cudaGetErrorString(e));
  }
  *out = b;
  return PK_OK;
}

void pk_batch_destroy(pk_batch* b) {
  if (!b) return;
  set_device(b->ctx);
  if (b->origin) cudaStreamSynchronize(b->origin);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  DevBuf* bufs[] = {&b->input, &b->scal, &b->res, &b->counter, &b->okeys, &b->osuf, &b->opre};
  for (DevBuf* d : bufs) dev_free(b->ctx, *d, b->origin);
  for (pk_job* j : b->jobs) pk_job_destroy(j);
  if (b->solo) pk_job_destroy(b->solo);
  for (cudaEvent_t ev : b->join) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  if (b->origin) {
    cudaStreamSynchronize(b->origin);
    cudaStreamDestroy(b->origin);
  }
  delete b;
}

pk_status pk_batch_run(pk_batch* b, const pk_batch_set* sets, int32_t n, pk_batch_result* results) {
  if (!b || (!sets && n) || (!results && n) || n < 0) return set_error(PK_ERR_INVALID, "null argument");
  PK_TRY(set_device(b->ctx));
  int wide = -1;
  for (int i = 0; i < n; i++) {
    PK_TRY(check_params(&sets[i].params));
    if (sets[i].fasta_bytes && !sets[i].fasta) return set_error(PK_ERR_INVALID, "a set's fasta is null");
    const int w = sets[i].params.k > 32;
    if (wide >= 0 && w != wide)
      return set_error(PK_ERR_INVALID, "all sets of a batch must use the same key width (k <= 32 or k > 32)");
    wide = w;
  }
  b->key_words = wide == 1 ? 2 : 1;
  // ---- plan: device offsets, branch assignment (largest first to the lightest branch)
  std::vector<SetPlan> plan(n);
  uint64_t off = 0, out_rows = 0;
  for (int i = 0; i < n; i++) {
    plan[i].off = off;
    plan[i].bytes = sets[i].fasta_bytes;
    plan[i].params = sets[i].params;
    plan[i].in_graph = sets[i].fasta_bytes > 0 && sets[i].fasta_bytes < (1ull << 32) - 1;
    plan[i].host = sets[i].fasta;
    off += (sets[i].fasta_bytes + kAlign - 1) / kAlign * kAlign;
    out_rows += kept_cap(sets[i].fasta_bytes) / 2;
  }
  // ---- input to the device.  When every set is in page-locked host memory the graph
  //      copies each set itself, on the set's branch ahead of its kernels, so the copies
  //      overlap the other branches' work; otherwise (and for the size classes still to
  //      be tuned, which are timed on their largest set) the sets are copied first.
  PK_TRY(dev_alloc(b->ctx, b->input, off + kAlign, b->origin));
  bool pinned = n > 0 && b->input_mode == PK_BATCH_INPUT_IN_GRAPH;
  for (int i = 0; i < n && pinned; i++) {
    if (!sets[i].fasta_bytes) continue;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, sets[i].fasta) != cudaSuccess || at.type != cudaMemoryTypeHost) pinned = false;
  }
  cudaGetLastError();
  if (!pinned || !untuned(b, plan).empty()) {
    for (int i = 0; i < n; i++)
      if (sets[i].fasta_bytes)
        PK_CUDA(cudaMemcpyAsync((char*)b->input.p + plan[i].off, sets[i].fasta, sets[i].fasta_bytes,
                                cudaMemcpyHostToDevice, b->origin));
    PK_CUDA(cudaStreamSynchronize(b->origin));
  }
  // ---- autotune digit widths of new size classes, then fix every set's digits
  PK_TRY(autotune(b, plan));
  for (int i = 0; i < n; i++) plan[i].params.bucket_bits = digits_for(b, plan[i].params, plan[i].bytes);
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return plan[x].bytes > plan[y].bytes; });
  std::vector<uint64_t> load(b->branches, 0);
  for (int i : order) {
    const int r = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    plan[i].branch = r;
    load[r] += plan[i].bytes;
  }
  // ---- (re)capture when the shape changed
  std::vector<uint64_t> sig;
  sig.push_back((uint64_t)n);
  sig.push_back(pinned ? 1 : 0);
  for (int i = 0; i < n; i++) {
    sig.push_back(plan[i].bytes);
    sig.push_back(plan[i].off);
    if (pinned) sig.push_back((uint64_t)(uintptr_t)plan[i].host);  // the graph reads these buffers
    const uint64_t* pw = (const uint64_t*)&plan[i].params;
    for (size_t w = 0; w < sizeof(pk_params) / 8; w++) sig.push_back(pw[w]);
  }
  const bool same = b->exec && sig == b->signature;
  b->plan = plan;
  b->copy_in_graph = pinned;
  b->out_cap = std::max<uint64_t>(1, out_rows);
  PK_TRY(dev_alloc(b->ctx, b->scal, sizeof(Scalars) * (size_t)std::max(1, n), b->origin));
  PK_TRY(dev_alloc(b->ctx, b->res, 24 * (size_t)std::max(1, n), b->origin));
  PK_TRY(dev_alloc(b->ctx, b->counter, 8, b->origin));
  PK_TRY(dev_alloc(b->ctx, b->okeys, 8 * b->key_words * b->out_cap, b->origin));
  PK_TRY(dev_alloc(b->ctx, b->osuf, 16 * b->out_cap, b->origin));
  PK_TRY(dev_alloc(b->ctx, b->opre, 16 * b->out_cap, b->origin));
  if (!same) {
    PK_TRY(capture(b));
    b->signature = sig;
  }
  // ---- per-set scalars initialised, one graph launch
  b->h_scal.assign(n, Scalars{});
  for (int i = 0; i < n; i++) {
    memset(&b->h_scal[i], 0, sizeof(Scalars));
    b->h_scal[i].s0 = ~0ull;
  }
  if (n) PK_CUDA(cudaMemcpyAsync(b->scal.p, b->h_scal.data(), sizeof(Scalars) * n, cudaMemcpyHostToDevice, b->origin));
  PK_CUDA(cudaMemsetAsync(b->counter.p, 0, 8, b->origin));
  PK_CUDA(cudaMemsetAsync(b->res.p, 0, 24 * (size_t)std::max(1, n), b->origin));
  PK_CUDA(cudaEventRecord(b->t0, b->origin));
  PK_CUDA(cudaGraphLaunch(b->exec, b->origin));
  PK_CUDA(cudaEventRecord(b->t1, b->origin));
  b->h_res.assign(3 * (size_t)std::max(1, n), 0);
  if (n) {
    PK_CUDA(cudaMemcpyAsync(b->h_scal.data(), b->scal.p, sizeof(Scalars) * n, cudaMemcpyDeviceToHost, b->origin));
    PK_CUDA(cudaMemcpyAsync(b->h_res.data(), b->res.p, 24 * n, cudaMemcpyDeviceToHost, b->origin));
  }
  PK_CUDA(cudaStreamSynchronize(b->origin));
  float gms = 0;
  cudaEventElapsedTime(&gms, b->t0, b->t1);
  b->st.last_graph_ms = gms;
  b->st.graph_launches++;
  // ---- results; sets that failed or overran a bound run again on their own
  b->extra.assign(n, HostTable{});
  uint64_t dev_rows = 0;
  for (int i = 0; i < n; i++) {
    const Scalars& sc = b->h_scal[i];
    const unsigned long long state = b->h_res[3 * i + 2];
    pk_batch_result& r = results[i];
    memset(&r, 0, sizeof(r));
    r.summary.n_reads = sc.n_reads;
    r.summary.n_windows = sc.n_windows;
    r.summary.n_unique = sc.n_unique;
    r.summary.n_kept = sc.n_kept;
    r.summary.cutoff = sc.cutoff;
    r.summary.key_bytes = wide == 1 ? 16 : 8;
    if (plan[i].in_graph && state == 1) {
      r.status = PK_OK;
      r.summary.n_nodes = b->h_res[3 * i + 1];
      r.mn_first = b->h_res[3 * i];
      dev_rows = std::max<uint64_t>(dev_rows, r.mn_first + r.summary.n_nodes);
    } else if (plan[i].in_graph && state == 4) {
      r.status = PK_ERR_EMPTY;
    } else {
      PK_TRY(run_alone(b, i, sets[i], &r));
    }
  }
  b->device_rows = dev_rows;
  uint64_t next = dev_rows;
  for (int i = 0; i < n; i++)
    if (results[i].rerun) {
      results[i].mn_first = next;
      next += b->extra[i].rows;
    }
  b->st.total_nodes = next;
  return PK_OK;
}

pk_status pk_batch_set_input_mode(pk_batch* b, int32_t mode) {
  if (!b) return set_error(PK_ERR_INVALID, "batch is null");
  if (mode != PK_BATCH_INPUT_IN_GRAPH && mode != PK_BATCH_INPUT_BEFORE)
    return set_error(PK_ERR_INVALID, "unknown batch input mode");
  b->input_mode = mode;
  return PK_OK;
}

pk_status pk_batch_copy_macro_nodes(pk_batch* b, void* keys, uint32_t* suf, uint32_t* pre, uint64_t cap) {
  if (!b) return set_error(PK_ERR_INVALID, "batch is null");
  if (cap < b->st.total_nodes) return set_error(PK_ERR_INVALID, "capacity smaller than the batch's node count");
  PK_TRY(set_device(b->ctx));
  const uint64_t m = b->device_rows;
  const int kw = b->key_words;
  if (m) {
    if (keys) PK_CUDA(cudaMemcpyAsync(keys, b->okeys.p, 8 * kw * m, cudaMemcpyDeviceToHost, b->origin));
    if (suf) PK_CUDA(cudaMemcpyAsync(suf, b->osuf.p, 16 * m, cudaMemcpyDeviceToHost, b->origin));
    if (pre) PK_CUDA(cudaMemcpyAsync(pre, b->opre.p, 16 * m, cudaMemcpyDeviceToHost, b->origin));
  }
  PK_CUDA(cudaStreamSynchronize(b->origin));
  uint64_t row = m;
  for (const HostTable& ht : b->extra) {
    if (!ht.rows) continue;
    if (keys) memcpy((uint64_t*)keys + row * kw, ht.keys.data(), 8 * kw * ht.rows);
    if (suf) memcpy(suf + 4 * row, ht.suf.data(), 16 * ht.rows);
    if (pre) memcpy(pre + 4 * row, ht.pre.data(), 16 * ht.rows);
    row += ht.rows;
  }
  return PK_OK;
}

pk_status pk_batch_get_stats(pk_batch* b, pk_batch_stats* out) {
  if (!b || !out) return set_error(PK_ERR_INVALID, "null argument");
  *out = b->st;
  return PK_OK;
}

pk_status pk_batch_tuned_shape(pk_batch* b, uint64_t fasta_bytes, int32_t k, int32_t* digits, int32_t* chunk_mult,
                               int32_t* table_ctas) {
  if (!b) return set_error(PK_ERR_INVALID, "batch is null");
  auto it = b->tuned.find({size_class(fasta_bytes), k});
  if (it == b->tuned.end()) return set_error(PK_ERR_STATE, "no tuned shape for this size and k");
  if (digits) *digits = it->second.digits;
  if (chunk_mult) *chunk_mult = it->second.chunk_mult;
  if (table_ctas) *table_ctas = it->second.table_ctas;
  return PK_OK;
}

int32_t pk_batch_tuned_bits(pk_batch* b, uint64_t fasta_bytes, int32_t k) {
  if (!b) return 0;
  auto it = b->tuned.find({size_class(fasta_bytes), k});
  return it == b->tuned.end() ? 0 : it->second.digits;
}
