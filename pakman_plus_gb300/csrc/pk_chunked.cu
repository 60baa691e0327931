// Counting in pieces: the device form of the reference's bounded batch flush.
//
// The reference counts any amount of input in bounded memory: its sliding window
// flushes every MAX_KMER_COUNT k-mers (-b, default 100000000,
// src/distribute_kmers.cpp:275-277) into a sort and run-length count whose result is
// merged into kmer_proc_buf (src/kmer_counting.cpp:3022-3139, 169-250).  Here a host
// FASTA buffer that does not fit the job's HBM budget in one pass (or any buffer, when
// pk_params.chunking asks for it) is cut into record-aligned pieces of at most -b bytes
// -- so at most -b k-mer windows each -- and every piece goes through the whole-input
// path (count_impl).  Each piece's sorted (k-mer, count) table is merged on the device
// into the accumulated table: both are sorted and unique, so every key is ranked into
// the merged order by a binary search in the other table, equal keys land next to each
// other, and one pass keeps the first of each run with the run's summed count.  The
// final table is installed as the job's table (as pk_table_load does), so the cutoff,
// macro-nodes and everything after them run unchanged.  The result is the same table
// for any piece size, as the reference's is for any -b.
//
// Pieces are cut only where a header line starts: at a '>' right after a newline whose
// line index, counted from the first '>' of the whole buffer, is even -- the lines of
// every piece then alternate header / sequence exactly as they do in the whole buffer,
// so windows, record checks and read counts are unchanged.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <utility>

#include "../../include/pakman_gb300.h"
#include "pk_internal.h"
#include "pk_runtime.h"

using namespace pk;

namespace {

typedef unsigned __int128 u128;

constexpr int kTileThreads = 256;
constexpr int kTilePer = 16;                           // elements per thread
constexpr int kTile = kTileThreads * kTilePer;         // elements per scan tile
constexpr uint64_t kMinPiece = 1ull << 20;             // smallest piece tried after NOMEM

template <typename KeyT>
__device__ __forceinline__ uint64_t lower_bound_g(const KeyT* __restrict__ a, uint64_t n, KeyT x) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <typename KeyT>
__device__ __forceinline__ uint64_t upper_bound_g(const KeyT* __restrict__ a, uint64_t n, KeyT x) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (x < a[mid]) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Merged order of two sorted unique tables: A's row i goes to i + |{b < A[i]}|, B's row
// j to j + |{a <= B[j]}|, so a key present in both sits at p (from A) and p + 1 (from B).
template <typename KeyT>
__global__ void __launch_bounds__(256) k_merge_place(const KeyT* __restrict__ a, const uint32_t* __restrict__ ca,
                                                     uint64_t na, const KeyT* __restrict__ b,
                                                     const uint32_t* __restrict__ cb, uint64_t nb,
                                                     KeyT* __restrict__ m, uint32_t* __restrict__ cm) {
  const uint64_t n = na + nb;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (uint64_t)gridDim.x * blockDim.x) {
    if (e < na) {
      const KeyT x = a[e];
      const uint64_t pos = e + lower_bound_g(b, nb, x);
      m[pos] = x;
      cm[pos] = ca[e];
    } else {
      const uint64_t i = e - na;
      const KeyT x = b[i];
      const uint64_t pos = i + upper_bound_g(a, na, x);
      m[pos] = x;
      cm[pos] = cb[i];
    }
  }
}

template <typename KeyT>
__device__ __forceinline__ bool is_head(const KeyT* __restrict__ m, uint64_t p) {
  return p == 0 || !(m[p - 1] == m[p]);
}

// first rows of the runs of equal keys, per scan tile
template <typename KeyT>
__global__ void __launch_bounds__(kTileThreads) k_merge_heads(const KeyT* __restrict__ m, uint64_t n,
                                                             uint32_t* __restrict__ part) {
  const uint64_t base = (uint64_t)blockIdx.x * kTile + (uint64_t)threadIdx.x * kTilePer;
  uint32_t c = 0;
  for (int q = 0; q < kTilePer; q++)
    if (base + q < n) c += is_head(m, base + q);
  c = __reduce_add_sync(0xffffffffu, c);
  __shared__ uint32_t s[kTileThreads / 32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kTileThreads / 32; w++) t += s[w];
    part[blockIdx.x] = t;
  }
}

// exclusive prefix of the tile counts (one block; total at part[tiles])
__global__ void __launch_bounds__(1024) k_merge_tile_prefix(uint32_t* part, uint64_t tiles) {
  __shared__ uint32_t s[1024];
  const uint64_t per = (tiles + 1023) / 1024;
  const uint64_t t0 = min(tiles, (uint64_t)threadIdx.x * per), t1 = min(tiles, t0 + per);
  uint32_t sum = 0;
  for (uint64_t t = t0; t < t1; t++) sum += part[t];
  s[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const uint32_t v = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = s[threadIdx.x] - sum;
  for (uint64_t t = t0; t < t1; t++) {
    const uint32_t v = part[t];
    part[t] = run;
    run += v;
  }
  if (threadIdx.x == 1023) part[tiles] = s[1023];
}

// one row per run of equal keys, its count the run's sum (a run has at most two rows)
template <typename KeyT>
__global__ void __launch_bounds__(kTileThreads) k_merge_emit(const KeyT* __restrict__ m, const uint32_t* __restrict__ cm,
                                                            uint64_t n, const uint32_t* __restrict__ part,
                                                            KeyT* __restrict__ ok, uint32_t* __restrict__ oc) {
  __shared__ uint32_t s[kTileThreads];
  const uint64_t base = (uint64_t)blockIdx.x * kTile + (uint64_t)threadIdx.x * kTilePer;
  uint32_t c = 0;
  for (int q = 0; q < kTilePer; q++)
    if (base + q < n) c += is_head(m, base + q);
  s[threadIdx.x] = c;
  __syncthreads();
  for (int o = 1; o < kTileThreads; o <<= 1) {
    const uint32_t v = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  uint64_t out = (uint64_t)part[blockIdx.x] + s[threadIdx.x] - c;
  for (int q = 0; q < kTilePer; q++) {
    const uint64_t p = base + q;
    if (p >= n || !is_head(m, p)) continue;
    uint32_t cnt = cm[p];
    if (p + 1 < n && m[p + 1] == m[p]) cnt += cm[p + 1];
    ok[out] = m[p];
    oc[out] = cnt;
    out++;
  }
}

template <typename KeyT>
cudaError_t launch_merge(const void* a, const uint32_t* ca, uint64_t na, const void* b, const uint32_t* cb,
                         uint64_t nb, void* m, uint32_t* cm, uint32_t* part, void* ok, uint32_t* oc,
                         cudaStream_t st) {
  const uint64_t n = na + nb;
  const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, 152ull * 64);
  if (n) {
    pk::note_launch(), k_merge_place<KeyT><<<grid, 256, 0, st>>>((const KeyT*)a, ca, na, (const KeyT*)b, cb, nb,
                                                                 (KeyT*)m, cm);
  }
  const uint64_t tiles = (n + kTile - 1) / kTile;
  if (tiles) pk::note_launch(), k_merge_heads<KeyT><<<(unsigned)tiles, kTileThreads, 0, st>>>((const KeyT*)m, n, part);
  pk::note_launch(), k_merge_tile_prefix<<<1, 1024, 0, st>>>(part, tiles);
  if (tiles)
    pk::note_launch(), k_merge_emit<KeyT><<<(unsigned)tiles, kTileThreads, 0, st>>>((const KeyT*)m, cm, n, part,
                                                                                    (KeyT*)ok, oc);
  return cudaGetLastError();
}

// Record-aligned cut points of a host FASTA buffer.
struct Cutter {
  const char* buf;
  uint64_t n;
  uint64_t s0;         // first '>' (n: none)
  uint64_t pos = 0;    // newline parity is known for [s0, pos)
  uint32_t par = 0;

  Cutter(const char* b, uint64_t len) : buf(b), n(len) {
    const void* q = len ? memchr(b, '>', (size_t)len) : nullptr;
    s0 = q ? (uint64_t)(static_cast<const char*>(q) - b) : len;
    pos = s0;
  }
  void advance(uint64_t x) {  // parity of the newlines in [s0, x)
    for (uint64_t i = pos; i < x; i++) par ^= buf[i] == '\n';
    pos = std::max(pos, x);
  }
  // the first header start at or after `target` (n when there is none)
  uint64_t next_cut(uint64_t target) {
    if (s0 >= n) return n;
    target = std::max(target, s0 + 1);
    if (target >= n) return n;
    advance(target);
    uint64_t p = pos;
    while (p < n) {
      const void* q = memchr(buf + p, '\n', (size_t)(n - p));
      if (!q) return n;
      const uint64_t r = (uint64_t)(static_cast<const char*>(q) - buf);
      advance(r + 1);  // the newline at r is counted
      p = r + 1;
      if (p < n && buf[p] == '>' && par == 0) return p;
    }
    return n;
  }
};

pk_status merge_into(pk_job* j, int cur, uint64_t na, uint64_t nb, uint64_t* nout) {
  const size_t W = j->wide ? 16 : 8;
  const uint64_t n = na + nb;
  if (n >= 0xffffffffull) return set_error(PK_ERR_LIMIT, "more than 2^32-2 distinct k-mers");
  const int nxt = cur ^ 1;
  PK_TRY(job_alloc(j, j->merge_keys, W * (n ? n : 1)));
  PK_TRY(job_alloc(j, j->merge_counts, 4 * (n ? n : 1)));
  PK_TRY(job_alloc(j, j->merge_part, 4 * ((n + kTile - 1) / kTile + 1)));
  PK_TRY(job_alloc(j, j->acc_keys[nxt], W * (n ? n : 1)));
  PK_TRY(job_alloc(j, j->acc_counts[nxt], 4 * (n ? n : 1)));
  const void* a = j->acc_keys[cur].p;
  const uint32_t* ca = (const uint32_t*)j->acc_counts[cur].p;
  cudaError_t e = j->wide ? launch_merge<u128>(a, ca, na, j->dkeys.p, (const uint32_t*)j->dcounts.p, nb,
                                              j->merge_keys.p, (uint32_t*)j->merge_counts.p,
                                              (uint32_t*)j->merge_part.p, j->acc_keys[nxt].p,
                                              (uint32_t*)j->acc_counts[nxt].p, j->stream)
                          : launch_merge<uint64_t>(a, ca, na, j->dkeys.p, (const uint32_t*)j->dcounts.p, nb,
                                                   j->merge_keys.p, (uint32_t*)j->merge_counts.p,
                                                   (uint32_t*)j->merge_part.p, j->acc_keys[nxt].p,
                                                   (uint32_t*)j->acc_counts[nxt].p, j->stream);
  PK_CUDA(e);
  uint32_t total = 0;
  const uint64_t tiles = (n + kTile - 1) / kTile;
  PK_CUDA(cudaMemcpyAsync(&total, (const uint32_t*)j->merge_part.p + tiles, 4, cudaMemcpyDeviceToHost, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  *nout = total;
  return PK_OK;
}

}  // namespace

// The whole pieces path for a host buffer; on success the job holds the merged table at
// stage 1, as after pk_count.
pk_status pk::count_pieces(pk_job* j, const char* host, uint64_t n, const pk_params* p, uint64_t piece) {
  if (piece == 0) piece = 100000000ull;
  j->params = *p;
  j->wide = p->k > 32;
  j->stage = 0;
  j->wired = false;
  j->compacted = false;
  Cutter cut(host, n);
  uint64_t start = 0, windows = 0, reads = 0, rows = 0;
  uint32_t pieces = 0;
  int cur = 0;
  const size_t W = j->wide ? 16 : 8;
  while (start < n || pieces == 0) {
    const uint64_t end = cut.next_cut(start + piece);
    const uint64_t len = end - start;
    PK_TRY(job_alloc(j, j->fasta, (size_t)len + 16));
    if (len) PK_CUDA(cudaMemcpyAsync(j->fasta.p, host + start, len, cudaMemcpyHostToDevice, j->stream));
    pk_status s = count_impl(j, j->fasta.p, len, p);
    if ((s == PK_ERR_NOMEM || s == PK_ERR_LIMIT) && piece > kMinPiece && len > kMinPiece) {
      piece = std::max(kMinPiece, piece / 2);  // this piece again, smaller
      PK_CUDA(cudaStreamSynchronize(j->stream));
      continue;
    }
    PK_TRY(s);
    PK_TRY(sync_scalars(j));
    windows += j->h_sc->n_windows;
    reads += j->h_sc->n_reads;
    const uint64_t u = j->h_sc->n_unique;
    PK_TRY(dense_table(j));
    if (pieces == 0) {
      PK_TRY(job_alloc(j, j->acc_keys[cur], W * (u ? u : 1)));
      PK_TRY(job_alloc(j, j->acc_counts[cur], 4 * (u ? u : 1)));
      if (u) {
        PK_CUDA(cudaMemcpyAsync(j->acc_keys[cur].p, j->dkeys.p, W * u, cudaMemcpyDeviceToDevice, j->stream));
        PK_CUDA(cudaMemcpyAsync(j->acc_counts[cur].p, j->dcounts.p, 4 * u, cudaMemcpyDeviceToDevice, j->stream));
      }
      rows = u;
    } else {
      uint64_t merged = 0;
      PK_TRY(merge_into(j, cur, rows, u, &merged));
      cur ^= 1;
      rows = merged;
    }
    pieces++;
    start = end;
  }
  PK_CUDA(cudaStreamSynchronize(j->stream));
  // the merged table becomes the job's table; the pieces' buffers are released
  std::swap(j->tkeys, j->acc_keys[cur]);
  std::swap(j->tcounts, j->acc_counts[cur]);
  release_piece_buffers(j);
  j->bsmall_valid = false;  // the merged table has no per-bucket small-count histogram
  const int k = p->k;
  int bb = p->bucket_bits;
  if (!bb) {  // about 4000 rows per bucket, as for a loaded table
    bb = 2;
    while (bb < kMaxPartBits && (double)rows / (double)(1u << bb) > 4000.0) bb++;
  }
  j->bbits = std::max(2, std::min(bb, std::min(kMaxPartBits, 2 * k - 2)));
  const int B = 1 << j->bbits;
  PK_TRY(job_alloc(j, j->bstart, sizeof(uint32_t) * (B + 1)));
  PK_TRY(job_alloc(j, j->tu, sizeof(uint32_t) * (size_t)B));
  PK_CUDA(launch_table_bounds(j->tkeys.p, rows, j->bbits, k, (uint32_t*)j->bstart.p, (uint32_t*)j->tu.p,
                              j->wide, j->stream));
  Scalars init{};
  memset(&init, 0, sizeof(init));
  init.n_unique = rows;
  init.n_windows = windows;
  init.n_reads = reads;
  *j->h_sc = init;
  PK_CUDA(cudaMemcpyAsync(j->d_sc, j->h_sc, sizeof(Scalars), cudaMemcpyHostToDevice, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  j->N = rows;
  j->F = n;
  j->t_hist = 0;  // no histogram was fused into a counting pass
  j->dense_valid = false;
  j->pieces = pieces;
  j->stage = 1;
  return PK_OK;
}

extern "C" pk_status pk_count_pieces(pk_job* j, uint32_t* pieces) {
  if (!j || !pieces) return set_error(PK_ERR_INVALID, "null argument");
  if (j->stage < 1) return set_error(PK_ERR_STATE, "no table: call pk_count first");
  *pieces = j->pieces;
  return PK_OK;
}
