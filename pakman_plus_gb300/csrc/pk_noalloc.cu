// Histogram cutoff that allocates nothing: pk_cutoff_noalloc.
//
// Some callers cannot allocate device memory at call time: an application that owns
// every device allocation through its own allocator or pool and forbids libraries
// from calling cudaMalloc, a latency-critical loop in which an allocation may block
// on the driver, or a process whose device-memory budget is already fully committed.
// For them this entry point computes the same histogram, cutoff and kept-row count
// as pk_cutoff, over a count column the caller already holds in device memory, using
// only the static scratch array below (no cudaMalloc, no cudaFree, no allocating
// library call).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pakman_gb300.h"
#include "pk_internal.h"

namespace {

// Histogram bins shared by every call in the process.  Any GPU that loads this
// library holds these PK_NOALLOC_MAX_BUCKETS x 8 bytes until the process exits.
static __device__ __align__(256) unsigned long long g_noalloc_hist[PK_NOALLOC_MAX_BUCKETS];

__global__ void __launch_bounds__(256) k_noalloc_clear(unsigned long long* h, int t) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < t; i += gridDim.x * blockDim.x) h[i] = 0;
}

__global__ void __launch_bounds__(256) k_noalloc_hist(const uint32_t* __restrict__ counts,
                                                      unsigned long long n, int t,
                                                      unsigned long long* h) {
  __shared__ uint32_t sh[PK_NOALLOC_MAX_BUCKETS];
  for (int i = threadIdx.x; i < t; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const uint32_t c = counts[i];
    if (c < (uint32_t)t) atomicAdd(&sh[c], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < t; i += blockDim.x)
    if (sh[i]) atomicAdd(&h[i], (unsigned long long)sh[i]);
}

// cutoff = first minimum of h[1..t) (t == 1 -> 1); kept = n - sum(h[1..cutoff)).
__global__ void __launch_bounds__(1024) k_noalloc_cutoff(const unsigned long long* __restrict__ h,
                                                         int t, unsigned long long n,
                                                         uint32_t* d_cutoff, uint64_t* d_hist,
                                                         uint64_t* d_kept) {
  __shared__ unsigned long long s_v[32];
  __shared__ int s_i[32];
  unsigned long long best = ~0ull;
  int bi = 0x7fffffff;
  for (int c = 1 + threadIdx.x; c < t; c += blockDim.x) {
    const unsigned long long v = h[c];
    if (v < best || (v == best && c < bi)) { best = v; bi = c; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v2 = __shfl_down_sync(0xffffffffu, best, o);
    const int i2 = __shfl_down_sync(0xffffffffu, bi, o);
    if (v2 < best || (v2 == best && i2 < bi)) { best = v2; bi = i2; }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { s_v[warp] = best; s_i[warp] = bi; }
  if (d_hist)
    for (int c = threadIdx.x; c < t; c += blockDim.x) d_hist[c] = h[c];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
      if (s_v[w] < best || (s_v[w] == best && s_i[w] < bi)) { best = s_v[w]; bi = s_i[w]; }
    const int cut = t > 1 ? bi : 1;
    unsigned long long below = 0;
    for (int c = 1; c < cut && c < t; c++) below += h[c];
    *d_cutoff = (uint32_t)cut;
    if (d_kept) *d_kept = n - below;
  }
}

}  // namespace

extern "C" pk_status pk_cutoff_noalloc(const uint32_t* d_counts, uint64_t n_rows, int32_t num_buckets,
                                       uint32_t* d_cutoff, uint64_t* d_hist, uint64_t* d_kept,
                                       void* stream) {
  if (num_buckets < 1 || num_buckets > PK_NOALLOC_MAX_BUCKETS)
    return pk::set_error(PK_ERR_INVALID, "num_buckets must be in 1..PK_NOALLOC_MAX_BUCKETS (4096): "
                                         "the static scratch holds that many bins");
  if (!d_cutoff) return pk::set_error(PK_ERR_INVALID, "d_cutoff is null");
  if (n_rows && !d_counts) return pk::set_error(PK_ERR_INVALID, "d_counts is null");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return pk::set_error(PK_ERR_NO_DEVICE, cudaGetErrorString(e));
  // the device address of the static scratch in the current context, looked up on every
  // call (a host-side query), so a reset or recreated context never leaves a stale
  // address behind; host code must not use the symbol itself as a device pointer
  unsigned long long* h = nullptr;
  e = cudaGetSymbolAddress((void**)&h, g_noalloc_hist);
  if (e != cudaSuccess) return pk::set_error(PK_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  cudaStream_t st = (cudaStream_t)stream;
  pk::note_launch(), k_noalloc_clear<<<(num_buckets + 255) / 256, 256, 0, st>>>(h, num_buckets);
  const uint64_t blocks = (n_rows + 255) / 256;  // clamped before narrowing
  const int grid = blocks > 1024 ? 1024 : (blocks < 1 ? 1 : (int)blocks);
  pk::note_launch(), k_noalloc_hist<<<grid, 256, 0, st>>>(d_counts, n_rows, num_buckets, h);
  pk::note_launch(), k_noalloc_cutoff<<<1, 1024, 0, st>>>(h, num_buckets, n_rows, d_cutoff, d_hist, d_kept);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pk::set_error(PK_ERR_CUDA, cudaGetErrorString(e));
  return PK_OK;
}
