// sm_103a kernels for PaKman's k-mer counting -> histogram cutoff -> macro-node path.
//
// Pipeline for one read set (FASTA bytes resident in HBM):
//   k_line_scan        newline count per 64 KB tile, first '>' and '>' count
//   k_tile_prefix      exclusive newline prefix over tiles, newlines before the first '>'
//   k_extract          per chunk: roll every k-mer window, histogram of bucket ids (smem)
//   k_col_prefix       per bucket: prefix over chunks; k_bucket_prefix: bucket starts;
//   k_coarse_offsets   each chunk's segment of every coarse region
//   k_scatter_coarse   roll again, keys to their coarse region through shared-memory rings
//   k_scatter_fine     per slice of a coarse region: keys to their bucket, staged by bucket
//   k_giant_chunks     chunk items of buckets too large for one CTA
//   k_bucket_table     per bucket: hash-aggregate in smem, sort the distinct keys, write
//                      the (k-mer, count) rows and the count histogram
//   k_cutoff           first minimum of the count histogram over [1, t)
//   k_filter_kept      kept rows (count >= cutoff), dense, with a decoupled look-back
//   k_macro_nodes      per (k-1)-mer unit: merge the suffix-side and prefix-side
//                      streams of kept k-mers into macro-node records
//   k_wire             initial wiring of every macro-node
//
// A bucket is the leading `bbits` bits of the 2k-bit key, so buckets in index order
// are the table in key order and no global merge is needed.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "pk_internal.h"

namespace pk {

typedef unsigned __int128 u128;

#define FULLMASK 0xffffffffu

// ----------------------------------------------------------------- key helpers ----
template <typename K>
struct KeyOps;

template <>
struct KeyOps<uint64_t> {
  static constexpr int W = 8;
  __device__ __forceinline__ static uint64_t mask(int bits) {
    return bits >= 64 ? ~0ull : ((1ull << bits) - 1ull);
  }
  __device__ __forceinline__ static uint64_t shr(uint64_t x, int s) { return s >= 64 ? 0ull : x >> s; }
  __device__ __forceinline__ static uint64_t shl(uint64_t x, int s) { return s >= 64 ? 0ull : x << s; }
  __device__ __forceinline__ static uint32_t low32(uint64_t x) { return (uint32_t)x; }
  __device__ __forceinline__ static uint64_t hash(uint64_t x) { return x * 0x9E3779B97F4A7C15ull; }
  __device__ __forceinline__ static unsigned match(unsigned m, uint64_t x) {
    return __match_any_sync(m, (unsigned long long)x);
  }
  __device__ __forceinline__ static int top_bit(uint64_t x) { return 63 - __clzll((long long)x); }
  __device__ __forceinline__ static uint64_t cas(uint64_t* p, uint64_t cmp, uint64_t val) {
    return atomicCAS(reinterpret_cast<unsigned long long*>(p), (unsigned long long)cmp,
                     (unsigned long long)val);
  }
};

template <>
struct KeyOps<u128> {
  static constexpr int W = 16;
  __device__ __forceinline__ static u128 mask(int bits) {
    return bits >= 128 ? ~(u128)0 : (((u128)1 << bits) - 1);
  }
  __device__ __forceinline__ static u128 shr(u128 x, int s) { return s >= 128 ? (u128)0 : x >> s; }
  __device__ __forceinline__ static u128 shl(u128 x, int s) { return s >= 128 ? (u128)0 : x << s; }
  __device__ __forceinline__ static uint32_t low32(u128 x) { return (uint32_t)(uint64_t)x; }
  __device__ __forceinline__ static uint64_t hash(u128 x) {
    uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
    return (lo ^ (hi * 0xC2B2AE3D27D4EB4Full)) * 0x9E3779B97F4A7C15ull;
  }
  __device__ __forceinline__ static unsigned match(unsigned m, u128 x) {
    return __match_any_sync(m, (unsigned long long)x) &
           __match_any_sync(m, (unsigned long long)(x >> 64));
  }
  __device__ __forceinline__ static int top_bit(u128 x) {
    const uint64_t hi = (uint64_t)(x >> 64);
    return hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)(uint64_t)x);
  }
  __device__ __forceinline__ static u128 cas(u128* p, u128 cmp, u128 val) { return atomicCAS(p, cmp, val); }
};

// A key loaded through L2 only (data another CTA of the same kernel wrote).
__device__ __forceinline__ uint64_t ldcg_key(const uint64_t* p) {
  return (uint64_t)__ldcg(reinterpret_cast<const unsigned long long*>(p));
}
__device__ __forceinline__ u128 ldcg_key(const u128* p) {
  const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2*>(p));
  return ((u128)v.y << 64) | v.x;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned r;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}


// Decoupled look-back words: status in bits 62-63 (1 = aggregate, 2 = inclusive).
constexpr unsigned long long kLbAgg = 1ull << 62;
constexpr unsigned long long kLbIncl = 2ull << 62;
constexpr unsigned long long kLbVal = (1ull << 62) - 1;
constexpr int kLbSpinLimit = 1 << 24;  // ~1-2 s with the back-off below (the default)
__device__ __forceinline__ int spin_limit(int limit) { return limit > 0 ? limit : kLbSpinLimit; }

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
  return v;
}

// Exclusive prefix of `flags[0..idx)`, computed by a whole warp (all 32 lanes call it
// and all get the sum).  Each step reads the 32 nearest unread predecessors at once
// (lane 0 = nearest): it stops at the nearest inclusive word, otherwise adds the
// aggregates up to the first word still unpublished and moves past them.  Waiting on
// an unpublished word is bounded: on expiry the error bit is set and the partial sum
// is returned.
__device__ unsigned long long lookback_exclusive(unsigned long long* flags, int idx, uint32_t* err,
                                                int limit) {
  const int max_spins = spin_limit(limit);
  const int lane = threadIdx.x & 31;
  unsigned long long sum = 0;
  int top = idx - 1;  // nearest predecessor not yet added
  int spins = 0;
  while (top >= 0) {
    const int j = top - lane;
    const unsigned long long f = j >= 0 ? ld_acquire(&flags[j]) : kLbIncl;  // below 0: inclusive 0
    const unsigned st = (unsigned)(f >> 62);
    const unsigned waiting = __ballot_sync(FULLMASK, st == 0);
    const unsigned incl = __ballot_sync(FULLMASK, st == 2);
    const int first_wait = waiting ? __ffs(waiting) - 1 : 32;
    const int first_incl = incl ? __ffs(incl) - 1 : 32;
    if (first_incl < first_wait) {
      sum += warp_sum_u64(lane <= first_incl ? (f & kLbVal) : 0ull);
      return sum;
    }
    if (first_wait > 0) {
      sum += warp_sum_u64(lane < first_wait ? (f & kLbVal) : 0ull);
      top -= first_wait;
      spins = 0;
      continue;
    }
    if (++spins >= max_spins) {
      if (lane == 0) atomicOr(err, ERR_LOOKBACK);
      return sum;
    }
    __nanosleep(spins < 64 ? 32 : 256);
  }
  return sum;
}

// Block-wide exclusive sum over `nthreads` (multiple of 32, <= 1024) threads.
__device__ __forceinline__ uint32_t block_exclusive_sum(uint32_t v, uint32_t* s_warp, uint32_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(FULLMASK, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nw ? s_warp[lane] : 0;
    uint32_t ws = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(FULLMASK, ws, o);
      if (lane >= o) ws += y;
    }
    if (lane < nw) s_warp[lane] = ws - w;
    if (lane == 31) s_warp[32] = ws;
  }
  __syncthreads();
  uint32_t res = s_warp[warp] + x - v;
  total = s_warp[32];
  __syncthreads();
  return res;
}

// Block-wide OR and AND of a key (result in x_or/x_and of every thread).
template <typename KeyT>
__device__ void block_or_and(KeyT& x_or, KeyT& x_and, KeyT* s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint64_t olo = (uint64_t)x_or, ohi = (uint64_t)(x_or >> 32 >> 32);
  uint64_t alo = (uint64_t)x_and, ahi = (uint64_t)(x_and >> 32 >> 32);
  for (int o = 16; o > 0; o >>= 1) {
    olo |= __shfl_xor_sync(FULLMASK, olo, o);
    ohi |= __shfl_xor_sync(FULLMASK, ohi, o);
    alo &= __shfl_xor_sync(FULLMASK, alo, o);
    ahi &= __shfl_xor_sync(FULLMASK, ahi, o);
  }
  if (lane == 0) {
    s_red[warp] = (KeyT)olo | ((KeyT)ohi << 32 << 32);
    s_red[nw + warp] = (KeyT)alo | ((KeyT)ahi << 32 << 32);
  }
  __syncthreads();
  KeyT ro = 0, ra = ~(KeyT)0;
  for (int w = 0; w < nw; w++) { ro |= s_red[w]; ra &= s_red[nw + w]; }
  x_or = ro;
  x_and = ra;
  __syncthreads();
}

// ------------------------------------------------------------- line scan (k_line_scan) -
// Newlines per 64 KB tile, the first '>' and the number of '>' bytes.
__global__ void __launch_bounds__(256) k_line_scan(const uint8_t* __restrict__ buf,
                                                   unsigned long long F, uint32_t* tile_nl,
                                                   Scalars* sc, unsigned long long tile0) {
  const unsigned long long tile = tile0 + blockIdx.x;
  const unsigned long long t0 = tile * kTileBytes;
  const unsigned long long t1 = min(t0 + (unsigned long long)kTileBytes, F);
  uint32_t nl = 0, gt = 0;
  unsigned long long first = ~0ull;
  for (unsigned long long p = t0 + 16ull * threadIdx.x; p < t1; p += 16ull * blockDim.x) {
    uint32_t w[4];
    if (p + 16 <= F) {
      uint4 v = __ldg(reinterpret_cast<const uint4*>(buf + p));
      w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
    } else {
      for (int i = 0; i < 4; i++) {
        uint32_t x = 0;
        for (int b = 0; b < 4; b++) {
          unsigned long long q = p + 4 * i + b;
          if (q < F) x |= (uint32_t)buf[q] << (8 * b);
        }
        w[i] = x;
      }
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
      nl += __popc(__vcmpeq4(w[i], 0x0A0A0A0Au)) >> 3;
      uint32_t g = __vcmpeq4(w[i], 0x3E3E3E3Eu);
      // a zero byte past F never compares equal to '>'
      gt += __popc(g) >> 3;
      if (g && first == ~0ull) first = p + 4 * i + (__ffs(g) - 1) / 8;
    }
  }
  __shared__ uint32_t s_nl[8], s_gt[8];
  __shared__ unsigned long long s_first[8];
  for (int o = 16; o > 0; o >>= 1) {
    nl += __shfl_down_sync(FULLMASK, nl, o);
    gt += __shfl_down_sync(FULLMASK, gt, o);
    unsigned long long f2 = __shfl_down_sync(FULLMASK, first, o);
    first = min(first, f2);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { s_nl[warp] = nl; s_gt[warp] = gt; s_first[warp] = first; }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t a = 0, b = 0;
    unsigned long long f = ~0ull;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) { a += s_nl[i]; b += s_gt[i]; f = min(f, s_first[i]); }
    tile_nl[tile] = a;
    if (b) atomicAdd(&sc->n_reads, (unsigned long long)b);
    if (f != ~0ull) atomicMin(&sc->s0, f);
  }
}

// One CTA: exclusive prefix of tile newline counts (in place, plus the grand total at
// [ntiles]) and the number of newlines before the first '>'.
__global__ void __launch_bounds__(1024) k_tile_prefix(const uint8_t* __restrict__ buf,
                                                      unsigned long long F, uint32_t* tile_nl,
                                                      int ntiles, Scalars* sc) {
  __shared__ uint32_t s_warp[33];
  uint32_t carry = 0;
  for (int base = 0; base < ntiles; base += blockDim.x) {
    int i = base + threadIdx.x;
    uint32_t v = i < ntiles ? tile_nl[i] : 0;
    uint32_t tot;
    uint32_t ex = block_exclusive_sum(v, s_warp, tot);
    if (i < ntiles) tile_nl[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) tile_nl[ntiles] = carry;
  __syncthreads();
  // newlines in [tile_start(s0), s0)
  const unsigned long long s0 = sc->s0;
  uint32_t cnt = 0;
  if (s0 < F) {
    const unsigned long long ts = (s0 / kTileBytes) * kTileBytes;
    for (unsigned long long p = ts + threadIdx.x; p < s0; p += blockDim.x) cnt += (buf[p] == '\n');
  }
  uint32_t tot;
  block_exclusive_sum(cnt, s_warp, tot);
  if (threadIdx.x == 0) {
    sc->nl_before_s0 = s0 < F ? tile_nl[s0 / kTileBytes] + tot : carry;
  }
}

// --------------------------------------------------------- k-mer window extraction --
// 16 input bytes -> 2-bit codes (byte 0 in the top bits), the bit-2 plane of the
// codes, newline flags and N flags.
__device__ __forceinline__ uint32_t pack4_codes(uint32_t w) {
  return (((w >> 1) & 0x03030303u) * 0x40100401u) >> 24;
}
__device__ __forceinline__ uint32_t pack4_nbits(uint32_t w) {
  return (((w >> 3) & 0x01010101u) * 0x40100401u) >> 24;
}
__device__ __forceinline__ uint32_t flags4(uint32_t eq) {
  return ((eq & 0x01010101u) * 0x01020408u) >> 24;
}

struct UnitBits {
  uint32_t codes;  // base j at bits 2(15-j)+1..2(15-j)
  uint32_t nbits;  // code bit 2 of byte j at bit 2(15-j)
  uint32_t nl;     // bit j: byte j is '\n'
  uint32_t nn;     // bit j: byte j is 'N' or 'n'
};

__device__ __forceinline__ UnitBits decode_unit(const uint32_t w[4], bool want_n = true) {
  UnitBits u;
  u.codes = (pack4_codes(w[0]) << 24) | (pack4_codes(w[1]) << 16) | (pack4_codes(w[2]) << 8) |
            pack4_codes(w[3]);
  u.nbits = (pack4_nbits(w[0]) << 24) | (pack4_nbits(w[1]) << 16) | (pack4_nbits(w[2]) << 8) |
            pack4_nbits(w[3]);
  u.nl = flags4(__vcmpeq4(w[0], 0x0A0A0A0Au)) | (flags4(__vcmpeq4(w[1], 0x0A0A0A0Au)) << 4) |
         (flags4(__vcmpeq4(w[2], 0x0A0A0A0Au)) << 8) | (flags4(__vcmpeq4(w[3], 0x0A0A0A0Au)) << 12);
  u.nn = 0;
  if (want_n)
    u.nn = flags4(__vcmpeq4(w[0] | 0x20202020u, 0x6E6E6E6Eu)) |
           (flags4(__vcmpeq4(w[1] | 0x20202020u, 0x6E6E6E6Eu)) << 4) |
           (flags4(__vcmpeq4(w[2] | 0x20202020u, 0x6E6E6E6Eu)) << 8) |
           (flags4(__vcmpeq4(w[3] | 0x20202020u, 0x6E6E6E6Eu)) << 12);
  return u;
}

__device__ __forceinline__ void load_unit(const uint8_t* __restrict__ buf, unsigned long long F,
                                          unsigned long long p, uint32_t w[4]) {
  if (p + 16 <= F) {
    uint4 v = __ldg(reinterpret_cast<const uint4*>(buf + p));
    w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
  } else {
#pragma unroll
    for (int i = 0; i < 4; i++) {
      uint32_t x = 0;
      for (int b = 0; b < 4; b++) {
        unsigned long long q = p + 4 * i + b;
        if (q < F) x |= (uint32_t)buf[q] << (8 * b);
      }
      w[i] = x;
    }
  }
}

// Rolling state: packed 2-bit codes (newest base in bits 0-1 of r0), the bit-2 plane
// of the codes at each byte's own low-bit position (n*), and a history of "window
// breakers" (newline, or N under the drop policy), newest at bit 0 of h0.
struct Roll {
  uint64_t r0, r1, r2;
  uint64_t n0, n1, n2;
  uint64_t h0, h1;
};

__device__ __forceinline__ void roll_push(Roll& s, const UnitBits& u, bool drop_n) {
  s.r2 = (s.r2 << 32) | (s.r1 >> 32);
  s.r1 = (s.r1 << 32) | (s.r0 >> 32);
  s.r0 = (s.r0 << 32) | (uint64_t)u.codes;
  s.n2 = (s.n2 << 32) | (s.n1 >> 32);
  s.n1 = (s.n1 << 32) | (s.n0 >> 32);
  s.n0 = (s.n0 << 32) | (uint64_t)u.nbits;
  uint32_t brk = u.nl | (drop_n ? u.nn : 0u);
  uint32_t rev = __brev(brk) >> 16;  // byte j -> age 15-j
  s.h1 = (s.h1 << 16) | (s.h0 >> 48);
  s.h0 = (s.h0 << 16) | (uint64_t)rev;
}

// The same roll from a packed unit (the coarse scatter: the counting pass already
// decided which windows count, so no breaker history is kept).
__device__ __forceinline__ void roll_push_codes(Roll& s, uint32_t codes, uint32_t nbits) {
  s.r2 = (s.r2 << 32) | (s.r1 >> 32);
  s.r1 = (s.r1 << 32) | (s.r0 >> 32);
  s.r0 = (s.r0 << 32) | (uint64_t)codes;
  s.n2 = (s.n2 << 32) | (s.n1 >> 32);
  s.n1 = (s.n1 << 32) | (s.n0 >> 32);
  s.n0 = (s.n0 << 32) | (uint64_t)nbits;
}

// The k-mer whose newest byte has age sh/2: kmer_shift ORs a byte's code bit 2 into
// the previous base's low bit, so only bytes inside the window (age >= sh/2)
// contribute their bit-2 plane, shifted up by one base.
template <typename KeyT>
__device__ __forceinline__ KeyT window_key(const Roll& s, int sh, const KeyT kmask);

template <>
__device__ __forceinline__ uint64_t window_key<uint64_t>(const Roll& s, int sh, const uint64_t kmask) {
  uint64_t x = sh ? ((s.r0 >> sh) | (s.r1 << (64 - sh))) : s.r0;
  uint64_t n = sh ? ((s.n0 >> sh) | (s.n1 << (64 - sh))) : s.n0;
  return (x | (n << 2)) & kmask;
}

template <>
__device__ __forceinline__ u128 window_key<u128>(const Roll& s, int sh, const u128 kmask) {
  uint64_t lo = sh ? ((s.r0 >> sh) | (s.r1 << (64 - sh))) : s.r0;
  uint64_t hi = sh ? ((s.r1 >> sh) | (s.r2 << (64 - sh))) : s.r1;
  uint64_t nlo = sh ? ((s.n0 >> sh) | (s.n1 << (64 - sh))) : s.n0;
  uint64_t nhi = sh ? ((s.n1 >> sh) | (s.n2 << (64 - sh))) : s.n1;
  const u128 x = ((u128)hi << 64) | lo;
  const u128 n = ((u128)nhi << 64) | nlo;
  return (x | (n << 2)) & kmask;
}

// window of ages [a, a+k) holds no breaker
__device__ __forceinline__ bool window_clear(const Roll& s, int a, int k) {
  uint64_t lo = a ? ((s.h0 >> a) | (s.h1 << (64 - a))) : s.h0;
  uint64_t m = k >= 64 ? ~0ull : ((1ull << k) - 1ull);
  return (lo & m) == 0;
}

// Reference record-start rule: a sequence line ending at `pos` (a newline) must be
// followed by '>' when its line start p satisfies p <= F - m.
__device__ void check_record_start(const uint8_t* __restrict__ buf, unsigned long long F, int m,
                                   unsigned long long pos, uint8_t next, uint32_t* err) {
  if (pos + 1 >= F || next == '>') return;
  long long lim = (long long)F - (long long)m;
  if (lim < 0) return;
  bool counts = true;
  if ((long long)pos > lim) {
    // line start <= lim  <=>  no newline in [lim, pos)
    for (long long q = lim; q < (long long)pos; q++)
      if (buf[q] == '\n') { counts = false; break; }
  }
  if (counts) atomicOr(err, ERR_FORMAT);
}

// Bucket of the window whose newest byte has age sh/2, for 64-bit keys whose bucket
// digits lie in the high word of the key (shift = 2k - digits >= 34): only the high words
// of the code and bit-2 planes are funnel-shifted.  The bit-2 plane's carry from the low
// word lands in bits 0-1 of the high word, below the digits.
__device__ __forceinline__ uint32_t window_bucket_hi(const Roll& s, int sh, int shift_hi, uint32_t hmask) {
  const uint32_t xh = __funnelshift_r((uint32_t)(s.r0 >> 32), (uint32_t)s.r1, sh);
  const uint32_t nh = __funnelshift_r((uint32_t)(s.n0 >> 32), (uint32_t)s.n1, sh);
  return ((xh | (nh << 2)) >> shift_hi) & hmask;
}

template <typename KeyT>
__device__ __forceinline__ void guarded_store(KeyT* __restrict__ out, uint32_t idx, KeyT v,
                                              unsigned long long cap, uint32_t* err) {
  if (idx < cap) out[idx] = v;
  else atomicOr(err, ERR_BOUNDS);
}

// Counting-pass threads: 1024 for 64-bit keys (more warps hide the decode's latency),
// 512 for 128-bit keys (whose windows need twice the registers)
template <typename KeyT>
struct CountCfg {
  static constexpr int T = sizeof(KeyT) == 8 ? 1024 : 512;
};

// Counting pass: per chunk, the bucket histogram of its windows (FASTB: the bucket is
// taken from the high words alone, see window_bucket_hi).
template <typename KeyT, bool FASTB>
__global__ void __launch_bounds__(CountCfg<KeyT>::T, 1)
k_extract(CountArgs a) {
  constexpr int NT = CountCfg<KeyT>::T;
  extern __shared__ uint32_t s_bins[];
  __shared__ uint32_t s_wpar[NT / 32];
  __shared__ uint32_t s_red[NT / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int NW = NT / 32;
  const int B = 1 << a.bbits;
  const int k = a.k;
  const int shift = 2 * k - a.bbits;
  const KeyT kmask = KeyOps<KeyT>::mask(2 * k);
  const bool drop_n = a.drop_n != 0;
  const uint8_t* __restrict__ buf = a.fasta;
  const unsigned long long F = a.F;
  const unsigned long long s0 = a.sc->s0;
  const int c = blockIdx.x;

  for (int i = tid; i < B; i += NT) s_bins[i] = 0;
  __syncthreads();

  const unsigned long long c0 = (unsigned long long)c * a.chunk;
  const unsigned long long c1 = min(c0 + a.chunk, F);
  uint32_t local = 0;
  const int warm_units = (k - 1 + 15) / 16;
  if (c0 < c1 && s0 < F) {
    uint32_t carry = (a.tile_nl[c0 / kTileBytes] ^ a.sc->nl_before_s0) & 1u;
    for (unsigned long long base = c0; base < c1; base += (unsigned long long)NT * kSegBytes) {
      const unsigned long long seg = base + (unsigned long long)tid * kSegBytes;
      const bool active = seg < c1;
      uint32_t w[4][4];
      uint32_t nlc = 0;
#pragma unroll
      for (int u = 0; u < 4; u++) {
        unsigned long long p = seg + 16ull * u;
        if (active && p < c1) {
          load_unit(buf, F, p, w[u]);
#pragma unroll
          for (int i = 0; i < 4; i++) nlc += __popc(__vcmpeq4(w[u][i], 0x0A0A0A0Au)) >> 3;
        } else {
          w[u][0] = w[u][1] = w[u][2] = w[u][3] = 0;
        }
      }
      // parity of the line count at the segment start (block XOR-scan)
      const unsigned bal = __ballot_sync(FULLMASK, nlc & 1u);
      if (lane == 0) s_wpar[warp] = __popc(bal) & 1u;
      __syncthreads();
      uint32_t wp = 0, tot = 0;
#pragma unroll
      for (int i = 0; i < NW; i++) {
        uint32_t x = s_wpar[i];
        tot ^= x;
        if (i < warp) wp ^= x;
      }
      __syncthreads();
      uint32_t pin = carry ^ wp ^ (__popc(bal & lanemask_lt()) & 1u);
      carry ^= tot;
      if (!active) continue;

      Roll s;
      s.r0 = s.r1 = s.r2 = 0;
      s.n0 = s.n1 = s.n2 = 0;
      s.h0 = s.h1 = 0;
      for (int u = warm_units; u >= 1; u--) {
        long long p = (long long)seg - 16ll * u;
        if (p < 0) continue;
        uint32_t ww[4];
        load_unit(buf, F, (unsigned long long)p, ww);
        roll_push(s, decode_unit(ww, drop_n), drop_n);
      }
      const unsigned long long g = seg / kSegBytes;
      unsigned long long counted = 0;  // windows counted, bit 16u + j
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const unsigned long long p = seg + 16ull * u;
        if (p >= c1) break;
        const UnitBits ub = decode_unit(w[u], drop_n);
        roll_push(s, ub, drop_n);
        a.unit_codes[u * a.nseg + g] = ub.codes;
        a.unit_nbits[u * a.nseg + g] = ub.nbits;
        // line parity per byte: exclusive prefix XOR of the newline bits
        uint32_t x = ub.nl;
        x ^= x << 1; x ^= x << 2; x ^= x << 4; x ^= x << 8;
        uint32_t ex = (x << 1) & 0xffffu;
        uint32_t odd = (pin ? ~ex : ex) & 0xffffu;
        pin ^= __popc(ub.nl) & 1u;
        uint32_t in = 0xffffu;
        if (p + 16 > F) in &= (1u << (uint32_t)(F - p)) - 1u;
        if (p < s0) in &= s0 - p >= 16 ? 0u : ~((1u << (uint32_t)(s0 - p)) - 1u);
        {
          uint32_t ends = ub.nl & odd & in;  // newlines that end sequence lines
          while (ends) {
            int q = __ffs(ends) - 1;
            ends &= ends - 1;
            // the byte after the newline, read from memory (it is in L1): picking it out of
            // w by a run-time index would keep w in local memory for the whole loop
            const uint8_t next = p + q + 1 < F ? __ldg(buf + p + q + 1) : (uint8_t)'>';
            check_record_start(buf, F, a.lmer_m, p + q, next, &a.sc->err);
          }
        }
        uint32_t v = odd & in & ~ub.nl;
        if (!v) continue;
        // all 16 windows of this unit span ages [0, k+15)
        const bool all_clear =
            k + 15 <= 64 ? window_clear(s, 0, k + 15)
                         : (s.h0 == 0 && (s.h1 & ((1ull << (k + 15 - 64)) - 1ull)) == 0);
#pragma unroll
        for (int j = 0; j < 16; j++) {
          if (!((v >> j) & 1u)) continue;
          const int age = 15 - j;
          if (!all_clear && !window_clear(s, age, k)) continue;
          uint32_t beta;
          if (FASTB) beta = window_bucket_hi(s, 2 * age, shift - 32, (uint32_t)(B - 1));
          else beta = (uint32_t)(window_key<KeyT>(s, 2 * age, kmask) >> shift);
          atomicAdd(&s_bins[beta], 1u);
          local++;
          counted |= 1ull << (16 * u + j);
        }
      }
      a.unit_windows[g] = counted;
    }
  }
  __syncthreads();
  {
    for (int i = tid; i < B; i += NT) a.counts[(size_t)c * B + i] = s_bins[i];
    uint32_t x = local;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(FULLMASK, x, o);
    if (lane == 0) s_red[warp] = x;
    __syncthreads();
    if (tid == 0) {
      unsigned long long tsum = 0;
      for (int i = 0; i < NW; i++) tsum += s_red[i];
      if (tsum) atomicAdd(&a.sc->n_windows, tsum);
    }
  }
}

// ----------------------------------------------------- two-pass partition of keys ---
// Pass 1 (k_scatter_coarse): roll the k-mers of a chunk again and append each key to a
// shared-memory ring of its coarse bucket (leading kCoarseBits bits); full 128-byte
// lines are flushed by warps to the chunk's segment of the coarse region, so global
// stores are whole lines instead of scattered 8/16-byte writes.
template <typename KeyT>
struct CoarseCfg {
  static constexpr int C = 1 << kCoarseBits;               // coarse buckets
  static constexpr int R = sizeof(KeyT) == 8 ? 128 : 64;    // ring slots per bucket
  static constexpr int FU = 128 / (int)sizeof(KeyT);        // keys per 128-byte line
  // threads: 1024 for 64-bit keys (the ring inserts and flushes are issue-bound and
  // gain from the extra warps), 512 for 128-bit keys (whose rings hold half the slots)
  static constexpr int T = sizeof(KeyT) == 8 ? 1024 : 512;
  // window positions per batch (T * BP keys between flushes): an average ring takes
  // about 80 of its 128 slots per batch for 64-bit keys and 35 of its 64 for 128-bit
  // keys (a ring that overflows sends its extra keys straight to global memory); flushing
  // every 8 positions instead cost 1.01 against 0.91 ms on the bacterial workload and
  // 5.09 against 4.29 ms on half the long-k workload
  static constexpr int BP = 16;
  static constexpr size_t smem = sizeof(KeyT) * C * R;
};

template <typename KeyT>
__device__ __forceinline__ void coarse_flush(KeyT* ring, uint32_t* w, uint32_t* f, const uint32_t* g,
                                             KeyT* __restrict__ out, bool final_flush,
                                             unsigned long long cap, uint32_t* err) {
  using CF = CoarseCfg<KeyT>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = CF::T / 32;
  for (int b = warp; b < CF::C; b += NW) {
    const uint32_t W = w[b];
    uint32_t Fv = f[b];
    KeyT* rb = ring + b * CF::R;
    const uint32_t gb = g[b];
    if (W - Fv > (uint32_t)CF::R) {
      // the ring overflowed this batch: keys past Fv+R went straight to global memory
      for (uint32_t x = lane; x < (uint32_t)CF::R; x += 32)
        guarded_store(out, gb + Fv + x, rb[(Fv + x) & (CF::R - 1)], cap, err);
      Fv = W;
    } else {
      while (W - Fv >= 32) {
        guarded_store(out, gb + Fv + lane, rb[(Fv + lane) & (CF::R - 1)], cap, err);
        Fv += 32;
      }
      if (W - Fv >= (uint32_t)CF::FU) {
        if (lane < CF::FU) guarded_store(out, gb + Fv + lane, rb[(Fv + lane) & (CF::R - 1)], cap, err);
        Fv += CF::FU;
      }
      if (final_flush && W > Fv) {
        if ((uint32_t)lane < W - Fv) guarded_store(out, gb + Fv + lane, rb[(Fv + lane) & (CF::R - 1)], cap, err);
        Fv = W;
      }
    }
    __syncwarp();
    if (lane == 0) f[b] = Fv;
  }
}

template <typename KeyT>
__global__ void __launch_bounds__(CoarseCfg<KeyT>::T, 1)
k_scatter_coarse(CountArgs a, const uint32_t* __restrict__ coff, KeyT* __restrict__ out) {
  using CF = CoarseCfg<KeyT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  KeyT* ring = reinterpret_cast<KeyT*>(smem_raw);
  __shared__ uint32_t s_w[CF::C], s_f[CF::C], s_g[CF::C];
  const int tid = threadIdx.x;
  const int k = a.k;
  const int cshift = 2 * k - a.cbits;  // coarse bucket = leading cbits bits
  const KeyT kmask = KeyOps<KeyT>::mask(2 * k);
  const unsigned long long F = a.F;
  const unsigned long long s0 = a.sc->s0;
  const int c = blockIdx.x;
  const int Cn = 1 << a.cbits;
  for (int i = tid; i < CF::C; i += CF::T) {
    s_w[i] = 0;
    s_f[i] = 0;
    s_g[i] = i < Cn ? coff[(size_t)c * Cn + i] : 0;
  }
  __syncthreads();
  const unsigned long long c0 = (unsigned long long)c * a.chunk;
  const unsigned long long c1 = min(c0 + a.chunk, F);
  const int warm_units = (k - 1 + 15) / 16;  // <= 4 (k <= 64): all in the previous segment
  const unsigned long long nseg = a.nseg;
  if (c0 < c1 && s0 < F) {
    for (unsigned long long base = c0; base < c1; base += (unsigned long long)CF::T * kSegBytes) {
      const unsigned long long seg = base + (unsigned long long)tid * kSegBytes;
      const bool active = seg < c1;
      const unsigned long long g = seg / kSegBytes;
      // the counting pass's packed units: codes, bit-2 plane and the windows it counted
      // (no FASTA decode, no line parity, no window checks here)
      Roll s;
      s.r0 = s.r1 = s.r2 = 0;
      s.n0 = s.n1 = s.n2 = 0;
      s.h0 = s.h1 = 0;
      unsigned long long counted = 0;
      if (active) {
        counted = __ldg(a.unit_windows + g);
        if (g > 0)
          for (int wu = warm_units; wu >= 1; wu--) {
            const unsigned long long q = (unsigned long long)(4 - wu) * nseg + g - 1;
            roll_push_codes(s, __ldg(a.unit_codes + q), __ldg(a.unit_nbits + q));
          }
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const bool live = active && seg + 16ull * u < c1;
        uint32_t v = 0;
        if (live) {
          const unsigned long long q = (unsigned long long)u * nseg + g;
          roll_push_codes(s, __ldg(a.unit_codes + q), __ldg(a.unit_nbits + q));
          v = (uint32_t)(counted >> (16 * u)) & 0xffffu;
        }
#pragma unroll
        for (int half = 0; half < 16 / CF::BP; half++) {
#pragma unroll
          for (int jj = 0; jj < CF::BP; jj++) {
            const int j = half * CF::BP + jj;
            if (!((v >> j) & 1u)) continue;
            const int age = 15 - j;
            const KeyT key = window_key<KeyT>(s, 2 * age, kmask);
            const uint32_t b = (uint32_t)(key >> cshift);
            const uint32_t pos = atomicAdd(&s_w[b], 1u);
            if (pos - s_f[b] < (uint32_t)CF::R) ring[b * CF::R + (pos & (CF::R - 1))] = key;
            else guarded_store(out, s_g[b] + pos, key, a.n_keys, &a.sc->err);
          }
          __syncthreads();
          coarse_flush<KeyT>(ring, s_w, s_f, s_g, out, false, a.n_keys, &a.sc->err);
          __syncthreads();
        }
      }
    }
  }
  __syncthreads();
  coarse_flush<KeyT>(ring, s_w, s_f, s_g, out, true, a.n_keys, &a.sc->err);
}

// Coarse offsets: coff[c][g] = start of chunk c's segment in coarse region g (the
// coarse region is the union of its fine buckets' regions); cstart[g] = region start;
// slice_start[g] = first pass-2 slice of region g.
__global__ void __launch_bounds__(256) k_coarse_offsets(const uint32_t* __restrict__ counts,
                                                        const uint32_t* __restrict__ bstart, int grid,
                                                        int bbits, int cbits, uint32_t* coff,
                                                        uint32_t* cstart, uint32_t* slice_start,
                                                        int slice_keys) {
  __shared__ uint32_t s_c[1 << kCoarseBits];
  const int c = blockIdx.x;
  const int B = 1 << bbits, Cn = 1 << cbits, fb = bbits - cbits;
  // a warp sums the 2^fb fine buckets of one coarse region at a time
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int g = warp; g < Cn; g += nw) {
    uint32_t sum = 0;
    for (int i = lane; i < (1 << fb); i += 32) sum += counts[(size_t)c * B + ((size_t)g << fb) + i];
    sum = __reduce_add_sync(FULLMASK, sum);
    if (lane == 0) s_c[g] = sum;
  }
  __syncthreads();
  for (int g = threadIdx.x; g < Cn; g += blockDim.x) coff[(size_t)c * Cn + g] = bstart[g << fb] + s_c[g];
  if (c == 0 && threadIdx.x == 0) {
    uint32_t acc = 0;
    for (int g = 0; g < Cn; g++) {
      cstart[g] = bstart[g << fb];
      slice_start[g] = acc;
      const uint32_t n = bstart[(g + 1) << fb] - bstart[g << fb];
      acc += (n + slice_keys - 1) / slice_keys;
    }
    cstart[Cn] = bstart[B];
    slice_start[Cn] = acc;
  }
}

// Pass 2 (k_scatter_fine): a slice of a coarse region (in chunk order) is counted by
// fine bucket in shared memory; one atomic per (slice, fine bucket) reserves a run in
// the bucket's region and every key goes to its run at a shared-memory-atomic rank.
// Keys stay in registers, so the CTA needs only three small tables and many CTAs fit
// an SM to hide the load latency.
template <typename KeyT>
struct FineCfg {
  static constexpr int T = 512;                             // threads
  static constexpr int PT = sizeof(KeyT) == 8 ? 16 : 8;      // keys per thread
  static constexpr int S = T * PT;                          // keys per slice (64 KB)
  static constexpr int FBMAX = 1 << (kMaxPartBits - kCoarseBits);  // fine buckets per coarse
  static constexpr size_t smem = sizeof(KeyT) * S;
};

template <typename KeyT>
__global__ void __launch_bounds__(512, 2) k_scatter_fine(const KeyT* __restrict__ in,
                                                        const uint32_t* __restrict__ cstart,
                                                        const uint32_t* __restrict__ slice_start,
                                                        uint32_t* fcur, KeyT* __restrict__ out,
                                                        int k, int bbits, int cbits, uint32_t* ticket,
                                                        unsigned long long cap, uint32_t* err) {
  using FC = FineCfg<KeyT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  KeyT* stage = reinterpret_cast<KeyT*>(smem_raw);  // the slice grouped by fine bucket
  __shared__ uint32_t s_hist[FC::FBMAX], s_loff[FC::FBMAX], s_goff[FC::FBMAX], s_fill[FC::FBMAX];
  __shared__ uint32_t s_warp[33];
  __shared__ uint32_t s_slice, s_g;
  const int tid = threadIdx.x;
  const int Cn = 1 << cbits, fb = bbits - cbits, FB = 1 << fb;
  const int fshift = 2 * k - bbits;
  const uint32_t nslices = slice_start[Cn];
  while (true) {
    __syncthreads();
    if (tid == 0) {
      s_slice = atomicAdd(ticket, 1u);
      if (s_slice < nslices) {
        int lo = 0, hi = Cn - 1;  // last g with slice_start[g] <= slice
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (slice_start[mid] <= s_slice) lo = mid; else hi = mid - 1;
        }
        s_g = lo;
      }
    }
    for (int i = tid; i < FB; i += FC::T) { s_hist[i] = 0; s_fill[i] = 0; }
    __syncthreads();
    const uint32_t sl = s_slice;
    if (sl >= nslices) break;
    const uint32_t g = s_g;
    const uint32_t r0 = cstart[g] + (sl - slice_start[g]) * FC::S;
    const uint32_t r1 = min(r0 + (uint32_t)FC::S, cstart[g + 1]);
    const uint32_t m = r1 - r0;
    KeyT xs[FC::PT];
    uint32_t fs[FC::PT];
#pragma unroll
    for (int q = 0; q < FC::PT; q++) {
      const uint32_t i = q * FC::T + tid;
      xs[q] = i < m ? in[r0 + i] : (KeyT)0;
    }
#pragma unroll
    for (int q = 0; q < FC::PT; q++) {
      const uint32_t i = q * FC::T + tid;
      fs[q] = (uint32_t)(xs[q] >> fshift) & (uint32_t)(FB - 1);
      if (i < m) atomicAdd(&s_hist[fs[q]], 1u);
    }
    __syncthreads();
    {
      // each thread owns a contiguous run of FB / T fine buckets (at least one)
      constexpr int FPT = (FC::FBMAX + FC::T - 1) / FC::T;
      const int per = (FB + FC::T - 1) / FC::T;
      const int f0 = min(FB, tid * per);
      uint32_t hv[FPT], sum = 0;
#pragma unroll
      for (int q = 0; q < FPT; q++) {
        hv[q] = (q < per && f0 + q < FB) ? s_hist[f0 + q] : 0u;
        sum += hv[q];
      }
      uint32_t tot;
      uint32_t ex = block_exclusive_sum(sum, s_warp, tot);
#pragma unroll
      for (int q = 0; q < FPT; q++) {
        if (q < per && f0 + q < FB) {
          s_loff[f0 + q] = ex;
          s_goff[f0 + q] = hv[q] ? atomicAdd(&fcur[(g << fb) + f0 + q], hv[q]) : 0u;
          ex += hv[q];
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < FC::PT; q++) {
      const uint32_t i = q * FC::T + tid;
      if (i < m) stage[s_loff[fs[q]] + atomicAdd(&s_fill[fs[q]], 1u)] = xs[q];
    }
    __syncthreads();
    // runs of one fine bucket are contiguous in `stage` and in `out`: coalesced stores
    for (uint32_t i = tid; i < m; i += FC::T) {
      const KeyT x = stage[i];
      const uint32_t f = (uint32_t)(x >> fshift) & (uint32_t)(FB - 1);
      guarded_store(out, s_goff[f] + (i - s_loff[f]), x, cap, err);
    }
  }
}

// Wide fan-out (2048 fine buckets per coarse region): a slice of 192 KB is
// staged in shared memory so that each fine bucket still gets runs of several keys.
// The slice is read twice (counting, then placing; the second read mostly hits L2),
// four keys per thread per round.
template <typename KeyT>
struct FineBigCfg {
  static constexpr int T = 1024;
  static constexpr int S = (192 * 1024) / (int)sizeof(KeyT);  // keys per slice
  static constexpr int PR = 4;                                 // keys per thread per round
  static constexpr size_t smem = sizeof(KeyT) * S;
};

template <typename KeyT>
__global__ void __launch_bounds__(1024, 1) k_scatter_fine_big(const KeyT* __restrict__ in,
                                                             const uint32_t* __restrict__ cstart,
                                                             const uint32_t* __restrict__ slice_start,
                                                             uint32_t* fcur, KeyT* __restrict__ out,
                                                             int k, int bbits, int cbits, uint32_t* ticket,
                                                             unsigned long long cap, uint32_t* err) {
  using FC = FineBigCfg<KeyT>;
  constexpr int FBMAX = FineCfg<KeyT>::FBMAX;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  KeyT* stage = reinterpret_cast<KeyT*>(smem_raw);
  __shared__ uint32_t s_hist[FBMAX], s_loff[FBMAX], s_goff[FBMAX], s_fill[FBMAX];
  __shared__ uint32_t s_warp[33];
  __shared__ uint32_t s_slice, s_g;
  const int tid = threadIdx.x;
  const int Cn = 1 << cbits, fb = bbits - cbits, FB = 1 << fb;
  const int fshift = 2 * k - bbits;
  // the region tables live in shared memory: the slice -> region search of every slice
  // reads no global memory
  __shared__ uint32_t s_ss[(1 << kCoarseBits) + 1], s_cs[(1 << kCoarseBits) + 1];
  for (int i = tid; i <= Cn; i += FC::T) {
    s_ss[i] = slice_start[i];
    s_cs[i] = cstart[i];
  }
  const uint32_t nslices = slice_start[Cn];
  while (true) {
    __syncthreads();
    if (tid == 0) {
      s_slice = atomicAdd(ticket, 1u);
      if (s_slice < nslices) {
        int lo = 0, hi = Cn - 1;  // last g with slice_start[g] <= slice
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (s_ss[mid] <= s_slice) lo = mid; else hi = mid - 1;
        }
        s_g = lo;
      }
    }
    for (int i = tid; i < FB; i += FC::T) { s_hist[i] = 0; s_fill[i] = 0; }
    __syncthreads();
    const uint32_t sl = s_slice;
    if (sl >= nslices) break;
    const uint32_t g = s_g;
    const uint32_t r0 = s_cs[g] + (sl - s_ss[g]) * FC::S;
    const uint32_t r1 = min(r0 + (uint32_t)FC::S, s_cs[g + 1]);
    const uint32_t m = r1 - r0;
    for (uint32_t i0 = 0; i0 < m; i0 += FC::PR * FC::T) {
      KeyT xs[FC::PR];
#pragma unroll
      for (int q = 0; q < FC::PR; q++) {
        const uint32_t i = i0 + q * FC::T + tid;
        xs[q] = i < m ? in[r0 + i] : (KeyT)0;
      }
#pragma unroll
      for (int q = 0; q < FC::PR; q++)
        if (i0 + q * FC::T + tid < m) atomicAdd(&s_hist[(uint32_t)(xs[q] >> fshift) & (uint32_t)(FB - 1)], 1u);
    }
    __syncthreads();
    {
      constexpr int FPT = (FBMAX + FC::T - 1) / FC::T;
      const int per = (FB + FC::T - 1) / FC::T;
      const int f0 = min(FB, tid * per);
      uint32_t hv[FPT], sum = 0;
#pragma unroll
      for (int q = 0; q < FPT; q++) {
        hv[q] = (q < per && f0 + q < FB) ? s_hist[f0 + q] : 0u;
        sum += hv[q];
      }
      uint32_t tot;
      uint32_t ex = block_exclusive_sum(sum, s_warp, tot);
#pragma unroll
      for (int q = 0; q < FPT; q++) {
        if (q < per && f0 + q < FB) {
          s_loff[f0 + q] = ex;
          s_goff[f0 + q] = hv[q] ? atomicAdd(&fcur[(g << fb) + f0 + q], hv[q]) : 0u;
          ex += hv[q];
        }
      }
    }
    __syncthreads();
    for (uint32_t i0 = 0; i0 < m; i0 += FC::PR * FC::T) {
      KeyT xs[FC::PR];
#pragma unroll
      for (int q = 0; q < FC::PR; q++) {
        const uint32_t i = i0 + q * FC::T + tid;
        xs[q] = i < m ? in[r0 + i] : (KeyT)0;
      }
#pragma unroll
      for (int q = 0; q < FC::PR; q++) {
        if (i0 + q * FC::T + tid < m) {
          const uint32_t f = (uint32_t)(xs[q] >> fshift) & (uint32_t)(FB - 1);
          stage[s_loff[f] + atomicAdd(&s_fill[f], 1u)] = xs[q];
        }
      }
    }
    __syncthreads();
    for (uint32_t i = tid; i < m; i += FC::T) {
      const KeyT x = stage[i];
      const uint32_t f = (uint32_t)(x >> fshift) & (uint32_t)(FB - 1);
      guarded_store(out, s_goff[f] + (i - s_loff[f]), x, cap, err);
    }
  }
}

int fine_slice_keys(int wide, int fb) {
  if (fb >= 11) return wide ? FineBigCfg<u128>::S : FineBigCfg<uint64_t>::S;
  return wide ? FineCfg<u128>::S : FineCfg<uint64_t>::S;
}

// Fine bucket sizes when the partition has more digits than the counting pass's
// histogram: slices of each coarse region are counted by their fine digits in shared
// memory and added to bcount[(g << fb) + f].
template <typename KeyT>
__global__ void __launch_bounds__(512, 2) k_fine_count(const KeyT* __restrict__ in,
                                                   const uint32_t* __restrict__ cstart,
                                                   const uint32_t* __restrict__ slice_start,
                                                   uint32_t* bcount, int k, int bbits, int cbits,
                                                   uint32_t* ticket, uint32_t slice_keys) {
  using FC = FineCfg<KeyT>;
  __shared__ uint32_t s_hist[FC::FBMAX];
  __shared__ uint32_t s_slice, s_g;
  const int tid = threadIdx.x;
  const int Cn = 1 << cbits, fb = bbits - cbits, FB = 1 << fb;
  const int fshift = 2 * k - bbits;
  // the region tables live in shared memory: the slice -> region search of every slice
  // reads no global memory
  __shared__ uint32_t s_ss[(1 << kCoarseBits) + 1], s_cs[(1 << kCoarseBits) + 1];
  for (int i = tid; i <= Cn; i += (int)blockDim.x) {
    s_ss[i] = slice_start[i];
    s_cs[i] = cstart[i];
  }
  const uint32_t nslices = slice_start[Cn];
  while (true) {
    __syncthreads();
    if (tid == 0) {
      s_slice = atomicAdd(ticket, 1u);
      if (s_slice < nslices) {
        int lo = 0, hi = Cn - 1;  // last g with slice_start[g] <= slice
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (s_ss[mid] <= s_slice) lo = mid; else hi = mid - 1;
        }
        s_g = lo;
      }
    }
    for (int i = tid; i < FB; i += (int)blockDim.x) s_hist[i] = 0;
    __syncthreads();
    const uint32_t sl = s_slice;
    if (sl >= nslices) break;
    const uint32_t g = s_g;
    const uint32_t r0 = s_cs[g] + (sl - s_ss[g]) * slice_keys;
    const uint32_t r1 = min(r0 + slice_keys, s_cs[g + 1]);
    for (uint32_t i = r0 + tid; i < r1; i += blockDim.x)
      atomicAdd(&s_hist[(uint32_t)(in[i] >> fshift) & (uint32_t)(FB - 1)], 1u);
    __syncthreads();
    for (int f = tid; f < FB; f += (int)blockDim.x)
      if (s_hist[f]) atomicAdd(&bcount[((uint32_t)g << fb) + f], s_hist[f]);
  }
}

// counts[c][b] -> exclusive prefix over chunks (in place); totals into bstart[b].
__global__ void __launch_bounds__(256) k_col_prefix(uint32_t* counts, int grid, int B, uint32_t* totals) {
  // a CTA takes 32 bucket columns; its 8 warps take consecutive bands of chunk rows,
  // sum them (coalesced 128-byte rows), and take their band's offset from the sums of
  // the bands above
  __shared__ uint32_t s_band[8][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = blockIdx.x * 32 + lane;
  const int per = (grid + 7) / 8;
  const int c0 = min(grid, warp * per), c1 = min(grid, c0 + per);
  uint32_t sum = 0;
  if (b < B)
    for (int c = c0; c < c1; c++) sum += counts[(size_t)c * B + b];
  s_band[warp][lane] = sum;
  __syncthreads();
  uint32_t run = 0;
  for (int w = 0; w < warp; w++) run += s_band[w][lane];
  if (b < B) {
    for (int c = c0; c < c1; c++) {
      const size_t i = (size_t)c * B + b;
      const uint32_t v = counts[i];
      counts[i] = run;
      run += v;
    }
    if (warp == 7) totals[b] = run;  // the last band ends at the last chunk
  }
}

// Exclusive prefix of bstart[0..B) in place, bstart[B] = total.  One block: each
// thread sums a contiguous run of ceil(B / 1024) entries, one block scan gives the run
// offsets, and each thread writes its run (B up to 2^18).
__global__ void __launch_bounds__(1024) k_bucket_prefix(uint32_t* bstart, int B) {
  __shared__ uint32_t s_warp[33];
  const int per = (B + (int)blockDim.x - 1) / (int)blockDim.x;
  const int b0 = min(B, (int)threadIdx.x * per), b1 = min(B, b0 + per);
  uint32_t sum = 0;
  for (int b = b0; b < b1; b++) sum += bstart[b];
  uint32_t tot;
  uint32_t run = block_exclusive_sum(sum, s_warp, tot);
  for (int b = b0; b < b1; b++) {
    const uint32_t v = bstart[b];
    bstart[b] = run;
    run += v;
  }
  if (threadIdx.x == 0) bstart[B] = tot;
}

// ------------------------------------------------------------- per-bucket table ------
template <typename KeyT>
struct BucketCfg;
template <>
struct BucketCfg<uint64_t> {
  static constexpr int H = 8192;
};
template <>
struct BucketCfg<u128> {
  static constexpr int H = 4096;
};

template <typename KeyT>
struct BucketSmem {
  static constexpr int H = BucketCfg<KeyT>::H;
  static constexpr int NW = kBucketThreads / 32;
  static constexpr size_t off_key = 0;
  static constexpr size_t off_cnt = off_key + sizeof(KeyT) * H;
  static constexpr size_t off_wc = off_cnt + sizeof(uint32_t) * H;
  static constexpr size_t off_hist = off_wc + sizeof(uint16_t) * NW * 256;
  static constexpr size_t bytes = off_hist + sizeof(uint32_t) * kHistSmem;
};

// Insert (r, c) into the open-addressing table: 0 = r was present, 1 = r is new,
// 2 = no slot within kMaxProbe probes (treated as an overflow of the sub-range).
constexpr int kMaxProbe = 256;
template <typename KeyT>
__device__ __forceinline__ int hash_insert(KeyT* skey, uint32_t* scnt, uint32_t hmask, KeyT r, uint32_t c) {
  const KeyT EMPTY = ~(KeyT)0;
  uint32_t h = (uint32_t)(KeyOps<KeyT>::hash(r) >> 40) & hmask;
  for (int probe = 0; probe < kMaxProbe; probe++) {
    KeyT cur = *(volatile KeyT*)&skey[h];
    if (cur == r) {
      atomicAdd(&scnt[h], c);
      return 0;
    }
    if (cur == EMPTY) {
      KeyT old = KeyOps<KeyT>::cas(&skey[h], EMPTY, r);
      if (old == EMPTY || old == r) {
        atomicAdd(&scnt[h], c);
        return old == EMPTY ? 1 : 0;
      }
    }
    h = (h + 1) & hmask;
  }
  return 2;
}

// One table row, plus its count in the bucket's histogram of small counts (sbsmall, folded
// into the count histogram when the bucket ends) or in the count histogram (counts below t).
template <typename KeyT>
__device__ __forceinline__ void emit_row(const BucketArgs& a, KeyT* __restrict__ tkeys, unsigned long long row,
                                         KeyT key, uint32_t cnt, uint32_t* shist, uint32_t* sbsmall) {
  if (row < a.cap) {
    tkeys[row] = key;
    a.tcounts[row] = cnt;
  } else {
    atomicOr(&a.sc->err, ERR_BOUNDS);
  }
  if (cnt < (uint32_t)kSmallCounts) {
    atomicAdd(&sbsmall[cnt], 1u);
  } else if (cnt < (uint32_t)a.t) {
    if (cnt < (uint32_t)kHistSmem) atomicAdd(&shist[cnt], 1u);
    else atomicAdd(&a.hist[cnt], 1ull);
  }
}

// Rows [base+acc, base+acc+u) of a bucket from the sorted on-chip run (sk, sc).
template <typename KeyT>
__device__ void write_bucket_rows(const KeyT* sk, const uint32_t* sc, uint32_t u, const BucketArgs& a,
                                  uint32_t beta, int rem, uint32_t base, uint32_t acc,
                                  KeyT* __restrict__ tkeys, uint32_t* shist, uint32_t* sbsmall) {
  const KeyT hi_bits = KeyOps<KeyT>::shl((KeyT)beta, rem);
  for (uint32_t i = threadIdx.x; i < u; i += kBucketThreads)
    emit_row<KeyT>(a, tkeys, (unsigned long long)base + acc + i, hi_bits | sk[i], sc[i], shist, sbsmall);
}

// Chunk items of the giant buckets (one thread per bucket): a bucket of at least
// kGiantKeys keys reserves floor(n / kChunkKeys) consecutive chunk items, gfirst[b] the
// first and gcount[b] how many, and marks them as its own in chunk_bucket; the number
// of chunk items ends in sc->n_chunk_items (zero beforehand); gdone = 0.
__global__ void __launch_bounds__(256) k_giant_chunks(const uint32_t* __restrict__ bstart, int B,
                                                      uint32_t* gfirst, uint32_t* gcount,
                                                      uint32_t* chunk_bucket, uint32_t* gdone, Scalars* sc) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const uint32_t n = bstart[b + 1] - bstart[b];
  const uint32_t c = n >= kGiantKeys ? n / kChunkKeys : 0u;
  gdone[b] = 0;
  gcount[b] = c;
  uint32_t g0 = 0;
  if (c) {
    g0 = atomicAdd(&sc->n_chunk_items, c);
    for (uint32_t i = 0; i < c; i++) chunk_bucket[g0 + i] = (uint32_t)b;
  }
  gfirst[b] = g0;
}

// One chunk item: keys [cb, cb + kChunkKeys) of a giant bucket are aggregated on chip.
// When their distinct keys fit half the table they are written back over the chunk's
// own slots as (remainder, count) pairs -- remainders in slots [cb, cb + u), counts as
// uint32 from slot cb + kChunkKeys / 2 on -- and chunk_u = u; otherwise the chunk keeps
// its keys and chunk_u = kChunkRaw.  The bucket item reads the pairs in place of the
// keys, so a heavy k-mer's copies are summed by many CTAs instead of one.
template <typename KeyT>
__device__ __forceinline__ void aggregate_chunk(const BucketArgs& a, KeyT* keys_rw, unsigned long long cb, uint32_t item,
                                uint32_t beta, KeyT rmask, KeyT* skey, uint32_t* scnt, uint32_t* s_warp,
                                uint32_t* s_flag, uint32_t* s_cnt) {
  constexpr int H = BucketCfg<KeyT>::H;
  constexpr int PF = 4;
  const KeyT EMPTY = ~(KeyT)0;
  const int tid = threadIdx.x, lane = tid & 31;
  for (uint32_t i = tid; i < (uint32_t)H; i += kBucketThreads) {
    skey[i] = EMPTY;
    scnt[i] = 0;
  }
  if (tid == 0) {
    *s_flag = 0;
    *s_cnt = 0;
  }
  __syncthreads();
  for (uint32_t i0 = 0; i0 < (uint32_t)kChunkKeys; i0 += PF * kBucketThreads) {
    if (*(volatile uint32_t*)s_flag) break;
    KeyT rr[PF];
#pragma unroll
    for (int q = 0; q < PF; q++) rr[q] = keys_rw[cb + i0 + q * kBucketThreads + tid] & rmask;
    uint32_t fresh = 0;
#pragma unroll
    for (int q = 0; q < PF; q++) {
      const int res = hash_insert<KeyT>(skey, scnt, H - 1, rr[q], 1u);
      if (res == 2) *s_flag = 1;
      fresh += res == 1;
    }
    fresh = __reduce_add_sync(FULLMASK, fresh);
    if (lane == 0 && fresh && atomicAdd(s_cnt, fresh) + fresh > (uint32_t)(H / 2)) *s_flag = 1;
  }
  __syncthreads();
  const bool raw = *(volatile uint32_t*)s_flag != 0;
  constexpr int SPT = H / kBucketThreads;
  KeyT rk[SPT];
  uint32_t rc[SPT];
  uint32_t occ = 0;
#pragma unroll
  for (int q = 0; q < SPT; q++) {
    rk[q] = skey[q * kBucketThreads + tid];
    rc[q] = scnt[q * kBucketThreads + tid];
    occ += rk[q] != EMPTY;
  }
  uint32_t u;
  uint32_t off = block_exclusive_sum(occ, s_warp, u);  // ends with a barrier: every key was read
  if (!raw && u <= (uint32_t)(H / 2)) {
    uint32_t* pc = reinterpret_cast<uint32_t*>(keys_rw + cb + kChunkKeys / 2);
#pragma unroll
    for (int q = 0; q < SPT; q++) {
      if (rk[q] != EMPTY) {
        keys_rw[cb + off] = rk[q];
        pc[off] = rc[q];
        off++;
      }
    }
  } else {
    u = kChunkRaw;
  }
  if (tid == 0) a.chunk_u[item] = u;
  __threadfence();
  __syncthreads();
  if (tid == 0) atomicAdd(&a.gdone[beta], 1u);
}

// A giant bucket's item waits (bounded) until its chunk items are done and returns the
// entries it will read: the chunks' pairs (or keys, where a chunk stayed raw) and the
// keys after the last chunk.  On expiry it sets ERR_LOOKBACK and *s_fail.
__device__ __forceinline__ uint32_t giant_entries(const BucketArgs& a, uint32_t beta, uint32_t n, uint32_t g0,
                                               uint32_t nch, uint32_t* s_warp, uint32_t* s_fail) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    int spins = 0;
    const int max_spins = spin_limit(a.spin_limit);
    while (ld_acquire_u32(&a.gdone[beta]) < nch) {
      if (++spins >= max_spins) {
        atomicOr(&a.sc->err, ERR_LOOKBACK);
        *s_fail = 1;
        break;
      }
      __nanosleep(spins < 64 ? 32 : 256);
    }
  }
  __syncthreads();
  uint32_t part = 0;
  for (uint32_t j = tid; j < nch; j += kBucketThreads) {
    const uint32_t cu = __ldcg(&a.chunk_u[g0 + j]);
    part += cu == kChunkRaw ? (uint32_t)kChunkKeys : cu;
  }
  uint32_t tot;
  block_exclusive_sum(part, s_warp, tot);
  return tot + (n - nch * (uint32_t)kChunkKeys);
}

// One hash pass of a giant bucket's sub-range [lo, hi): chunk by chunk (pairs carry
// their counts), then the tail keys.  Loads go through L2, as other CTAs wrote the
// pairs during this kernel.
template <typename KeyT>
__device__ __forceinline__ void giant_pass(const BucketArgs& a, const KeyT* keys_rw, uint32_t base, uint32_t n,
                                        uint32_t g0, uint32_t nch, bool whole, KeyT lo, KeyT hi, KeyT rmask,
                                        KeyT* skey, uint32_t* scnt, uint32_t hmask, uint32_t ulimit,
                                        uint32_t* s_ovf, uint32_t* s_unew) {
  const int tid = threadIdx.x, lane = tid & 31;
  for (uint32_t j = 0; j <= nch; j++) {
    if (*(volatile uint32_t*)s_ovf) break;
    const unsigned long long cb = (unsigned long long)base + (unsigned long long)j * kChunkKeys;
    uint32_t len = n - nch * (uint32_t)kChunkKeys;
    bool pairs = false;
    if (j < nch) {
      const uint32_t cu = __ldcg(&a.chunk_u[g0 + j]);
      pairs = cu != kChunkRaw;
      len = pairs ? cu : (uint32_t)kChunkKeys;
    }
    const uint32_t* pc = reinterpret_cast<const uint32_t*>(keys_rw + cb + kChunkKeys / 2);
    uint32_t fresh = 0;
    for (uint32_t i = tid; i < len; i += kBucketThreads) {
      const KeyT r = ldcg_key(keys_rw + cb + i) & rmask;
      if (whole || (!(r < lo) && r < hi)) {
        const int res = hash_insert<KeyT>(skey, scnt, hmask, r, pairs ? __ldcg(pc + i) : 1u);
        if (res == 2) *s_ovf = 1;
        fresh += res == 1;
      }
    }
    fresh = __reduce_add_sync(FULLMASK, fresh);
    if (lane == 0 && fresh && atomicAdd(s_unew, fresh) + fresh > ulimit) *s_ovf = 1;
  }
}

// Per bucket: aggregate the bucket's keys into (remainder, count) in an on-chip
// hash table, radix-sort the distinct remainders and write them as table rows at
// the bucket's own key range [bstart, bstart + u) ("sparse" table: no inter-bucket
// dependency).  When the distinct keys of a bucket exceed the on-chip capacity the
// bucket is counted in 2^slog sub-passes, each taking the keys whose next slog
// remainder bits equal the sub-pass index (so sub-passes come out in key order).
template <typename KeyT, bool GIANT>
__global__ void __launch_bounds__(kBucketThreads, 2) k_bucket_table(BucketArgs a) {
  using SM = BucketSmem<KeyT>;
  constexpr int H = SM::H;
  constexpr int NW = SM::NW;
  constexpr int HALF = H / 2;
  constexpr int RMAX = (HALF + kBucketThreads - 1) / kBucketThreads;  // radix rounds per warp
  extern __shared__ __align__(16) unsigned char smem[];
  KeyT* skey = reinterpret_cast<KeyT*>(smem + SM::off_key);
  uint32_t* scnt = reinterpret_cast<uint32_t*>(smem + SM::off_cnt);
  uint16_t* wc = reinterpret_cast<uint16_t*>(smem + SM::off_wc);
  uint32_t* shist = reinterpret_cast<uint32_t*>(smem + SM::off_hist);
  __shared__ uint32_t s_warp[33];
  __shared__ uint32_t s_beta, s_ovf, s_fail, s_nb[2], s_unew;
  __shared__ int s_sp;
  __shared__ KeyT s_stk_lo[kBucketStack];  // pending sub-ranges [lo, hi) of the bucket
  __shared__ KeyT s_stk_hi[kBucketStack];
  __shared__ KeyT s_split[kSplitWays];
  __shared__ float s_ratio;
  __shared__ uint32_t s_bsmall[kSmallCounts];  // the current bucket's rows by small count

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int B = 1 << a.bbits;
  const int rem = 2 * a.k - a.bbits;  // remainder bits below the bucket id
  const KeyT rmask = KeyOps<KeyT>::mask(rem);
  const KeyT rtop = KeyOps<KeyT>::shl((KeyT)1, rem);  // end of the remainder range
  const KeyT EMPTY = ~(KeyT)0;
  const KeyT* __restrict__ keys = reinterpret_cast<const KeyT*>(a.keys);
  KeyT* __restrict__ tkeys = reinterpret_cast<KeyT*>(a.tkeys);
  const int hbins = a.t < kHistSmem ? a.t : kHistSmem;
  for (int i = tid; i < hbins; i += kBucketThreads) shist[i] = 0;
  if (tid < kSmallCounts) s_bsmall[tid] = 0;
  // running distinct/keys ratio of this CTA's buckets; read sets at 20x-80x coverage
  // with sub-percent errors start near 0.2 (a high guess splits the first buckets
  // needlessly, a low one costs one overflowing pass)
  if (tid == 0) s_ratio = 0.2f;
  const int slog_max = rem < 4 ? rem : 4;  // initial split guess (<= 16 sub-ranges)

  // Work tickets: the chunk items of giant buckets first (tickets [0, nci)), then the
  // buckets.  A giant bucket waits (bounded) until its chunks are reduced; every chunk
  // ticket was taken before any bucket ticket, by a CTA that waits on nothing, so the
  // wait ends.  The next ticket and its bucket's extent are fetched while the current
  // one is counted.
  // Two instantiations are launched back to back and exactly one of them works: GIANT
  // = false when the partition has no giant bucket (it carries none of their code, so
  // the common case keeps its registers), GIANT = true otherwise, taking the chunk
  // items first and then every bucket, so the giant buckets' own passes overlap the
  // other buckets.
  const uint32_t ng = a.gfirst ? a.sc->n_chunk_items : 0u;
  if ((ng != 0) != GIANT) return;
  const uint32_t nci = GIANT ? ng : 0u;
  const uint32_t nt = nci + (uint32_t)B;
  uint32_t* ticket = &a.sc->ticket_bucket;
  KeyT* keys_rw = reinterpret_cast<KeyT*>(a.keys);
  uint32_t next_t = 0, next_base = 0, next_end = 0;
  auto bucket_of = [&](uint32_t tk) { return tk - nci; };
  if (tid == 0) {
    next_t = atomicAdd(ticket, 1u);
    if ((!GIANT || next_t >= nci) && next_t < nt) {
      const uint32_t b = bucket_of(next_t);
      next_base = a.bstart[b];
      next_end = a.bstart[b + 1];
    }
  }
  while (true) {
    __syncthreads();
    if (tid == 0) {
      s_beta = next_t;
      s_nb[0] = next_base;
      s_nb[1] = next_end;
      if (next_t < nt) {
        next_t = atomicAdd(ticket, 1u);
        if ((!GIANT || next_t >= nci) && next_t < nt) {
          const uint32_t b = bucket_of(next_t);
          next_base = a.bstart[b];
          next_end = a.bstart[b + 1];
        }
      }
    }
    __syncthreads();
    const uint32_t t = s_beta;
    if (t >= nt) break;
    if (GIANT && t < nci) {
      if (tid == 0) {
        const uint32_t gb = a.chunk_bucket[t];
        s_nb[0] = gb;
        s_nb[1] = a.bstart[gb] + (t - a.gfirst[gb]) * (uint32_t)kChunkKeys;
      }
      __syncthreads();
      aggregate_chunk<KeyT>(a, keys_rw, s_nb[1], t, s_nb[0], rmask, skey, scnt, s_warp, &s_ovf, &s_unew);
      continue;
    }
    const uint32_t beta = bucket_of(t);
    const uint32_t base = s_nb[0];
    const uint32_t n = s_nb[1] - base;
    if (tid == 0) s_fail = 0;
    if (n == 0) {
      if (tid == 0) a.tu[beta] = 0;
      if (tid < kSmallCounts && a.bsmall) a.bsmall[(size_t)beta * kSmallCounts + tid] = 0;
      continue;
    }
    // a giant bucket reads its chunks' pairs (or keys, where a chunk stayed raw) and the
    // keys after its last chunk; n_eff = entries it reads
    const uint32_t g0 = GIANT ? a.gfirst[beta] : 0u;
    const uint32_t nch = GIANT ? a.gcount[beta] : 0u;
    const uint32_t n_eff = nch ? giant_entries(a, beta, n, g0, nch, s_warp, &s_fail) : n;
    // Sub-ranges of the bucket are counted one at a time, in key order.  A sub-range
    // is an interval [lo, hi) of remainders.  The first split guesses from the
    // distinct/keys ratio seen so far; a sub-range whose distinct keys overflow the
    // on-chip table is cut at quantiles of a sample of its distinct keys, so skewed
    // buckets (a heavy k-mer and its error variants) split evenly.
    int slog = 0;
    while (slog < slog_max && (float)(n_eff >> slog) * s_ratio * 1.2f > (float)HALF) slog++;
    if (tid == 0 && s_fail) s_sp = 0;
    if (tid == 0 && !s_fail) {
      s_sp = 0;
      const int psh0 = rem - slog;
      for (int j = (1 << slog) - 1; j >= 0; j--) {
        s_stk_lo[s_sp] = KeyOps<KeyT>::shl((KeyT)(uint32_t)j, psh0);
        s_stk_hi[s_sp] = KeyOps<KeyT>::shl((KeyT)(uint32_t)(j + 1), psh0);
        s_sp++;
      }
    }
    uint32_t acc = 0;
    int attempts = 0;
    __syncthreads();
    bool failed = s_fail != 0;  // a giant bucket whose chunks did not finish in time
    while (s_sp > 0) {
      const KeyT lo = s_stk_lo[s_sp - 1];
      const KeyT hi = s_stk_hi[s_sp - 1];
      __syncthreads();
      if (tid == 0) s_sp--;
      if (++attempts > kMaxBucketAttempts) { failed = true; break; }
      const bool whole = lo == (KeyT)0 && hi == rtop;
      // bits below the interval's common prefix (all its keys share the bits above)
      const KeyT span = lo ^ (hi - (KeyT)1);
      const int psh = span == (KeyT)0 ? 0 : KeyOps<KeyT>::top_bit(span) + 1;
      // table sized for the distinct keys expected (2.5x), at least 1024 slots; an
      // overflow splits the sub-range
      uint32_t Heff = 1024;
      {
        const float uest = (float)n_eff * s_ratio * 2.5f;
        while ((float)Heff < uest && Heff < (uint32_t)H) Heff <<= 1;
        if (!whole) Heff = H;
      }
      const uint32_t hmask = Heff - 1;
      for (uint32_t i = tid; i < Heff; i += kBucketThreads) {
        skey[i] = EMPTY;
        scnt[i] = 0;
      }
      // sort bins (counts, then fill cursors) of the distinct remainders: the top
      // bits below the sub-range's common prefix
      const int dbits = psh < kSortBinBits ? psh : kSortBinBits;
      const uint32_t nbins = 1u << dbits;
      const int dsh = psh - dbits;
      uint32_t* bh = reinterpret_cast<uint32_t*>(wc);  // [nbins] counts -> offsets
      uint32_t* bf = bh + (1u << kSortBinBits);        // [nbins] fill
      for (uint32_t i = tid; i < nbins; i += kBucketThreads) {
        bh[i] = 0;
        bf[i] = 0;
      }
      if (tid == 0) {
        s_ovf = 0;
        s_unew = 0;
      }
      __syncthreads();
      // --- hash aggregation of this sub-range; it stops as soon as the distinct keys
      //     exceed half the table (the sort needs the other half)
      constexpr int PF = 4;  // keys loaded per thread before inserting
      const uint32_t ulimit = Heff / 2;
      if (nch)
        giant_pass<KeyT>(a, keys_rw, base, n, g0, nch, whole, lo, hi, rmask, skey, scnt, hmask, ulimit, &s_ovf,
                         &s_unew);
      for (uint32_t i0 = 0; i0 < n && !nch; i0 += PF * kBucketThreads) {
        if (*(volatile uint32_t*)&s_ovf) break;
        KeyT rr[PF];
#pragma unroll
        for (int q = 0; q < PF; q++) {
          const uint32_t i = i0 + q * kBucketThreads + tid;
          rr[q] = i < n ? (keys[base + i] & rmask) : EMPTY;
        }
        uint32_t fresh = 0;  // distinct keys this thread added in this round
#pragma unroll
        for (int q = 0; q < PF; q++) {
          const KeyT r = rr[q];
          const bool v = r != EMPTY && (whole || (!(r < lo) && r < hi));
          if (v) {
            const int res = hash_insert<KeyT>(skey, scnt, hmask, r, 1u);
            if (res == 2) s_ovf = 1;
            fresh += res == 1;
          }
        }
        // the distinct-key count grows once per warp and round (one shared atomic per
        // new key cost 7 % of the kernel)
        fresh = __reduce_add_sync(FULLMASK, fresh);
        if (lane == 0 && fresh && atomicAdd(&s_unew, fresh) + fresh > ulimit) s_ovf = 1;
      }
      __syncthreads();
      bool ovf = s_ovf != 0;
      // --- occupied slots into registers, counted, with their sort bins histogrammed;
      // order is irrelevant here, so slots are read with a stride of one block:
      // conflict-free shared-memory access
      constexpr int SPT = H / kBucketThreads;
      const uint32_t spt = Heff / kBucketThreads;
      KeyT rk[SPT];
      uint32_t rc[SPT];
      uint32_t occ = 0;
#pragma unroll
      for (int q = 0; q < SPT; q++) {
        rk[q] = EMPTY;
        rc[q] = 0;
        if ((uint32_t)q < spt) {
          rk[q] = skey[q * kBucketThreads + tid];
          rc[q] = scnt[q * kBucketThreads + tid];
          if (rk[q] != EMPTY) {
            occ++;
            if (!ovf) atomicAdd(&bh[(uint32_t)KeyOps<KeyT>::shr(rk[q], dsh) & (nbins - 1)], 1u);
          }
        }
      }
      uint32_t u;
      block_exclusive_sum(occ, s_warp, u);
      if (u > Heff / 2) ovf = true;  // the sort needs a second half
      if (ovf) {
        // cut [lo, hi) at quantiles of a sample of the distinct keys in the table
        // (one per thread: the first occupied slot of its stride)
        KeyT* samp = reinterpret_cast<KeyT*>(wc);  // kBucketThreads keys
        KeyT mine = EMPTY;
#pragma unroll
        for (int q = SPT - 1; q >= 0; q--)
          if (rk[q] != EMPTY) mine = rk[q];
        samp[tid] = mine;
        const int m = __syncthreads_count(mine != EMPTY);
        const int ways = m < kSplitWays ? m : kSplitWays;
        if (ways < 2) {
          if (tid == 0) s_fail = 1;
        } else if (mine != EMPTY) {
          int rank = 0;
          for (int j = 0; j < kBucketThreads; j++) {
            const KeyT o = samp[j];
            rank += (o != EMPTY && o < mine);
          }
          // splitter w (1 <= w < ways) is the sample of rank floor(w * m / ways)
          for (int w = 1; w < ways; w++)
            if (rank == (w * m) / ways) s_split[w] = mine;
        }
        __syncthreads();
        if (tid == 0 && !s_fail) {
          if (s_sp + ways > kBucketStack) {
            s_fail = 1;
          } else {
            // push the pieces highest first, so the lowest is counted next
            KeyT top = hi;
            for (int w = ways - 1; w >= 1; w--) {
              s_stk_lo[s_sp] = s_split[w];
              s_stk_hi[s_sp] = top;
              top = s_split[w];
              s_sp++;
            }
            s_stk_lo[s_sp] = lo;
            s_stk_hi[s_sp] = top;
            s_sp++;
          }
        }
        __syncthreads();
        if (s_fail) { failed = true; break; }
        continue;
      }
      // --- sort the u distinct remainders: bins (top bits below the prefix) are offset
      //     by a block scan and the slots go from registers straight into their bins;
      //     each element's rank among its bin (a bin holds a few keys) then gives its
      //     row, written at once.  A bin above kBinMax falls back to a stable LSD
      //     radix sort of the binned run.
      {
        constexpr int BPT = (1 << kSortBinBits) / kBucketThreads;
        uint32_t hv[BPT], hs = 0, hm = 0;
#pragma unroll
        for (int q = 0; q < BPT; q++) {
          const uint32_t bi = tid * BPT + q;
          hv[q] = bi < nbins ? bh[bi] : 0u;
          hs += hv[q];
          hm = max(hm, hv[q]);
        }
        uint32_t tot;
        uint32_t ex = block_exclusive_sum(hs, s_warp, tot);
#pragma unroll
        for (int q = 0; q < BPT; q++) {
          const uint32_t bi = tid * BPT + q;
          if (bi < nbins) bh[bi] = ex;
          ex += hv[q];
        }
        const bool radix = __syncthreads_or(hm > (uint32_t)kBinMax) != 0;
#pragma unroll
        for (int q = 0; q < SPT; q++) {
          if (rk[q] != EMPTY) {
            const uint32_t bi = (uint32_t)KeyOps<KeyT>::shr(rk[q], dsh) & (nbins - 1);
            const uint32_t pos = bh[bi] + atomicAdd(&bf[bi], 1u);
            skey[pos] = rk[q];
            scnt[pos] = rc[q];
          }
        }
        __syncthreads();
        if (!radix) {
          // element i of the binned run lands at row b0 + rank, within its bin's rows,
          // so neighbouring threads store to neighbouring rows
          const KeyT hi_bits = KeyOps<KeyT>::shl((KeyT)beta, rem);
          for (uint32_t i = tid; i < u; i += kBucketThreads) {
            const KeyT x = skey[i];
            const uint32_t bi = (uint32_t)KeyOps<KeyT>::shr(x, dsh) & (nbins - 1);
            const uint32_t b0 = bh[bi], b1 = b0 + bf[bi];
            uint32_t rank = 0;
            for (uint32_t j = b0; j < b1; j++) rank += skey[j] < x;
            emit_row<KeyT>(a, tkeys, (unsigned long long)base + acc + b0 + rank, hi_bits | x, scnt[i], shist,
                           s_bsmall);
          }
        } else {
          // stable LSD radix sort of the binned run in [0, u) through [H/2, H/2 + u)
          KeyT* sk = skey;
          uint32_t* sc = scnt;
          KeyT* dk = skey + Heff / 2;
          uint32_t* dc = scnt + Heff / 2;
          const int npass = (psh + 7) / 8;
          const uint32_t E = (u + NW - 1) / NW;
          const uint32_t e0 = (uint32_t)warp * E;
          const uint32_t e1 = min(e0 + E, u);
          const uint32_t rounds = (E + 31) / 32;
          for (int pass = 0; pass < npass; pass++) {
            const int sh = 8 * pass;
            __syncthreads();
            for (int i = lane; i < 256; i += 32) wc[warp * 256 + i] = 0;
            __syncwarp();
            uint32_t dig[RMAX], offs[RMAX];
#pragma unroll
            for (int rr = 0; rr < RMAX; rr++) {
              dig[rr] = 0;
              offs[rr] = 0;
              if ((uint32_t)rr >= rounds) continue;
              const uint32_t idx = e0 + rr * 32 + lane;
              const bool v = idx < e1;
              const uint32_t d = v ? (uint32_t)(KeyOps<KeyT>::shr(sk[idx], sh) & 0xff) : 0u;
              const unsigned vm = __ballot_sync(FULLMASK, v);
              uint32_t bse = 0;
              unsigned peers = 0;
              if (v) {
                peers = __match_any_sync(vm, d);
                if (lane == __ffs(peers) - 1) {
                  bse = wc[warp * 256 + d];
                  wc[warp * 256 + d] = (uint16_t)(bse + __popc(peers));
                }
              }
              __syncwarp();
              const int leader = v ? __ffs(peers) - 1 : lane;
              bse = __shfl_sync(FULLMASK, bse, leader);
              dig[rr] = d;
              offs[rr] = bse + __popc(peers & lanemask_lt());
            }
            __syncthreads();
            {
              constexpr int PER = (256 * NW) / kBucketThreads;
              uint32_t vals[PER];
              uint32_t sum = 0;
#pragma unroll
              for (int q = 0; q < PER; q++) {
                const int e = tid * PER + q;  // e = d * NW + w
                const int d = e / NW, w = e % NW;
                vals[q] = wc[w * 256 + d];
                sum += vals[q];
              }
              uint32_t tot2;
              uint32_t ex2 = block_exclusive_sum(sum, s_warp, tot2);
#pragma unroll
              for (int q = 0; q < PER; q++) {
                const int e = tid * PER + q;
                const int d = e / NW, w = e % NW;
                wc[w * 256 + d] = (uint16_t)ex2;
                ex2 += vals[q];
              }
            }
            __syncthreads();
#pragma unroll
            for (int rr = 0; rr < RMAX; rr++) {
              if ((uint32_t)rr >= rounds) continue;
              const uint32_t idx = e0 + rr * 32 + lane;
              if (idx < e1) {
                const uint32_t pos = wc[warp * 256 + dig[rr]] + offs[rr];
                dk[pos] = sk[idx];
                dc[pos] = sc[idx];
              }
            }
            __syncthreads();
            KeyT* tk = sk; sk = dk; dk = tk;
            uint32_t* tc = sc; sc = dc; dc = tc;
          }
          write_bucket_rows<KeyT>(sk, sc, u, a, beta, rem, base, acc, tkeys, shist, s_bsmall);
        }
      }
      acc += u;
      __syncthreads();
    }
    if (failed) {
      if (tid == 0) atomicOr(&a.sc->err, ERR_BUCKET);
      acc = 0;
    }
    __syncthreads();
    // the bucket's rows by small count: stored for the kept filter and folded into the
    // count histogram (counts below t); zeroed for the next bucket, whose rows come after
    // the barrier at the top of the loop
    if (tid < kSmallCounts) {
      const uint32_t c = s_bsmall[tid];
      if (a.bsmall) a.bsmall[(size_t)beta * kSmallCounts + tid] = c;
      if (c && tid < a.t) atomicAdd(&shist[tid], c);
      s_bsmall[tid] = 0;
    }
    if (tid == 0) {
      a.tu[beta] = acc;
      atomicAdd(&a.sc->n_unique, (unsigned long long)acc);
      s_ratio = 0.5f * s_ratio + 0.5f * ((float)acc / (float)n_eff);
    }
  }
  __syncthreads();
  for (int i = tid; i < hbins; i += kBucketThreads)
    if (shist[i]) atomicAdd(&a.hist[i], (unsigned long long)shist[i]);
}

// Dense copy of the sparse table: rows of bucket b move to doff[b] (exclusive prefix
// of tu).  mode 0: keys + counts arrays; mode 1: packed KmerPairs records.
template <typename KeyT>
__global__ void __launch_bounds__(256) k_compact_rows(const KeyT* __restrict__ skeys,
                                                      const uint32_t* __restrict__ scounts,
                                                      const uint32_t* __restrict__ bstart,
                                                      const uint32_t* __restrict__ tu,
                                                      const uint32_t* __restrict__ doff, int B,
                                                      KeyT* __restrict__ dkeys,
                                                      uint32_t* __restrict__ dcounts,
                                                      uint32_t* __restrict__ packed, int mode) {
  constexpr int WORDS = (sizeof(KeyT) + 4) / 4;
  for (int b = blockIdx.x; b < B; b += gridDim.x) {
    const uint32_t src = bstart[b], dst = doff[b], u = tu[b];
    for (uint32_t i = threadIdx.x; i < u; i += blockDim.x) {
      const KeyT x = skeys[src + i];
      const uint32_t c = scounts[src + i];
      if (mode == 0) {
        dkeys[dst + i] = x;
        dcounts[dst + i] = c;
      } else {
        uint32_t* o = packed + (size_t)(dst + i) * WORDS;
#pragma unroll
        for (int w = 0; w < WORDS - 1; w++) o[w] = (uint32_t)(x >> (32 * w));
        o[WORDS - 1] = c;
      }
    }
  }
}

// ------------------------------------------------------ histogram (other t) / cutoff --
__global__ void __launch_bounds__(256) k_histogram(const uint32_t* __restrict__ tcounts,
                                                   unsigned long long u, int t,
                                                   unsigned long long* hist) {
  __shared__ uint32_t sh[kHistSmem];
  const int hb = t < kHistSmem ? t : kHistSmem;
  for (int i = threadIdx.x; i < hb; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < u;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t c = tcounts[i];
    if (c < (uint32_t)t) {
      if (c < (uint32_t)kHistSmem) atomicAdd(&sh[c], 1u);
      else atomicAdd(&hist[c], 1ull);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < hb; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], (unsigned long long)sh[i]);
}

// cutoff = first minimum of hist[1..t) (t == 1 -> 1); kept = U - sum(hist[1..cutoff))
__global__ void __launch_bounds__(1024) k_cutoff(const unsigned long long* __restrict__ hist, int t,
                                                 Scalars* sc) {
  __shared__ unsigned long long s_v[32];
  __shared__ int s_i[32];
  unsigned long long best = ~0ull;
  int bi = 0x7fffffff;
  for (int c = 1 + threadIdx.x; c < t; c += blockDim.x) {
    unsigned long long v = hist[c];
    if (v < best || (v == best && c < bi)) { best = v; bi = c; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long v2 = __shfl_down_sync(FULLMASK, best, o);
    int i2 = __shfl_down_sync(FULLMASK, bi, o);
    if (v2 < best || (v2 == best && i2 < bi)) { best = v2; bi = i2; }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { s_v[warp] = best; s_i[warp] = bi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
      if (s_v[w] < best || (s_v[w] == best && s_i[w] < bi)) { best = s_v[w]; bi = s_i[w]; }
    const int cut = t > 1 ? bi : 1;
    unsigned long long below = 0;
    for (int c = 1; c < cut && c < t; c++) below += hist[c];
    sc->cutoff = (uint32_t)cut;
    sc->n_kept = sc->n_unique - below;
  }
}

// ----------------------------------------------------------------- macro-nodes -------
template <typename KeyT>
struct MnSmem {
  static constexpr size_t off_key = 0;
  static constexpr size_t off_cnt = off_key + sizeof(KeyT) * kMnCap;
  static constexpr size_t off_tag = off_cnt + sizeof(uint32_t) * kMnCap;
  static constexpr size_t off_ord = off_tag + sizeof(uint8_t) * kMnCap;
  static constexpr size_t off_nid = off_ord + sizeof(uint16_t) * kMnCap;
  static constexpr size_t bytes = off_nid + sizeof(uint16_t) * kMnCap;
};

template <typename KeyT>
__device__ __forceinline__ uint32_t lower_bound_s(const KeyT* k, uint32_t lo, uint32_t hi, KeyT x) {
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (k[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}
template <typename KeyT>
__device__ __forceinline__ uint32_t upper_bound_s(const KeyT* k, uint32_t lo, uint32_t hi, KeyT x) {
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (!(x < k[mid])) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Counts of table rows [q, q+4) (one 16-byte load when the four rows lie inside the
// count buffer) and the mask of those rows that are inside [r0, e) and kept.
__device__ __forceinline__ uint32_t kept_group(const FilterArgs& a, uint32_t q, uint32_t r0, uint32_t e,
                                               uint32_t cut, uint32_t c[4]) {
  c[0] = c[1] = c[2] = c[3] = 0;
  if (q >= e) return 0;
  if ((unsigned long long)q + 4 <= a.trows) {
    const uint4 v = *reinterpret_cast<const uint4*>(a.tcounts + q);
    c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
  } else {
#pragma unroll
    for (int t = 0; t < 4; t++)
      if ((unsigned long long)q + t < a.trows) c[t] = a.tcounts[q + t];
  }
  uint32_t m = 0;
#pragma unroll
  for (int t = 0; t < 4; t++)
    if (q + t >= r0 && q + t < e && c[t] >= cut) m |= 1u << t;
  return m;
}

// Kept rows (count >= cutoff) of every table bucket, written densely in key order --
// the k-mers construct_kmer_histogram hands to macro-node construction.  Per bucket:
// kstart (first kept row), kcount, and ksub (kept rows whose next two key bits are
// < 1, 2, 3).  Bucket offsets come from a decoupled look-back (every bucket publishes
// its aggregate before waiting).
template <typename KeyT>
__global__ void __launch_bounds__(256) k_filter_kept(FilterArgs a) {
  // one warp per table bucket: no block-wide barriers.  Lane l takes the rows
  // [g + 4l, g + 4l + 4) of each 128-row step, with g aligned to four rows, so one
  // 16-byte load brings its four counts and lane order is row order.
  const int lane = threadIdx.x & 31;
  const int B = 1 << a.bbits;
  const int rem = 2 * a.k - a.bbits;
  const uint32_t cut = a.sc->cutoff;
  const KeyT* __restrict__ tkeys = reinterpret_cast<const KeyT*>(a.tkeys);
  KeyT* __restrict__ kkeys = reinterpret_cast<KeyT*>(a.kkeys);
  while (true) {
    uint32_t beta = 0;
    if (lane == 0) beta = atomicAdd(&a.sc->ticket_filter, 1u);
    beta = __shfl_sync(FULLMASK, beta, 0);
    if (beta >= (uint32_t)B) break;
    const uint32_t r0 = a.bstart[beta], e = r0 + a.tu[beta];
    const uint32_t g0 = r0 & ~3u;
    uint32_t v = 0;
    if (a.bsmall && cut <= (uint32_t)kSmallCounts) {
      // kept rows = the bucket's rows minus those counted fewer than cut times
      uint32_t below = (lane >= 1 && (uint32_t)lane < cut) ? a.bsmall[(size_t)beta * kSmallCounts + lane] : 0u;
      below = __reduce_add_sync(FULLMASK, below);
      v = (e - r0) - below;
    } else {
      for (uint32_t g = g0; g < e; g += 128) {
        uint32_t c[4];
        v += __popc(kept_group(a, g + 4 * lane, r0, e, cut, c));
      }
      v = __reduce_add_sync(FULLMASK, v);
    }
    if (lane == 0) st_release(&a.flags[beta], kLbAgg | (unsigned long long)v);
    __syncwarp();
    unsigned long long K = lookback_exclusive(a.flags, (int)beta, &a.sc->err, a.spin_limit);
    if (lane == 0) {
      st_release(&a.flags[beta], kLbIncl | (K + v));
      if (beta == (uint32_t)B - 1) a.sc->n_kept_rows = K + v;
    }
    uint32_t pos = (uint32_t)K;
    uint32_t dl0 = 0, dl1 = 0, dl2 = 0;
    for (uint32_t g = g0; g < e; g += 128) {
      const uint32_t q = g + 4 * lane;
      uint32_t c[4];
      const uint32_t m = kept_group(a, q, r0, e, cut, c);
      const uint32_t n = __popc(m);
      uint32_t inc = n;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULLMASK, inc, o);
        if (lane >= o) inc += y;
      }
      uint32_t o = pos + inc - n;
#pragma unroll
      for (int t = 0; t < 4; t++) {
        if (!((m >> t) & 1u)) continue;
        const KeyT x = tkeys[q + t];
        if (o < a.cap) {
          kkeys[o] = x;
          a.kcounts[o] = c[t];
        } else {
          atomicOr(&a.sc->err, ERR_BOUNDS);
        }
        o++;
        const uint32_t d2 = (uint32_t)(KeyOps<KeyT>::shr(x, rem - 2) & 3);
        dl0 += d2 == 0;
        dl1 += d2 == 1;
        dl2 += d2 == 2;
      }
      pos += __shfl_sync(FULLMASK, inc, 31);
    }
    dl0 = __reduce_add_sync(FULLMASK, dl0);
    dl1 = __reduce_add_sync(FULLMASK, dl1);
    dl2 = __reduce_add_sync(FULLMASK, dl2);
    if (lane == 0) {
      a.kstart[beta] = (uint32_t)K;
      a.kcount[beta] = v;
      a.ksub[3 * beta + 0] = dl0;
      a.ksub[3 * beta + 1] = dl0 + dl1;
      a.ksub[3 * beta + 2] = dl0 + dl1 + dl2;
    }
  }
}

// Node key of kept row `row` as seen from stream `st`: the prefix (k-1)-mer x >> 2 for
// the suffix-side stream (st == 0), the suffix (k-1)-mer for the others.
template <typename KeyT>
__device__ __forceinline__ KeyT node_key(const KeyT* __restrict__ kk, uint32_t row, int st,
                                         KeyT succ_mask) {
  const KeyT x = kk[row];
  return st == 0 ? (x >> 2) : (x & succ_mask);
}

// first row in [lo, hi) whose node key is > piv
template <typename KeyT>
__device__ uint32_t upper_bound_rows(const KeyT* __restrict__ kk, uint32_t lo, uint32_t hi, int st,
                                     KeyT succ_mask, KeyT piv) {
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (!(piv < node_key(kk, mid, st, succ_mask))) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Per (k-1)-mer bucket: the suffix-side stream (kept rows of table bucket beta, node =
// x >> 2, extension = last base) and four prefix-side streams (kept rows of the table
// buckets whose remaining bits continue with beta, node = x & SUCC_MASK, extension =
// first base f) are each sorted by node key; merged they give the bucket's
// macro-nodes in key order.  A bucket larger than kMnCap rows is processed in
// segments split at node-key pivots.
template <typename KeyT>
__global__ void __launch_bounds__(kMnThreads, 8) k_macro_nodes(MnArgs a) {
  using SM = MnSmem<KeyT>;
  extern __shared__ __align__(16) unsigned char smem[];
  KeyT* ikey = reinterpret_cast<KeyT*>(smem + SM::off_key);
  uint32_t* icnt = reinterpret_cast<uint32_t*>(smem + SM::off_cnt);
  uint8_t* itag = reinterpret_cast<uint8_t*>(smem + SM::off_tag);
  uint16_t* ord = reinterpret_cast<uint16_t*>(smem + SM::off_ord);
  uint16_t* nid = reinterpret_cast<uint16_t*>(smem + SM::off_nid);
  __shared__ uint32_t s_warp[33];
  __shared__ uint32_t s_beta, s_off[6], s_cur[5], s_end[5], s_segend[5], s_beg[5], s_last;
  __shared__ unsigned long long s_NO;
  // counting-sort bins of a segment: offset (low 16 bits) and fill (high 16 bits)
  __shared__ uint32_t s_bin[kMnBins];

  const int tid = threadIdx.x;
  const int Bu = 1 << (a.bbits - 2 * a.level);  // node units
  const int k = a.k;
  const int nb = 2 * (k - 1);
  const KeyT succ_mask = KeyOps<KeyT>::mask(nb);
  const KeyT KINF = ~(KeyT)0;  // above every (k-1)-mer key
  const KeyT* __restrict__ kk = reinterpret_cast<const KeyT*>(a.kkeys);
  KeyT* __restrict__ nkeys = reinterpret_cast<KeyT*>(a.nkeys);
  constexpr uint32_t CAP = kMnCap - 16;  // rows per segment before ties
  // every node key of a unit shares its top pbits bits; the sort bins are the next
  // (at most kMnBinBits) bits
  const int pbits = a.bbits - 2 * a.level;
  const int rbits = nb - pbits > 0 ? nb - pbits : 0;
  const int dbits = rbits < kMnBinBits ? rbits : kMnBinBits;
  const int bsh = rbits - dbits;
  const uint32_t bmask = (1u << dbits) - 1u;

  // kept rows beyond the kept buffers were not written: nothing to merge (every CTA
  // reads the same flag, so all of them leave)
  if (tid == 0) s_beta = (a.sc->err & ERR_BOUNDS) ? 1u : 0u;
  // merge positions start in range, so even runs that break the sorted-input contract
  // only ever index the segment arrays
  for (int i = tid; i < kMnCap; i += kMnThreads) ord[i] = 0;
  __syncthreads();
  if (s_beta) return;

  while (true) {
    __syncthreads();
    if (tid == 0) s_beta = atomicAdd(&a.sc->ticket_mn, 1u);
    __syncthreads();
    const uint32_t beta = s_beta;
    if (beta >= (uint32_t)Bu) break;
    if (tid == 0) {
      if (a.level == 0) {
        // node bucket = table bucket: suffix stream = the bucket's kept rows, prefix
        // streams = the part of bucket (f, beta >> 2) whose next two bits are beta & 3
        s_cur[0] = a.kstart[beta];
        s_end[0] = a.kstart[beta] + a.kcount[beta];
        for (int f = 0; f < 4; f++) {
          const uint32_t bp = ((uint32_t)f << (a.bbits - 2)) | (beta >> 2);
          const uint32_t d = beta & 3;
          const uint32_t b0 = a.kstart[bp];
          s_cur[f + 1] = b0 + (d == 0 ? 0u : a.ksub[3 * bp + d - 1]);
          s_end[f + 1] = b0 + (d == 3 ? a.kcount[bp] : a.ksub[3 * bp + d]);
        }
      } else {
        // node unit = the node keys whose top bbits - 2 level bits are beta: suffix
        // stream = table buckets [beta << 2L, (beta + 1) << 2L), prefix stream f =
        // table buckets (f, beta, any 2L - 2 bits) -- contiguous kept rows each
        const int L2 = 2 * a.level;
        const uint32_t s0b = beta << L2, s1b = s0b + (1u << L2) - 1;
        s_cur[0] = a.kstart[s0b];
        s_end[0] = a.kstart[s1b] + a.kcount[s1b];
        for (int f = 0; f < 4; f++) {
          const uint32_t p0 = ((uint32_t)f << (a.bbits - 2)) | (beta << (L2 - 2));
          const uint32_t p1 = p0 + (1u << (L2 - 2)) - 1;
          s_cur[f + 1] = a.kstart[p0];
          s_end[f + 1] = a.kstart[p1] + a.kcount[p1];
        }
      }
      for (int st = 0; st < 5; st++)
        if (s_end[st] > a.kcap || s_cur[st] > s_end[st]) {  // never read past the kept rows
          atomicOr(&a.sc->err, ERR_BOUNDS);
          s_cur[st] = s_end[st] = 0;
        }
    }
    if (tid == 0)
      for (int st = 0; st < 5; st++) s_beg[st] = s_cur[st];
    __syncthreads();
    // A bucket that fits one segment is merged, counted and written in one pass.  A
    // larger one is first merged to count its nodes (so its aggregate is published
    // before any wait and later buckets do not queue behind it), then merged again
    // and written.
    bool counting = false;
    unsigned long long NO = 0, total = 0;
    for (int pass = 0; pass < 2; pass++) {
      bool first = true;
      unsigned long long done_nodes = 0;
      while (true) {
        // ---- choose this segment's rows: everything left, or rows up to a pivot key
        if (tid == 0) {
          uint32_t rows = 0;
          for (int st = 0; st < 5; st++) rows += s_end[st] - s_cur[st];
          KeyT piv = KINF;
          if (rows > CAP) {
            const float frac = 0.9f * (float)CAP / (float)rows;
            for (int st = 0; st < 5; st++) {
              const uint32_t take = (uint32_t)((float)(s_end[st] - s_cur[st]) * frac);
              if (take >= 1) {
                const KeyT kx = node_key(kk, s_cur[st] + take - 1, st, succ_mask);
                if (kx < piv) piv = kx;
              }
            }
          }
          s_last = 1;
          for (int st = 0; st < 5; st++) {
            s_segend[st] = piv == KINF ? s_end[st]
                                       : upper_bound_rows(kk, s_cur[st], s_end[st], st, succ_mask, piv);
            if (s_segend[st] != s_end[st]) s_last = 0;
          }
          uint32_t o = 0;
          for (int st = 0; st < 5; st++) {
            s_off[st] = o;
            o += s_segend[st] - s_cur[st];
          }
          s_off[5] = o;
        }
        __syncthreads();
        const bool last = s_last != 0;
        if (pass == 0 && first && !last) counting = true;
        uint32_t mm = s_off[5];
        if (mm > (uint32_t)kMnCap) {  // cannot happen with CAP-sized segments
          if (tid == 0) atomicOr(&a.sc->err, ERR_MN_CAPACITY);
          mm = 0;
        }
        // ---- gather the five sorted runs
        for (uint32_t i = tid; i < mm; i += kMnThreads) {
          int st = 0;
          while (i >= s_off[st + 1]) st++;
          const uint32_t row = s_cur[st] + (i - s_off[st]);
          const KeyT x = kk[row];
          ikey[i] = st == 0 ? (x >> 2) : (x & succ_mask);
          itag[i] = (uint8_t)(st == 0 ? (uint32_t)(x & 3) : (uint32_t)(3 + st));
          icnt[i] = a.kcounts[row];
        }
        __syncthreads();
        // ---- order of the items by node key, ties by run and then position (the stable
        //      merge of the five runs): a counting sort on the key bits below the unit's
        //      common prefix, then each item's rank among its bin, which holds a few items.
        //      A crowded bin falls back to merge ranks across the runs.
        for (int b = tid; b < kMnBins; b += kMnThreads) s_bin[b] = 0;
        __syncthreads();
        for (uint32_t i = tid; i < mm; i += kMnThreads)
          atomicAdd(&s_bin[(uint32_t)KeyOps<KeyT>::shr(ikey[i], bsh) & bmask], 1u);
        __syncthreads();
        {
          constexpr int BPT = kMnBins / kMnThreads;
          uint32_t hv[BPT], hs = 0, hm = 0;
#pragma unroll
          for (int q = 0; q < BPT; q++) {
            hv[q] = s_bin[tid * BPT + q];
            hs += hv[q];
            hm = max(hm, hv[q]);
          }
          uint32_t tot;
          uint32_t ex = block_exclusive_sum(hs, s_warp, tot);
#pragma unroll
          for (int q = 0; q < BPT; q++) {
            s_bin[tid * BPT + q] = ex;
            ex += hv[q];
          }
          const bool crowded = __syncthreads_or(hm > (uint32_t)kMnBinMax) != 0;
          if (!crowded) {
            uint16_t* binned = nid;  // scratch until the node ids are computed
            for (uint32_t i = tid; i < mm; i += kMnThreads) {
              const uint32_t o = atomicAdd(&s_bin[(uint32_t)KeyOps<KeyT>::shr(ikey[i], bsh) & bmask], 1u << 16);
              binned[(o & 0xffffu) + (o >> 16)] = (uint16_t)i;
            }
            __syncthreads();
            for (uint32_t p = tid; p < mm; p += kMnThreads) {
              const uint32_t i = binned[p];
              const KeyT x = ikey[i];
              const uint32_t o = s_bin[(uint32_t)KeyOps<KeyT>::shr(x, bsh) & bmask];
              const uint32_t b0 = o & 0xffffu, b1 = b0 + (o >> 16);
              uint32_t rank = 0;
              for (uint32_t j = b0; j < b1; j++) {
                const uint32_t ij = binned[j];
                const KeyT y = ikey[ij];
                rank += (y < x || (!(x < y) && ij < i)) ? 1u : 0u;
              }
              ord[b0 + rank] = (uint16_t)i;
            }
          } else {
            for (uint32_t i = tid; i < mm; i += kMnThreads) {
              int st = 0;
              while (i >= s_off[st + 1]) st++;
              const KeyT x = ikey[i];
              uint32_t rank = i - s_off[st];
              for (int b = 0; b < 5; b++) {
                if (b == st) continue;
                const uint32_t lo = s_off[b], hi = s_off[b + 1];
                rank += (b < st ? upper_bound_s(ikey, lo, hi, x) : lower_bound_s(ikey, lo, hi, x)) - lo;
              }
              ord[rank] = (uint16_t)i;
            }
          }
        }
        __syncthreads();
        // ---- node boundaries and node index per merged position: each thread takes
        //      a contiguous run of positions, so one block scan serves the segment
        uint32_t nodes = 0;
        {
          const uint32_t per = (mm + kMnThreads - 1) / kMnThreads;
          const uint32_t r0 = min(mm, tid * per), r1 = min(mm, r0 + per);
          uint32_t cnt = 0;
          for (uint32_t r = r0; r < r1; r++) cnt += (r == 0) || !(ikey[ord[r - 1]] == ikey[ord[r]]);
          uint32_t tot;
          uint32_t run = block_exclusive_sum(cnt, s_warp, tot);
          for (uint32_t r = r0; r < r1; r++) {
            run += (r == 0) || !(ikey[ord[r - 1]] == ikey[ord[r]]);
            nid[r] = (uint16_t)(run - 1);
          }
          nodes = tot;
        }
        __syncthreads();  // nid is read across threads below
        if (!counting) {
          // ---- node offset: decoupled look-back over node buckets
          if (first) {
            if (tid < 32) {  // warp 0 looks back
              const unsigned long long mine = pass == 0 ? nodes : total;
              // a withheld unit (bounded-wait tests) publishes nothing: its successors'
              // waits run out and report ERR_LOOKBACK
              const bool publish = (int)beta != a.withhold_unit;
              if (tid == 0 && publish) st_release(&a.flags[beta], kLbAgg | mine);
              __syncwarp();
              const unsigned long long ex = lookback_exclusive(a.flags, (int)beta, &a.sc->err, a.spin_limit);
              if (tid == 0) {
                if (publish) st_release(&a.flags[beta], kLbIncl | (ex + mine));
                s_NO = ex;
              }
            }
            __syncthreads();
            NO = s_NO;
          }
          const unsigned long long q0 = NO + done_nodes;
          if (q0 + nodes <= a.cap) {
            for (uint32_t r = tid; r < mm; r += kMnThreads) {
              if (r == 0 || nid[r] != nid[r - 1]) {
                const unsigned long long q = q0 + nid[r];
                nkeys[q] = ikey[ord[r]];
                reinterpret_cast<uint4*>(a.nsuf)[q] = make_uint4(0, 0, 0, 0);
                reinterpret_cast<uint4*>(a.npre)[q] = make_uint4(0, 0, 0, 0);
              }
            }
            __syncthreads();
            for (uint32_t r = tid; r < mm; r += kMnThreads) {
              const uint32_t i = ord[r];
              const unsigned long long q = q0 + nid[r];
              const uint32_t tg = itag[i];
              if (tg < 4) a.nsuf[4 * q + tg] = icnt[i];
              else a.npre[4 * q + (tg - 4)] = icnt[i];
            }
          } else if (tid == 0) {
            atomicOr(&a.sc->err, ERR_MN_CAPACITY);
          }
        }
        done_nodes += nodes;
        first = false;
        __syncthreads();
        if (tid == 0)
          for (int st = 0; st < 5; st++) s_cur[st] = s_segend[st];
        __syncthreads();
        if (last) break;
      }
      total = done_nodes;
      if (!counting) break;
      // counted: rewind and write
      counting = false;
      if (tid == 0)
        for (int st = 0; st < 5; st++) s_cur[st] = s_beg[st];
      __syncthreads();
    }
    if (tid == 0 && beta == (uint32_t)Bu - 1) a.sc->n_nodes = NO + total;
  }
}

// ------------------------------------------------------- loaded (external) tables --
// Bucket extents of a dense ascending table: bstart[b] = first row whose key's top
// `bbits` bits are >= b, tu[b] = rows of bucket b (the sparse layout with no gaps).
template <typename KeyT>
__global__ void __launch_bounds__(256) k_table_bounds(const KeyT* __restrict__ keys, unsigned long long n,
                                                      int bbits, int rem, uint32_t* bstart) {
  const int B = 1 << bbits;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > B) return;
  unsigned long long lo = 0, hi = n;
  if (b == B) {
    lo = n;
  } else {
    const KeyT x = KeyOps<KeyT>::shl((KeyT)(uint32_t)b, rem);
    while (lo < hi) {
      const unsigned long long mid = (lo + hi) >> 1;
      if (keys[mid] < x) lo = mid + 1; else hi = mid;
    }
  }
  bstart[b] = (uint32_t)lo;
}

__global__ void __launch_bounds__(256) k_table_sizes(const uint32_t* bstart, int B, uint32_t* tu) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B) tu[b] = bstart[b + 1] - bstart[b];
}

// =================================================================== launchers =====
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static int g_sms = 0;
// SM count the calling thread's launches are sized for: a serving worker running a
// request on an SM partition sets it to the partition's SMs (0: the whole device)
static thread_local int t_sms = 0;
void set_thread_sms(int n) { t_sms = n > 0 ? n : 0; }
int thread_sms(int device_sms) { return t_sms > 0 ? t_sms : device_sms; }

static int sm_count() {
  if (t_sms > 0) return t_sms;
  if (!g_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 1;
  }
  return g_sms;
}

size_t bucket_smem_bytes(int wide) {
  return wide ? BucketSmem<u128>::bytes : BucketSmem<uint64_t>::bytes;
}
size_t mn_smem_bytes(int wide) { return wide ? MnSmem<u128>::bytes : MnSmem<uint64_t>::bytes; }
int bucket_ctas_per_sm(int) { return 2; }
int mn_ctas_per_sm(int wide) { return wide ? 5 : 8; }

cudaError_t launch_line_tiles(const uint8_t* buf, unsigned long long F, uint32_t* tile_nl, Scalars* sc,
                              unsigned long long tile0, unsigned long long ntiles, cudaStream_t st) {
  if (ntiles > 0) pk::note_launch(), k_line_scan<<<(unsigned)ntiles, 256, 0, st>>>(buf, F, tile_nl, sc, tile0);
  return cudaGetLastError();
}

cudaError_t launch_tile_prefix(const CountArgs& a, cudaStream_t st) {
  const int ntiles = (int)((a.F + kTileBytes - 1) / kTileBytes);
  pk::note_launch(), k_tile_prefix<<<1, 1024, 0, st>>>(a.fasta, a.F, a.tile_nl, ntiles, a.sc);
  return cudaGetLastError();
}

cudaError_t launch_line_scan(const CountArgs& a, cudaStream_t st) {
  const unsigned long long ntiles = (a.F + kTileBytes - 1) / kTileBytes;
  cudaError_t e = launch_line_tiles(a.fasta, a.F, a.tile_nl, a.sc, 0, ntiles, st);
  if (e != cudaSuccess) return e;
  return launch_tile_prefix(a, st);
}

template <typename KeyT, bool FASTB>
static cudaError_t launch_extract_t(const CountArgs& a, cudaStream_t st) {
  const size_t smem = sizeof(uint32_t) << a.bbits;
  // the attribute is shared by every thread launching this kernel, so it is always
  // set to the largest histogram (15 partition digits), never to this launch's size
  static bool attr_set = false;  // same value from every thread, so a race is benign
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_extract<KeyT, FASTB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(uint32_t) << kHistBits));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  pk::note_launch(), k_extract<KeyT, FASTB><<<a.grid, CountCfg<KeyT>::T, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_bucket_count(const CountArgs& a, int wide, cudaStream_t st) {
  if (wide) return launch_extract_t<u128, false>(a, st);
  // bucket digits in the key's high word: the 32-bit bucket path
  if (2 * a.k - a.bbits >= 34) return launch_extract_t<uint64_t, true>(a, st);
  return launch_extract_t<uint64_t, false>(a, st);
}

template <typename KeyT>
static cudaError_t launch_coarse_t(const CountArgs& a, const uint32_t* coff, KeyT* out, cudaStream_t st) {
  const size_t smem = CoarseCfg<KeyT>::smem;
  static bool attr_set = false;  // a constant, so concurrent first calls agree
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_scatter_coarse<KeyT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  pk::note_launch(), k_scatter_coarse<KeyT><<<a.grid, CoarseCfg<KeyT>::T, smem, st>>>(a, coff, out);
  return cudaGetLastError();
}

cudaError_t launch_scatter_coarse(const CountArgs& a, const uint32_t* coff, void* out, int wide,
                                  cudaStream_t st) {
  return wide ? launch_coarse_t<u128>(a, coff, reinterpret_cast<u128*>(out), st)
              : launch_coarse_t<uint64_t>(a, coff, reinterpret_cast<uint64_t*>(out), st);
}

cudaError_t launch_coarse_offsets(const CountArgs& a, uint32_t* coff, uint32_t* cstart,
                                  uint32_t* slice_start, int slice_keys, cudaStream_t st) {
  const int sk = slice_keys;
  pk::note_launch(), k_coarse_offsets<<<a.grid, 256, 0, st>>>(a.counts, a.bstart, a.grid, a.bbits, a.cbits, coff, cstart,
                                           slice_start, sk);
  return cudaGetLastError();
}

template <typename KeyT>
static cudaError_t launch_fine_t(const KeyT* in, const uint32_t* cstart, const uint32_t* slice_start,
                                 uint32_t* fcur, KeyT* out, int k, int bbits, int cbits, uint32_t* ticket,
                                 unsigned long long cap, uint32_t* err, cudaStream_t st) {
  const size_t smem = FineCfg<KeyT>::smem;
  static bool attr_set = false;  // a constant, so concurrent first calls agree
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_scatter_fine<KeyT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  if (bbits - cbits >= 11) {
    const size_t bsmem = FineBigCfg<KeyT>::smem;
    static bool big_attr_set = false;
    if (!big_attr_set) {
      cudaError_t e = cudaFuncSetAttribute(k_scatter_fine_big<KeyT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bsmem);
      if (e != cudaSuccess) return e;
      big_attr_set = true;
    }
    pk::note_launch(), k_scatter_fine_big<KeyT><<<sm_count(), FineBigCfg<KeyT>::T, bsmem, st>>>(in, cstart, slice_start, fcur, out, k,
                                                                             bbits, cbits, ticket, cap, err);
    return cudaGetLastError();
  }
  pk::note_launch(), k_scatter_fine<KeyT><<<sm_count() * 2, FineCfg<KeyT>::T, smem, st>>>(in, cstart, slice_start, fcur, out,
                                                                        k, bbits, cbits, ticket, cap, err);
  return cudaGetLastError();
}

cudaError_t launch_scatter_fine(const void* in, const uint32_t* cstart, const uint32_t* slice_start,
                                uint32_t* fcur, void* out, int k, int bbits, int cbits, int wide,
                                uint32_t* ticket, unsigned long long cap, uint32_t* err, cudaStream_t st) {
  return wide ? launch_fine_t<u128>(reinterpret_cast<const u128*>(in), cstart, slice_start, fcur,
                                    reinterpret_cast<u128*>(out), k, bbits, cbits, ticket, cap, err, st)
              : launch_fine_t<uint64_t>(reinterpret_cast<const uint64_t*>(in), cstart, slice_start, fcur,
                                        reinterpret_cast<uint64_t*>(out), k, bbits, cbits, ticket, cap, err,
                                        st);
}

cudaError_t launch_fine_count(const void* in, const uint32_t* cstart, const uint32_t* slice_start,
                              uint32_t* bcount, int k, int bbits, int cbits, int wide, uint32_t* ticket,
                              cudaStream_t st) {
  const uint32_t sk = (uint32_t)fine_slice_keys(wide, bbits - cbits);
  if (wide)
    pk::note_launch(), k_fine_count<u128><<<sm_count() * 2, 512, 0, st>>>(reinterpret_cast<const u128*>(in), cstart, slice_start,
                                                      bcount, k, bbits, cbits, ticket, sk);
  else
    pk::note_launch(), k_fine_count<uint64_t><<<sm_count() * 2, 512, 0, st>>>(reinterpret_cast<const uint64_t*>(in), cstart,
                                                          slice_start, bcount, k, bbits, cbits, ticket, sk);
  return cudaGetLastError();
}

cudaError_t launch_prefix(uint32_t* counts, int B, cudaStream_t st) {
  pk::note_launch(), k_bucket_prefix<<<1, 1024, 0, st>>>(counts, B);
  return cudaGetLastError();
}

cudaError_t launch_bucket_offsets(const CountArgs& a, cudaStream_t st) {
  const int B = 1 << a.bbits;
  pk::note_launch(), k_col_prefix<<<(B + 31) / 32, 256, 0, st>>>(a.counts, a.grid, B, a.bstart);
  pk::note_launch(), k_bucket_prefix<<<1, 1024, 0, st>>>(a.bstart, B);
  return cudaGetLastError();
}


template <typename KeyT>
static cudaError_t launch_bucket_t(const BucketArgs& a, int grid, cudaStream_t st) {
  const size_t smem = BucketSmem<KeyT>::bytes;
  static bool attr_set = false;  // a constant, so concurrent first calls agree
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_bucket_table<KeyT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_bucket_table<KeyT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  if (grid <= 0) grid = sm_count() * bucket_ctas_per_sm(sizeof(KeyT) == 16);
  // exactly one of the two works (giant buckets present or not); the other returns
  pk::note_launch(), k_bucket_table<KeyT, false><<<grid, kBucketThreads, smem, st>>>(a);
  pk::note_launch(), k_bucket_table<KeyT, true><<<grid, kBucketThreads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_bucket_table(const BucketArgs& a, int wide, int grid, cudaStream_t st) {
  return wide ? launch_bucket_t<u128>(a, grid, st) : launch_bucket_t<uint64_t>(a, grid, st);
}

cudaError_t launch_giant_chunks(const uint32_t* bstart, int bbits, uint32_t* gfirst, uint32_t* gcount,
                                uint32_t* chunk_bucket, uint32_t* gdone, Scalars* sc, cudaStream_t st) {
  const int B = 1 << bbits;
  pk::note_launch(), k_giant_chunks<<<(B + 255) / 256, 256, 0, st>>>(bstart, B, gfirst, gcount, chunk_bucket, gdone, sc);
  return cudaGetLastError();
}

cudaError_t launch_histogram(const uint32_t* tcounts, unsigned long long u, int t,
                             unsigned long long* hist, cudaStream_t st) {
  int grid = (int)((u + 255) / 256);
  if (grid > sm_count() * 8) grid = sm_count() * 8;
  if (grid < 1) grid = 1;
  pk::note_launch(), k_histogram<<<grid, 256, 0, st>>>(tcounts, u, t, hist);
  return cudaGetLastError();
}

cudaError_t launch_cutoff(const unsigned long long* hist, int t, Scalars* sc, cudaStream_t st) {
  pk::note_launch(), k_cutoff<<<1, 1024, 0, st>>>(hist, t, sc);
  return cudaGetLastError();
}

template <typename KeyT>
static cudaError_t launch_filter_t(const FilterArgs& a, int grid, cudaStream_t st) {
  if (grid <= 0) grid = sm_count() * 8;
  pk::note_launch(), k_filter_kept<KeyT><<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_filter_kept(const FilterArgs& a, int wide, int grid, cudaStream_t st) {
  return wide ? launch_filter_t<u128>(a, grid, st) : launch_filter_t<uint64_t>(a, grid, st);
}

template <typename KeyT>
static cudaError_t launch_mn_t(const MnArgs& a, int grid, cudaStream_t st) {
  const size_t smem = MnSmem<KeyT>::bytes;
  static bool attr_set = false;  // a constant, so concurrent first calls agree
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_macro_nodes<KeyT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  if (grid <= 0) grid = sm_count() * mn_ctas_per_sm(sizeof(KeyT) == 16);
  pk::note_launch(), k_macro_nodes<KeyT><<<grid, kMnThreads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_macro_nodes(const MnArgs& a, int wide, int grid, cudaStream_t st) {
  return wide ? launch_mn_t<u128>(a, grid, st) : launch_mn_t<uint64_t>(a, grid, st);
}

__global__ void __launch_bounds__(1024) k_copy_prefix(const uint32_t* __restrict__ in,
                                                      uint32_t* __restrict__ out, int B) {
  __shared__ uint32_t s_warp[33];
  uint32_t carry = 0;
  for (int base = 0; base < B; base += blockDim.x) {
    int i = base + threadIdx.x;
    uint32_t v = i < B ? in[i] : 0;
    uint32_t tot;
    uint32_t ex = block_exclusive_sum(v, s_warp, tot);
    if (i < B) out[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) out[B] = carry;
}

cudaError_t launch_row_offsets(const uint32_t* tu, uint32_t* doff, int B, cudaStream_t st) {
  pk::note_launch(), k_copy_prefix<<<1, 1024, 0, st>>>(tu, doff, B);
  return cudaGetLastError();
}

cudaError_t launch_compact_rows(const void* tkeys, const uint32_t* tcounts, const uint32_t* bstart,
                                const uint32_t* tu, const uint32_t* doff, int B, int wide,
                                void* dkeys, uint32_t* dcounts, void* packed, cudaStream_t st) {
  int grid = B < sm_count() * 16 ? B : sm_count() * 16;
  if (grid < 1) grid = 1;
  const int mode = packed ? 1 : 0;
  if (wide)
    pk::note_launch(), k_compact_rows<u128><<<grid, 256, 0, st>>>(reinterpret_cast<const u128*>(tkeys), tcounts, bstart,
                                               tu, doff, B, reinterpret_cast<u128*>(dkeys), dcounts,
                                               reinterpret_cast<uint32_t*>(packed), mode);
  else
    pk::note_launch(), k_compact_rows<uint64_t><<<grid, 256, 0, st>>>(reinterpret_cast<const uint64_t*>(tkeys), tcounts,
                                                   bstart, tu, doff, B,
                                                   reinterpret_cast<uint64_t*>(dkeys), dcounts,
                                                   reinterpret_cast<uint32_t*>(packed), mode);
  return cudaGetLastError();
}

}  // namespace pk

namespace pk {
cudaError_t launch_table_bounds(const void* keys, unsigned long long n, int bbits, int k, uint32_t* bstart,
                                uint32_t* tu, int wide, cudaStream_t st) {
  const int B = 1 << bbits;
  const int rem = 2 * k - bbits;
  const int grid = (B + 1 + 255) / 256;
  if (wide) {
    pk::note_launch(), k_table_bounds<u128><<<grid, 256, 0, st>>>((const u128*)keys, n, bbits, rem, bstart);
    pk::note_launch(), k_table_sizes<<<(B + 255) / 256, 256, 0, st>>>(bstart, B, tu);
  } else {
    pk::note_launch(), k_table_bounds<uint64_t><<<grid, 256, 0, st>>>((const uint64_t*)keys, n, bbits, rem, bstart);
    pk::note_launch(), k_table_sizes<<<(B + 255) / 256, 256, 0, st>>>(bstart, B, tu);
  }
  return cudaGetLastError();
}
}  // namespace pk

// ----------------------------------------------------------------- batch output ----
namespace pk {

// One set of a captured batch: reserve its rows in the batch's macro-node table.
// res = {first row, rows, state}; state 1 ok, 2 table full, 3 device error, 4 nothing kept.
__global__ void k_batch_reserve(const Scalars* sc, unsigned long long* counter, unsigned long long cap,
                                unsigned long long* res) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (sc->err != 0) {
    res[0] = 0; res[1] = 0; res[2] = 3;
    return;
  }
  if (sc->n_kept == 0) {
    res[0] = 0; res[1] = 0; res[2] = 4;
    return;
  }
  const unsigned long long m = sc->n_nodes;
  const unsigned long long off = atomicAdd(counter, m);
  if (off + m > cap) {
    res[0] = 0; res[1] = 0; res[2] = 2;
    return;
  }
  res[0] = off; res[1] = m; res[2] = 1;
}

// Copy the set's nodes (key words, 4 suffix and 4 prefix counts) to its reserved rows.
__global__ void __launch_bounds__(256) k_batch_copy(const unsigned long long* __restrict__ nkeys,
                                                    const uint4* __restrict__ nsuf,
                                                    const uint4* __restrict__ npre, int key_words,
                                                    const unsigned long long* res,
                                                    unsigned long long* okeys, uint4* osuf, uint4* opre) {
  if (res[2] != 1) return;
  const unsigned long long off = res[0], m = res[1];
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < m;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    for (int w = 0; w < key_words; w++) okeys[(off + i) * key_words + w] = nkeys[i * key_words + w];
    osuf[off + i] = nsuf[i];
    opre[off + i] = npre[i];
  }
}

cudaError_t launch_batch_emit(const Scalars* sc, unsigned long long* counter, unsigned long long cap,
                              unsigned long long* res, const void* nkeys, const void* nsuf, const void* npre,
                              int wide, void* okeys, void* osuf, void* opre, cudaStream_t st) {
  pk::note_launch(), k_batch_reserve<<<1, 32, 0, st>>>(sc, counter, cap, res);
  pk::note_launch(), k_batch_copy<<<sm_count() * 2, 256, 0, st>>>((const unsigned long long*)nkeys, (const uint4*)nsuf,
                                               (const uint4*)npre, wide ? 2 : 1, res,
                                               (unsigned long long*)okeys, (uint4*)osuf, (uint4*)opre);
  return cudaGetLastError();
}

}  // namespace pk

// ------------------------------------------------------------------ initial wiring --
namespace pk {

// One thread per macro-node: the initial wiring of src/wire.cpp:66-121 /
// MacroNode::setup_wiring (includes/distribute_kmers.h:549-655).  Lists: present
// extensions in ascending base code, then the terminal entry (count 1, visit =
// max(other side's visit sum - own side's, 0)); entries ranked by visit then count,
// both descending, equal entries in list order; a two-pointer walk pairs prefix
// visits with suffix visits.
__global__ void __launch_bounds__(256) k_wire(const uint4* __restrict__ nsuf, const uint4* __restrict__ npre,
                                              unsigned long long m, int coverage, WireRow* __restrict__ out) {
  const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint4 s4 = nsuf[i], p4 = npre[i];
  const uint32_t sraw[4] = {s4.x, s4.y, s4.z, s4.w}, praw[4] = {p4.x, p4.y, p4.z, p4.w};
  int32_t scnt[5], svis[5], pcnt[5], pvis[5];
  int ns = 0, np = 0, sc = 0, pc = 0;
  const uint32_t cov = (uint32_t)coverage;
#pragma unroll
  for (int e = 0; e < 4; e++) {
    if (sraw[e]) {
      scnt[ns] = (int32_t)sraw[e];
      svis[ns] = (int32_t)((sraw[e] + cov - 1) / cov);
      sc += svis[ns];
      ns++;
    }
    if (praw[e]) {
      pcnt[np] = (int32_t)praw[e];
      pvis[np] = (int32_t)((praw[e] + cov - 1) / cov);
      pc += pvis[np];
      np++;
    }
  }
  scnt[ns] = 1;
  svis[ns] = max(pc - sc, 0);
  ns++;
  pcnt[np] = 1;
  pvis[np] = max(sc - pc, 0);
  np++;
  // rank the entries (insertion sort: equal entries keep list order)
  int os[5], op[5];
  for (int a = 0; a < ns; a++) os[a] = a;
  for (int a = 0; a < np; a++) op[a] = a;
  for (int a = 1; a < ns; a++) {
    const int x = os[a];
    int b = a - 1;
    while (b >= 0 && (svis[x] > svis[os[b]] || (svis[x] == svis[os[b]] && scnt[x] > scnt[os[b]]))) {
      os[b + 1] = os[b];
      b--;
    }
    os[b + 1] = x;
  }
  for (int a = 1; a < np; a++) {
    const int x = op[a];
    int b = a - 1;
    while (b >= 0 && (pvis[x] > pvis[op[b]] || (pvis[x] == pvis[op[b]] && pcnt[x] > pcnt[op[b]]))) {
      op[b + 1] = op[b];
      b--;
    }
    op[b + 1] = x;
  }
  WireRow r;
  r.ns = ns;
  r.np = np;
  r.term_suf = svis[ns - 1];
  r.term_pre = pvis[np - 1];
  for (int a = 0; a < 27; a++) (&r.wire[0][0])[a] = 0;
  for (int a = 0; a < 10; a++) (&r.begin[0][0])[a] = 0;
  int leftover = sc + svis[ns - 1];
  int off_s[5] = {0, 0, 0, 0, 0};
  int top_p = 0, top_s = 0, var_p = 0, var_s = 0, wi = 0, p_size = 0, last_pid = -1, begin_pos = -1;
  while (leftover > 0 && wi < 9) {
    const int sid = os[top_s], pid = op[top_p];
    const int cnt = min(pvis[pid] - var_p, svis[sid] - var_s);
    r.wire[wi][0] = sid;
    r.wire[wi][1] = off_s[sid];
    r.wire[wi][2] = cnt;
    if (last_pid != pid) {
      begin_pos = wi;
      last_pid = pid;
    }
    p_size++;
    wi++;
    leftover -= cnt;
    var_p += cnt;
    var_s += cnt;
    off_s[sid] += cnt;
    if (var_p == pvis[pid]) {
      var_p = 0;
      top_p++;
      r.begin[pid][0] = begin_pos;
      r.begin[pid][1] = p_size;
      p_size = 0;
    }
    if (var_s == svis[sid]) {
      var_s = 0;
      top_s++;
    }
  }
  r.nw = wi;
  out[i] = r;
}

cudaError_t launch_wire(const void* nsuf, const void* npre, unsigned long long m, int coverage, WireRow* out,
                        cudaStream_t st) {
  if (m == 0) return cudaSuccess;
  pk::note_launch(), k_wire<<<(unsigned)((m + 255) / 256), 256, 0, st>>>((const uint4*)nsuf, (const uint4*)npre, m, coverage, out);
  return cudaGetLastError();
}

}  // namespace pk

extern "C" uint64_t pk_kernel_launches(void) { return pk::g_launches.load(std::memory_order_relaxed); }
