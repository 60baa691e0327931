// Iterative compaction of the macro-node graph behind pk_compact (include/pakman_gb300.h):
// the rounds of independent-set merging that the reference's begin_iterative_compaction
// (src/iterative_compaction.cpp:131-464) runs, for one rank, on sm_103a.
//
// State in HBM (one copy per side, ping-ponged every round; nodes sorted by key):
//   key[n]            (k-1)-mer of the node (uint64, or u128 for k > 32)
//   eoff[n+1]         the node's entries are [eoff[i], eoff[i+1]): prefixes first
//   npre[n]           (npre[i] of them), then suffixes
//   per entry         xoff (base offset of the extension in the arena), xlen (bases,
//                     bit 31 = terminal), count, visit, nbr (the neighbour (k-1)-mer
//                     the extension leads to), beg (prefix_pos, num_wires; prefixes)
//   wire[eoff[i]+i ..] the node's np+ns+1 wire slots (suffix_id, offset, count), as the
//                     reference sizes wiring_info (src/wire.cpp:90-92)
// Extensions are views into one append-only arena of 2-bit bases packed 32 to a
// 64-bit word, first base in the top bits.  Merging a wire (prefix P -> node K ->
// suffix S) writes its string W = P + K + S once, word-aligned; the new suffix of the
// predecessor (W[k-1:]), the new prefix of the successor (W[:|P|+|S|]), both search
// extensions and the partial contig are substrings of W, so no string is copied again.
//
// One round (the reference's loop body, src/iterative_compaction.cpp:276-432):
//   k_cp_mark     ID-set test (generate_id_set, src/merge_mn.cpp:289-432) and the
//                 transfer / contig / arena counts of every ID node's wires
//   scan          offsets and totals (one host read per round)
//   k_cp_emit     survivors to the other side; W strings, transfers and contigs of the
//                 ID nodes in the reference's generation order (iterate_and_pack_mn,
//                 src/merge_mn.cpp:433-550)
//   k_cp_resolve  transfer -> target node by binary search (find_mnode_exists)
//   k_cp_fill     per-target lists of incoming transfers
//   k_cp_apply<0> replays push_to_pred / push_to_succ (src/merge_mn.cpp:1325-1411) per
//                 target in generation order and sizes the new lists
//   k_cp_apply<1> writes the lists and re-wires touched nodes (MacroNode::setup_wiring,
//                 includes/distribute_kmers.h:550-657); other nodes keep their wiring
// and, on the compacted map, the walk (pk_walk; k_walk, below).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/pakman_gb300.h"
#include "pk_internal.h"
#include "pk_runtime.h"
#include "pk_stdsort.cuh"

using namespace pk;

namespace {

typedef unsigned __int128 u128;

constexpr int kMaxList = pk_sort::kSortMax;  // entries per prefix or suffix list on device
constexpr uint32_t kTerm = 0x80000000u;  // xlen bit: terminal entry
constexpr uint32_t kLenMask = 0x7fffffffu;
constexpr int kScanT = 1024, kScanPer = 4, kScanTile = kScanT * kScanPer;

// device error bits of a compaction
enum : uint32_t {
  CE_LIST = 1u,
  CE_TARGET = 2u,
  CE_BALANCE = 4u,
  CE_TERMINAL = 8u,
  CE_BOUNDS = 16u,
  CE_WALK_PREFIX = 32u,  // no prefix of the successor matches (the reference exits)
  CE_WALK_SHARE = 64u,   // a wire's share of the visits is empty (the reference asserts)
  CE_WALK_LONG = 128u,   // a contig reached 500000 bases (the reference asserts)
  CE_WALK_DEPTH = 256u,  // a walk went deeper than its stack
};
constexpr uint32_t kWalkMaxBases = 500000;  // src/walk.cpp:285

struct Tr {            // one TransferNode (src/merge_mn.cpp:483-525)
  uint64_t w;          // arena base offset of W = P + K + S
  uint32_t plen, slen;
  int32_t cnt, vis;    // mn_count
  uint32_t flags;      // bit 0: direction P (push_to_pred), bit 1: mn_terminal
  uint32_t pad;
};
struct Ct {
  uint64_t w, len;
};

template <typename KeyT>
struct Side {
  KeyT* key;
  uint32_t* eoff;
  uint32_t* npre;
  uint64_t* xoff;
  uint32_t* xlen;
  int32_t* cnt;
  int32_t* vis;
  KeyT* nbr;
  int2* beg;
  int3* wire;
};

// ---------------------------------------------------------------- arena ----------
__device__ __forceinline__ uint64_t ar_get(const uint64_t* __restrict__ ar, uint64_t b) {
  const uint64_t w = b >> 5;
  const int s = (int)(b & 31) * 2;
  const uint64_t x = ar[w];
  return s ? (x << s) | (ar[w + 1] >> (64 - s)) : x;
}

// m (1..64) bases of the arena from base offset b, right-aligned
template <typename KeyT>
__device__ __forceinline__ KeyT ar_bases(const uint64_t* __restrict__ ar, uint64_t b, int m) {
  if (m <= 32) return (KeyT)(ar_get(ar, b) >> (64 - 2 * m));
  if constexpr (sizeof(KeyT) == 16) {
    const int r = m - 32;
    return ((KeyT)ar_get(ar, b) << (2 * r)) | (KeyT)(ar_get(ar, b + 32) >> (64 - 2 * r));
  } else {
    return 0;
  }
}

__device__ __forceinline__ bool ar_equal(const uint64_t* __restrict__ ar, uint64_t a, uint64_t b, uint32_t n) {
  for (uint32_t i = 0; i < n; i += 32) {
    const uint32_t m = min(32u, n - i);
    const uint64_t x = ar_get(ar, a + i), y = ar_get(ar, b + i);
    if ((x ^ y) >> (64 - 2 * m)) return false;
  }
  return true;
}

template <typename KeyT>
__device__ __forceinline__ KeyT low_mask(int bases) {
  return bases >= (int)(4 * sizeof(KeyT)) ? ~(KeyT)0 : (((KeyT)1 << (2 * bases)) - 1);
}

// m bases (1..32) of the key from base q (of L), right-aligned
template <typename KeyT>
__device__ __forceinline__ uint64_t key_bases(KeyT key, int L, int q, int m) {
  return (uint64_t)((key >> (2 * (L - q - m))) & low_mask<KeyT>(m));
}

// Writes W = P + K + S at word-aligned base offset d.
template <typename KeyT>
__device__ void write_wire(uint64_t* __restrict__ ar, uint64_t d, uint64_t pb, uint32_t pl, KeyT key, int L,
                           uint64_t sb, uint32_t sl, uint64_t cap_words, uint32_t* err) {
  const uint64_t n = (uint64_t)pl + L + sl;
  const uint64_t words = (n + 31) >> 5, w0 = d >> 5;
  if (w0 + words > cap_words) {
    atomicOr(err, CE_BOUNDS);
    return;
  }
  for (uint64_t j = 0; j < words; j++) {
    const uint64_t lo = j * 32, hi = min(lo + 32, n);
    uint64_t word = 0;
    // P: [0, pl)
    if (lo < pl) {
      const uint64_t a = lo, b = min(hi, (uint64_t)pl);
      const int m = (int)(b - a);
      word |= (ar_get(ar, pb + a) >> (64 - 2 * m)) << (2 * (32 - (int)(a - lo) - m));
    }
    // K: [pl, pl + L)
    {
      const uint64_t a = max(lo, (uint64_t)pl), b = min(hi, (uint64_t)pl + L);
      if (a < b) {
        const int m = (int)(b - a);
        word |= key_bases(key, L, (int)(a - pl), m) << (2 * (32 - (int)(a - lo) - m));
      }
    }
    // S: [pl + L, n)
    {
      const uint64_t a = max(lo, (uint64_t)pl + L), b = hi;
      if (a < b) {
        const int m = (int)(b - a);
        word |= (ar_get(ar, sb + (a - pl - L)) >> (64 - 2 * m)) << (2 * (32 - (int)(a - lo) - m));
      }
    }
    ar[w0 + j] = word;
  }
}

// std::sort as libstdc++ does it (pk_stdsort.cuh)
using pk_sort::RankLess;
using pk_sort::std_sort;

// MacroNode::setup_wiring on lists held in registers / local memory.  The empty
// (terminal) entry of each side gets (1, max(other sum - own sum, 0)) while its count
// is still -1, as on the first wiring.  Writes np+ns+1 wire slots and np begin slots.
__device__ bool setup_wiring(int np, int32_t* pcnt, int32_t* pvis, const bool* pempty, int ns, int32_t* scnt,
                             int32_t* svis, const bool* sempty, int3* wire, int2* beg, uint32_t* err) {
  int pc = 0, sc = 0, ns_id = -1, np_id = -1;
  for (int i = 0; i < ns; i++)
    if (!sempty[i]) sc += svis[i];
  for (int i = 0; i < np; i++)
    if (!pempty[i]) pc += pvis[i];
  for (int i = 0; i < ns; i++)
    if (sempty[i]) {
      ns_id = i;
      if (scnt[i] == -1) {
        scnt[i] = 1;
        svis[i] = max(pc - sc, 0);
      }
    }
  for (int i = 0; i < np; i++)
    if (pempty[i]) {
      np_id = i;
      if (pcnt[i] == -1) {
        pcnt[i] = 1;
        pvis[i] = max(sc - pc, 0);
      }
    }
  const int nw = np + ns + 1;
  for (int w = 0; w < nw; w++) wire[w] = make_int3(0, 0, 0);
  for (int p = 0; p < np; p++) beg[p] = make_int2(0, 0);
  if (ns_id < 0 || np_id < 0) {
    atomicOr(err, CE_TERMINAL);
    return false;
  }
  if (sc + svis[ns_id] != pc + pvis[np_id]) {
    atomicOr(err, CE_BALANCE);
    return false;
  }
  int ip[kMaxList], is[kMaxList];
  for (int i = 0; i < np; i++) ip[i] = i;
  for (int i = 0; i < ns; i++) is[i] = i;
  std_sort(ip, np, RankLess{pvis, pcnt});
  std_sort(is, ns, RankLess{svis, scnt});
  int offs[kMaxList];
  for (int i = 0; i < ns; i++) offs[i] = 0;
  int leftover = sc + svis[ns_id];
  int top_p = 0, top_s = 0, var_p = 0, var_s = 0, wi = 0, p_size = 0, last_pid = -1, begin_pos = -1;
  while (leftover > 0) {
    if (top_p >= np || top_s >= ns || wi >= nw) {
      atomicOr(err, CE_BOUNDS);
      return false;
    }
    const int sid = is[top_s], pid = ip[top_p];
    const int c = min(pvis[pid] - var_p, svis[sid] - var_s);
    wire[wi] = make_int3(sid, offs[sid], c);
    if (last_pid != pid) {
      begin_pos = wi;
      last_pid = pid;
    }
    p_size++;
    wi++;
    leftover -= c;
    var_p += c;
    var_s += c;
    offs[sid] += c;
    if (var_p == pvis[pid]) {
      var_p = 0;
      top_p++;
      beg[pid] = make_int2(begin_pos, p_size);
      p_size = 0;
    }
    if (var_s == svis[sid]) {
      var_s = 0;
      top_s++;
    }
  }
  return true;
}

// ---------------------------------------------------------------- scans ----------
__device__ __forceinline__ uint4 operator+(uint4 a, uint4 b) {
  return make_uint4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ uint4 shfl_up4(uint4 v, int d) {
  return make_uint4(__shfl_up_sync(~0u, v.x, d), __shfl_up_sync(~0u, v.y, d), __shfl_up_sync(~0u, v.z, d),
                    __shfl_up_sync(~0u, v.w, d));
}

// exclusive block scan of one uint4 per thread (kScanT threads); returns the total too
__device__ uint4 block_scan4(uint4 v, uint4* s_w, uint4& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint4 inc = v;
  for (int d = 1; d < 32; d <<= 1) {
    const uint4 o = shfl_up4(inc, d);
    if (lane >= d) inc = inc + o;
  }
  if (lane == 31) s_w[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint4 x = lane < (kScanT / 32) ? s_w[lane] : make_uint4(0, 0, 0, 0);
    for (int d = 1; d < 32; d <<= 1) {
      const uint4 o = shfl_up4(x, d);
      if (lane >= d) x = x + o;
    }
    s_w[lane] = x;  // inclusive over warps
  }
  __syncthreads();
  total = s_w[kScanT / 32 - 1];
  const uint4 before = wid ? s_w[wid - 1] : make_uint4(0, 0, 0, 0);
  const uint4 ex = inc + make_uint4(0u - v.x, 0u - v.y, 0u - v.z, 0u - v.w);
  __syncthreads();
  return before + ex;
}

// pass 1: tile-local exclusive scan into out, tile totals into part
__global__ void __launch_bounds__(kScanT) k_scan_tiles(const uint4* __restrict__ in, uint4* __restrict__ out,
                                                      uint4* __restrict__ part, uint32_t n) {
  __shared__ uint4 s_w[32];
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  uint4 v[kScanPer], sum = make_uint4(0, 0, 0, 0);
#pragma unroll
  for (int q = 0; q < kScanPer; q++) {
    v[q] = base + q < n ? in[base + q] : make_uint4(0, 0, 0, 0);
    sum = sum + v[q];
  }
  uint4 tot;
  uint4 ex = block_scan4(sum, s_w, tot);
#pragma unroll
  for (int q = 0; q < kScanPer; q++) {
    if (base + q < n) out[base + q] = ex;
    ex = ex + v[q];
  }
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// pass 2: one CTA scans the tile totals (any count) and writes the grand total to out[n]
__global__ void __launch_bounds__(kScanT) k_scan_parts(uint4* __restrict__ part, uint32_t nparts,
                                                      uint4* __restrict__ out, uint32_t n) {
  __shared__ uint4 s_w[32];
  uint4 carry = make_uint4(0, 0, 0, 0);
  for (uint32_t b = 0; b < nparts; b += kScanT) {
    const uint32_t i = b + threadIdx.x;
    const uint4 v = i < nparts ? part[i] : make_uint4(0, 0, 0, 0);
    uint4 tot;
    const uint4 ex = block_scan4(v, s_w, tot);
    if (i < nparts) part[i] = carry + ex;
    carry = carry + tot;
  }
  if (threadIdx.x == 0) out[n] = carry;
}

__global__ void k_scan_add(uint4* __restrict__ out, const uint4* __restrict__ part, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = out[i] + part[i / kScanTile];
}

// ------------------------------------------------------------ initial state ------
// Entry counts of the wired map the reference hands to compaction
// (src/wire.cpp:84-92): present extensions plus one terminal entry per side.
__global__ void k_cp_init_count(const uint4* __restrict__ nsuf, const uint4* __restrict__ npre, uint32_t m,
                                uint4* __restrict__ col) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint4 s = nsuf[i], p = npre[i];
  const uint32_t c = (s.x != 0) + (s.y != 0) + (s.z != 0) + (s.w != 0) + (p.x != 0) + (p.y != 0) + (p.z != 0) +
                     (p.w != 0) + 2;
  col[i] = make_uint4(c, 0, 0, 0);
}

__device__ __forceinline__ int32_t visit_of(int32_t c, int32_t cov) {  // (int)ceil(count / coverage)
  int32_t q = c / cov;
  const int32_t r = c % cov;
  if (r != 0 && ((r > 0) == (cov > 0))) q++;
  return q;
}

template <typename KeyT>
__global__ void k_cp_init(const KeyT* __restrict__ nkeys, const uint4* __restrict__ nsuf,
                          const uint4* __restrict__ npre, uint32_t m, int L, int32_t cov,
                          const uint4* __restrict__ col, Side<KeyT> s, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > m) return;
  if (i == m) {
    s.eoff[m] = col[m].x;
    return;
  }
  const KeyT key = nkeys[i];
  const uint32_t e0 = col[i].x;
  s.eoff[i] = e0;
  const uint32_t sc4[4] = {nsuf[i].x, nsuf[i].y, nsuf[i].z, nsuf[i].w};
  const uint32_t pc4[4] = {npre[i].x, npre[i].y, npre[i].z, npre[i].w};
  int32_t pcnt[5], pvis[5], scnt[5], svis[5];
  bool pempty[5], sempty[5];
  int np = 0, ns = 0;
  const KeyT lmask = low_mask<KeyT>(L);
  uint32_t e = e0;
  for (int b = 0; b < 4; b++)
    if (pc4[b]) {
      pcnt[np] = (int32_t)pc4[b];
      pvis[np] = visit_of(pcnt[np], cov);
      pempty[np] = false;
      s.xoff[e] = (uint64_t)b;  // the arena's first word holds A, C, T, G
      s.xlen[e] = 1;
      s.nbr[e] = ((KeyT)b << (2 * (L - 1))) | (key >> 2);
      e++;
      np++;
    }
  pcnt[np] = -1;
  pvis[np] = -1;
  pempty[np] = true;
  s.xoff[e] = 0;
  s.xlen[e] = kTerm;
  s.nbr[e] = 0;
  e++;
  np++;
  for (int b = 0; b < 4; b++)
    if (sc4[b]) {
      scnt[ns] = (int32_t)sc4[b];
      svis[ns] = visit_of(scnt[ns], cov);
      sempty[ns] = false;
      s.xoff[e] = (uint64_t)b;
      s.xlen[e] = 1;
      s.nbr[e] = ((key << 2) | (KeyT)b) & lmask;
      e++;
      ns++;
    }
  scnt[ns] = -1;
  svis[ns] = -1;
  sempty[ns] = true;
  s.xoff[e] = 0;
  s.xlen[e] = kTerm;
  s.nbr[e] = 0;
  ns++;
  s.key[i] = key;
  s.npre[i] = (uint32_t)np;
  setup_wiring(np, pcnt, pvis, pempty, ns, scnt, svis, sempty, s.wire + e0 + i, s.beg + e0, err);
  for (int q = 0; q < np; q++) {
    s.cnt[e0 + q] = pcnt[q];
    s.vis[e0 + q] = pvis[q];
  }
  for (int q = 0; q < ns; q++) {
    s.cnt[e0 + np + q] = scnt[q];
    s.vis[e0 + np + q] = svis[q];
    s.beg[e0 + np + q] = make_int2(0, 0);
  }
}

// ------------------------------------------------------------------ round --------
// Walks the ID node's wires in the reference's order (prefix list order, then the
// prefix's wires) and calls f(p_entry, s_entry, wire_count, emit_pred, emit_succ,
// contig, pred_terminal, succ_terminal) for every wire that emits something.
template <typename KeyT, typename F>
__device__ __forceinline__ void for_each_emit(const Side<KeyT>& s, uint32_t i, KeyT key, F&& f) {
  const uint32_t e0 = s.eoff[i], np = s.npre[i];
  const int3* wire = s.wire + e0 + i;
  for (uint32_t p = 0; p < np; p++) {
    const int2 b = s.beg[e0 + p];
    if (!b.y) continue;
    const uint32_t pe = e0 + p;
    const bool pt = (s.xlen[pe] & kTerm) != 0;
    const bool self_p = !pt && s.nbr[pe] == key;
    for (int t = 0; t < b.y; t++) {
      const int3 w = wire[b.x + t];
      const uint32_t se = e0 + np + (uint32_t)w.x;
      const bool st = (s.xlen[se] & kTerm) != 0;
      if (pt && st) {
        f(pe, se, w.z, false, false, true, false, false);
        continue;
      }
      const bool self_s = !st && s.nbr[se] == key;
      const bool ep = !pt && !self_p, es = !st && !self_s;
      if (ep || es) f(pe, se, w.z, ep, es, false, st || self_s, pt || self_p);
    }
  }
}

template <typename KeyT>
__global__ void __launch_bounds__(256) k_cp_mark(Side<KeyT> s, uint32_t n, int L, uint4* __restrict__ col,
                                                 uint8_t* __restrict__ is_id) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const KeyT key = s.key[i];
  const uint32_t e0 = s.eoff[i], e1 = s.eoff[i + 1];
  bool id = true;
  for (uint32_t e = e0; e < e1; e++)
    if (!(s.xlen[e] & kTerm) && s.nbr[e] > key) {
      id = false;
      break;
    }
  is_id[i] = id;
  uint4 c = make_uint4(0, 0, 0, id ? 0u : 1u);
  if (id) {
    for_each_emit(s, i, key, [&](uint32_t pe, uint32_t se, int, bool ep, bool es, bool contig, bool, bool) {
      const uint32_t len = (s.xlen[pe] & kLenMask) + (uint32_t)L + (s.xlen[se] & kLenMask);
      c.x += (uint32_t)ep + (uint32_t)es;
      c.y += contig;
      c.z += (len + 31) >> 5;
    });
  }
  col[i] = c;
}

template <typename KeyT>
__global__ void __launch_bounds__(256) k_cp_emit(Side<KeyT> s, uint32_t n, int L, const uint4* __restrict__ off,
                                                 const uint8_t* __restrict__ is_id, uint64_t* __restrict__ ar,
                                                 uint64_t ar_word0, uint64_t ar_cap_words, KeyT* __restrict__ tkey,
                                                 Tr* __restrict__ tr, Ct* __restrict__ ct, uint64_t ct0,
                                                 KeyT* __restrict__ nkey, uint32_t* __restrict__ old_of,
                                                 uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const KeyT key = s.key[i];
  const uint4 o = off[i];
  if (!is_id[i]) {
    nkey[o.w] = key;
    old_of[o.w] = i;
    return;
  }
  uint32_t t = o.x, c = o.y;
  uint64_t wd = ar_word0 + o.z;
  for_each_emit(s, i, key, [&](uint32_t pe, uint32_t se, int wcount, bool ep, bool es, bool contig, bool pterm,
                               bool sterm) {
    const uint32_t pl = s.xlen[pe] & kLenMask, sl = s.xlen[se] & kLenMask;
    const uint64_t wb = wd << 5;
    write_wire<KeyT>(ar, wb, s.xoff[pe], pl, key, L, s.xoff[se], sl, ar_cap_words, err);
    wd += ((uint64_t)pl + L + sl + 31) >> 5;
    if (contig) {
      ct[ct0 + c] = Ct{wb, (uint64_t)pl + L + sl};
      c++;
      return;
    }
    const int32_t mc = min(s.cnt[pe], s.cnt[se]);
    if (ep) {  // to the predecessor: its suffix W[L:L+pl] becomes W[L:]
      tkey[t] = s.nbr[pe];
      tr[t] = Tr{wb, pl, sl, mc, wcount, 1u | (pterm ? 2u : 0u), 0u};
      t++;
    }
    if (es) {  // to the successor: its prefix W[pl:pl+sl] becomes W[:pl+sl]
      tkey[t] = s.nbr[se];
      tr[t] = Tr{wb, pl, sl, mc, wcount, sterm ? 2u : 0u, 0u};
      t++;
    }
  });
}

template <typename KeyT>
__global__ void k_cp_resolve(const KeyT* __restrict__ tkey, uint32_t T, const KeyT* __restrict__ nkey, uint32_t n,
                             uint32_t* __restrict__ tgt, uint4* __restrict__ incnt, uint32_t* err) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const KeyT k = tkey[t];
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (nkey[mid] < k) lo = mid + 1;
    else hi = mid;
  }
  if (lo >= n || nkey[lo] != k) {  // the reference prints "was not found in map" and exits
    atomicOr(err, CE_TARGET);
    tgt[t] = ~0u;
    return;
  }
  tgt[t] = lo;
  atomicAdd(&incnt[lo].x, 1u);
}

__global__ void k_cp_fill(const uint32_t* __restrict__ tgt, uint32_t T, const uint4* __restrict__ inoff,
                          uint32_t* __restrict__ fill, uint32_t* __restrict__ inlist) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const uint32_t g = tgt[t];
  if (g == ~0u) return;
  inlist[inoff[g].x + atomicAdd(&fill[g], 1u)] = t;
}

// A list entry during the replay: an old entry (>= 0) or incoming transfer t (-1 - t).
template <typename KeyT>
struct Replay {
  int pre[kMaxList], suf[kMaxList];
  int np, ns;
};

template <typename KeyT, int PASS>
__global__ void __launch_bounds__(128) k_cp_apply(Side<KeyT> a, Side<KeyT> b, uint32_t n, int L,
                                                  const uint32_t* __restrict__ old_of,
                                                  const uint4* __restrict__ inoff, uint32_t* __restrict__ inlist,
                                                  const Tr* __restrict__ tr, const uint64_t* __restrict__ ar,
                                                  uint4* __restrict__ ecol, uint32_t* err) {
  const uint32_t ni = blockIdx.x * blockDim.x + threadIdx.x;
  if (ni > n) return;
  if (PASS == 1 && ni == n) {
    b.eoff[n] = ecol[n].x;
    return;
  }
  if (ni == n) return;
  if (PASS == 1) b.eoff[ni] = ecol[ni].x;
  const uint32_t i = old_of[ni];
  const uint32_t e0 = a.eoff[i], e1 = a.eoff[i + 1], np0 = a.npre[i];
  const uint32_t q0 = inoff[ni].x, q1 = inoff[ni + 1].x;
  if (q0 == q1) {  // untouched: entries, begin slots and wires carry over
    if (PASS == 0) {
      ecol[ni] = make_uint4(e1 - e0, 0, 0, 0);
      return;
    }
    const uint32_t d0 = ecol[ni].x;
    b.npre[ni] = np0;
    for (uint32_t e = e0; e < e1; e++) {
      const uint32_t d = d0 + (e - e0);
      b.xoff[d] = a.xoff[e];
      b.xlen[d] = a.xlen[e];
      b.cnt[d] = a.cnt[e];
      b.vis[d] = a.vis[e];
      b.nbr[d] = a.nbr[e];
      b.beg[d] = a.beg[e];
    }
    for (uint32_t w = 0; w <= e1 - e0; w++) b.wire[d0 + ni + w] = a.wire[e0 + i + w];
    return;
  }
  if (PASS == 0) {  // generation order within the target
    for (uint32_t x = q0 + 1; x < q1; x++) {
      const uint32_t v = inlist[x];
      uint32_t y = x;
      while (y > q0 && inlist[y - 1] > v) {
        inlist[y] = inlist[y - 1];
        y--;
      }
      inlist[y] = v;
    }
  }
  Replay<KeyT> r;
  r.np = (int)np0;
  r.ns = (int)(e1 - e0 - np0);
  if (r.np > kMaxList || r.ns > kMaxList) {
    atomicOr(err, CE_LIST);
    if (PASS == 0) ecol[ni] = make_uint4(e1 - e0, 0, 0, 0);
    return;
  }
  for (int q = 0; q < r.np; q++) r.pre[q] = (int)(e0 + q);
  for (int q = 0; q < r.ns; q++) r.suf[q] = (int)(e0 + np0 + q);
  auto ext_of = [&](int ref, uint64_t& off, uint32_t& len, bool& term) {
    if (ref >= 0) {
      off = a.xoff[ref];
      len = a.xlen[ref] & kLenMask;
      term = (a.xlen[ref] & kTerm) != 0;
    } else {
      const Tr& x = tr[-1 - ref];
      off = x.w + ((x.flags & 1u) ? (uint64_t)L : 0ull);
      len = x.plen + x.slen;
      term = (x.flags & 2u) != 0;
    }
  };
  bool over = false;
  for (uint32_t q = q0; q < q1 && !over; q++) {
    const uint32_t t = inlist[q];
    const Tr x = tr[t];
    const bool to_pred = (x.flags & 1u) != 0;
    // the extension on the target that pointed at the merged node
    const uint64_t so = to_pred ? x.w + L : x.w + x.plen;
    const uint32_t sl = to_pred ? x.plen : x.slen;
    int* lst = to_pred ? r.suf : r.pre;
    int& cnt = to_pred ? r.ns : r.np;
    int hit = -1;
    for (int j = 0; j < cnt; j++) {
      uint64_t eo;
      uint32_t el;
      bool et;
      ext_of(lst[j], eo, el, et);
      if (el == sl && ar_equal(ar, eo, so, sl)) {
        hit = j;
        break;
      }
    }
    bool hterm = false;
    if (hit >= 0) {
      uint64_t eo;
      uint32_t el;
      ext_of(lst[hit], eo, el, hterm);
    }
    if (hit < 0 || hterm) {
      if (cnt >= kMaxList) {
        over = true;
        break;
      }
      lst[cnt++] = -1 - (int)t;
    } else {
      lst[hit] = -1 - (int)t;
    }
  }
  if (over) {
    atomicOr(err, CE_LIST);
    if (PASS == 0) ecol[ni] = make_uint4(e1 - e0, 0, 0, 0);
    return;
  }
  if (PASS == 0) {
    ecol[ni] = make_uint4((uint32_t)(r.np + r.ns), 0, 0, 0);
    return;
  }
  // write the lists, then re-wire
  const uint32_t d0 = ecol[ni].x;
  int32_t pcnt[kMaxList], pvis[kMaxList], scnt[kMaxList], svis[kMaxList];
  bool pempty[kMaxList], sempty[kMaxList];
  for (int side = 0; side < 2; side++) {
    const int* lst = side ? r.suf : r.pre;
    const int cnt = side ? r.ns : r.np;
    const uint32_t base = d0 + (side ? (uint32_t)r.np : 0u);
    for (int j = 0; j < cnt; j++) {
      const int ref = lst[j];
      const uint32_t d = base + j;
      int32_t c, v;
      uint32_t len;
      if (ref >= 0) {
        b.xoff[d] = a.xoff[ref];
        b.xlen[d] = a.xlen[ref];
        b.nbr[d] = a.nbr[ref];
        c = a.cnt[ref];
        v = a.vis[ref];
        len = a.xlen[ref] & kLenMask;
      } else {
        const Tr& x = tr[-1 - ref];
        const bool to_pred = (x.flags & 1u) != 0;
        const uint32_t wl = x.plen + (uint32_t)L + x.slen;
        len = x.plen + x.slen;
        b.xoff[d] = to_pred ? x.w + L : x.w;
        b.xlen[d] = len | ((x.flags & 2u) ? kTerm : 0u);
        // neighbour across the new extension: last k-1 bases of W (a new suffix) or
        // its first k-1 (a new prefix)
        b.nbr[d] = (x.flags & 2u) ? (KeyT)0 : ar_bases<KeyT>(ar, to_pred ? x.w + (wl - L) : x.w, L);
        c = x.cnt;
        v = x.vis;
      }
      b.cnt[d] = c;
      b.vis[d] = v;
      if (side) {
        scnt[j] = c;
        svis[j] = v;
        sempty[j] = len == 0;
      } else {
        pcnt[j] = c;
        pvis[j] = v;
        pempty[j] = len == 0;
      }
    }
  }
  b.npre[ni] = (uint32_t)r.np;
  for (int j = 0; j < r.ns; j++) b.beg[d0 + r.np + j] = make_int2(0, 0);
  setup_wiring(r.np, pcnt, pvis, pempty, r.ns, scnt, svis, sempty, b.wire + d0 + ni, b.beg + d0, err);
  for (int j = 0; j < r.np; j++) b.cnt[d0 + j] = pcnt[j], b.vis[d0 + j] = pvis[j];
  for (int j = 0; j < r.ns; j++) b.cnt[d0 + r.np + j] = scnt[j], b.vis[d0 + r.np + j] = svis[j];
}

// ------------------------------------------------------------------ walk ---------
// traverse_pakgraph / walk (src/walk.cpp:268-533) on the compacted map.
//   k_wk_links   every suffix entry's successor: the node its neighbour key names
//                (find_mnode_exists) and that node's first prefix equal to the first
//                |S| bases of key + S, resolved for all entries in parallel
//   k_walk<0>    one thread per begin k-mer (identify_begin_kmers,
//                src/iterative_compaction.cpp:65-93) runs the depth-first walk over the
//                links, the current frame in registers and the path's frames on a
//                bounded stack in HBM; it counts contigs, bases and pieces
//   k_walk<1>    the same walk writes each contig's begin key and its pieces (the begin
//                prefix and every frame's suffix, as arena views)
//   k_wk_expand  one warp per piece writes its bases (one byte per base)
struct WFrame {
  uint32_t node, e0, np;
  int32_t p, oip, wi, off, rem, share, bpx, bpy, wz, sid;
  uint32_t lenb;  // contig length before this frame's current suffix
};
struct WPiece {
  uint64_t src;  // arena base offset
  uint64_t dst;  // output byte offset
  uint32_t len, pad;
};

__global__ void k_wk_begin_count(const uint32_t* __restrict__ eoff, const uint32_t* __restrict__ npre,
                                 const uint32_t* __restrict__ xlen, const int32_t* __restrict__ vis, uint32_t n,
                                 uint4* __restrict__ col) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t c = 0;
  for (uint32_t e = eoff[i], e1 = eoff[i] + npre[i]; e < e1; e++) c += (vis[e] > 0 && (xlen[e] & kTerm)) ? 1u : 0u;
  col[i] = make_uint4(c, 0, 0, 0);
}

__global__ void k_wk_begins(const uint32_t* __restrict__ eoff, const uint32_t* __restrict__ npre,
                            const uint32_t* __restrict__ xlen, const int32_t* __restrict__ vis, uint32_t n,
                            const uint4* __restrict__ off, uint2* __restrict__ begins) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t o = off[i].x;
  const uint32_t e0 = eoff[i];
  for (uint32_t q = 0; q < npre[i]; q++)
    if (vis[e0 + q] > 0 && (xlen[e0 + q] & kTerm)) begins[o++] = make_uint2(i, q);
}

// m (<= 32) bases of key + S from position q, right-aligned
template <typename KeyT>
__device__ __forceinline__ uint64_t ks_bases(const uint64_t* __restrict__ ar, KeyT key, int L, uint64_t soff,
                                             uint32_t q, int m) {
  uint64_t v = 0;
  const uint32_t a = q, b = q + m;
  if (a < (uint32_t)L) {
    const int mk = (int)(min(b, (uint32_t)L) - a);
    v = key_bases(key, L, (int)a, mk);
    if (b > (uint32_t)L) {
      const int ms = (int)(b - L);
      v = (v << (2 * ms)) | (ar_get(ar, soff) >> (64 - 2 * ms));
    }
  } else {
    v = ar_get(ar, soff + (a - L)) >> (64 - 2 * m);
  }
  return v;
}

// link[e] for suffix entry e of node i: (successor node, its prefix index);
// (~0, 0) when no node has the neighbour key, (node, ~0) when no prefix matches
template <typename KeyT>
__global__ void __launch_bounds__(256) k_wk_links(Side<KeyT> s, uint32_t n, int L, const uint64_t* __restrict__ ar,
                                                  uint2* __restrict__ link) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t e0 = s.eoff[i], e1 = s.eoff[i + 1], np = s.npre[i];
  const KeyT ckey = s.key[i];
  for (uint32_t se = e0 + np; se < e1; se++) {
    if (s.xlen[se] & kTerm) continue;
    const uint32_t sl = s.xlen[se] & kLenMask;
    const KeyT nk = s.nbr[se];
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (s.key[mid] < nk) lo = mid + 1;
      else hi = mid;
    }
    if (lo >= n || s.key[lo] != nk) {
      link[se] = make_uint2(~0u, 0u);
      continue;
    }
    const uint32_t q0 = s.eoff[lo], qn = s.npre[lo];
    uint32_t q = ~0u;
    for (uint32_t j = 0; j < qn && q == ~0u; j++) {
      if ((s.xlen[q0 + j] & kLenMask) != sl) continue;
      bool eq = true;
      for (uint32_t x = 0; x < sl && eq; x += 32) {
        const int m = (int)min(32u, sl - x);
        eq = (ar_get(ar, s.xoff[q0 + j] + x) >> (64 - 2 * m)) == ks_bases(ar, ckey, L, s.xoff[se], x, m);
      }
      if (eq) q = j;
    }
    link[se] = make_uint2(lo, q);
  }
}

template <typename KeyT, int PASS>
__global__ void __launch_bounds__(128) k_walk(Side<KeyT> s, int L, const uint2* __restrict__ begins, uint32_t nb,
                                              const uint2* __restrict__ link, WFrame* __restrict__ stk, uint32_t cap,
                                              uint4* __restrict__ col, const uint4* __restrict__ off,
                                              uint64_t* __restrict__ ct_off, WPiece* __restrict__ pieces,
                                              uint8_t* __restrict__ out, uint32_t* err) {
  // one walk per warp (lane 0): independent walks diverge completely, so they do not
  // share a warp
  const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if ((threadIdx.x & 31) != 0 || b >= nb) return;
  WFrame* st = stk + (uint64_t)b * cap;
  const uint2 bg = begins[b];
  const uint32_t be = s.eoff[bg.x] + bg.y;
  const uint32_t plen0 = s.xlen[be] & kLenMask;
  uint32_t nct = 0, npc = 0;
  uint64_t nbases = 0;
  uint32_t ci = PASS ? off[b].x : 0u, pc = PASS ? off[b].z : 0u;
  uint64_t bo = PASS ? off[b].y : 0ull;
  int d = 0;
  WFrame f;
  f.node = bg.x;
  f.e0 = s.eoff[bg.x];
  f.np = s.npre[bg.x];
  f.p = (int32_t)bg.y;
  f.oip = 0;
  f.wi = 0;
  f.off = 0;
  f.rem = s.vis[be];
  f.share = -1;
  {
    const int2 bp = s.beg[f.e0 + f.p];
    f.bpx = bp.x;
    f.bpy = bp.y;
  }
  f.wz = 0;
  f.sid = -1;
  f.lenb = 0;
  uint32_t len = plen0 + (uint32_t)L;
  while (true) {
    if (f.wi >= f.bpy) {  // this walk is done: back to the parent
      if (d == 0) break;
      f = st[--d];
      f.rem -= f.share;
      f.share = -1;
      len = f.lenb;
      f.off += f.wz;
      f.wi++;
      continue;
    }
    const int3 w = s.wire[f.e0 + f.node + f.bpx + f.wi];
    if (f.off + w.z <= f.oip || f.off > f.oip + f.rem) {
      f.off += w.z;
      f.wi++;
      continue;
    }
    const int oiw = f.oip <= f.off ? 0 : f.oip - f.off;
    const int next_off = w.y + oiw;
    const int share = min(f.rem, w.z - oiw);
    const uint32_t se = f.e0 + f.np + (uint32_t)w.x;
    const uint32_t xl = s.xlen[se], sl = xl & kLenMask;
    if (xl & kTerm) {  // a contig: begin prefix, begin key, the frames' suffixes, this one
      const uint32_t clen = len + sl;
      if (PASS) {
        ct_off[ci++] = bo;
        for (int x = 0; x < L; x++)
          out[bo + plen0 + x] = (uint8_t)key_bases(s.key[bg.x], L, x, 1);
        if (plen0) pieces[pc++] = WPiece{s.xoff[be], bo, plen0, 0};
        for (int q = 0; q < d; q++) {
          const WFrame& g = st[q];
          const uint32_t ge = g.e0 + g.np + (uint32_t)g.sid;
          const uint32_t gl = s.xlen[ge] & kLenMask;
          if (gl) pieces[pc++] = WPiece{s.xoff[ge], bo + g.lenb, gl, 0};
        }
        if (sl) pieces[pc++] = WPiece{s.xoff[se], bo + len, sl, 0};
        bo += clen;
      } else {
        npc += (plen0 ? 1u : 0u) + (sl ? 1u : 0u);
        for (int q = 0; q < d; q++) npc++;
      }
      nct++;
      nbases += clen;
      f.rem -= share;
      f.off += w.z;
      f.wi++;
      continue;
    }
    const uint2 lk = link[se];
    if (lk.x == ~0u) {
      atomicOr(err, CE_TARGET);
      break;
    }
    if (lk.y == ~0u) {
      atomicOr(err, CE_WALK_PREFIX);
      break;
    }
    if (share <= 0) {
      atomicOr(err, CE_WALK_SHARE);
      break;
    }
    if (len + sl >= kWalkMaxBases) {
      atomicOr(err, CE_WALK_LONG);
      break;
    }
    if (d + 1 >= (int)cap) {
      atomicOr(err, CE_WALK_DEPTH);
      break;
    }
    f.share = share;
    f.sid = w.x;
    f.wz = w.z;
    f.lenb = len;
    st[d++] = f;
    len += sl;
    f.node = lk.x;
    f.e0 = s.eoff[lk.x];
    f.np = s.npre[lk.x];
    f.p = (int32_t)lk.y;
    f.oip = next_off;
    f.wi = 0;
    f.off = 0;
    f.rem = share;
    f.share = -1;
    const int2 bp = s.beg[f.e0 + f.p];
    f.bpx = bp.x;
    f.bpy = bp.y;
  }
  if (!PASS) col[b] = make_uint4(nct, (uint32_t)nbases, npc, 0);
}

// one warp per piece: its bases, one byte each
__global__ void k_wk_expand(const WPiece* __restrict__ pieces, uint32_t np, const uint64_t* __restrict__ ar,
                            uint8_t* __restrict__ out) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= np) return;
  const WPiece pc = pieces[w];
  for (uint32_t i = lane; i < pc.len; i += 32) out[pc.dst + i] = (uint8_t)(ar_get(ar, pc.src + i) >> 62);
}

// ------------------------------------------------------------- copy-out ---------
__global__ void k_cp_lengths(const uint32_t* __restrict__ xlen, uint32_t E, uint4* __restrict__ col) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < E) col[e] = make_uint4(xlen[e] & kLenMask, 0, 0, 0);
}
__global__ void k_cp_ct_lengths(const Ct* __restrict__ ct, uint32_t C, uint4* __restrict__ col) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C) col[c] = make_uint4((uint32_t)ct[c].len, 0, 0, 0);
}

// one warp per string: bases to one byte each (codes 0..3)
__global__ void k_cp_unpack(const uint64_t* __restrict__ ar, const uint64_t* __restrict__ src,
                            const uint32_t* __restrict__ len_or_null, const Ct* __restrict__ ct,
                            const uint4* __restrict__ dst, uint32_t count, uint8_t* __restrict__ out) {
  const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (s >= count) return;
  uint64_t b;
  uint32_t n;
  if (ct) {
    b = ct[s].w;
    n = (uint32_t)ct[s].len;
  } else {
    b = src[s];
    n = len_or_null[s] & kLenMask;
  }
  uint8_t* o = out + dst[s].x;
  for (uint32_t i = lane; i < n; i += 32) o[i] = (uint8_t)(ar_get(ar, b + i) >> 62);
}

__global__ void k_cp_entries(const uint32_t* __restrict__ xlen, const int32_t* __restrict__ cnt,
                             const int32_t* __restrict__ vis, const int2* __restrict__ beg,
                             const uint4* __restrict__ pos, uint32_t E, pk_compact_entry* __restrict__ out) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  pk_compact_entry x;
  x.ext_offset = pos[e].x;
  x.ext_length = xlen[e] & kLenMask;
  x.count = cnt[e];
  x.visit = vis[e];
  x.terminal = (xlen[e] & kTerm) ? 1 : 0;
  x.prefix_pos = beg[e].x;
  x.num_wires = beg[e].y;
  out[e] = x;
}

}  // namespace

// ================================================================ host ==============
namespace pk {

// Buffers of one compaction, owned by the job (freed with it).
struct CpState {
  enum {
    KEY, EOFF, NPRE, XOFF, XLEN, CNT, VIS, NBR, BEG, WIRE, NSIDE
  };
  DevBuf side[2][NSIDE];
  DevBuf arena, col, off, part, is_id, tkey, tr, tgt, incnt, inoff, fill, inlist, ecol, eoff2, old_of, ct, tot,
      epos, cpos, ubuf, wk_begins, wk_stack, wk_col, wk_pos, wk_off, wk_out, wk_links, wk_pieces;
  uint64_t wk_begins_n = 0, wk_n = 0, wk_bases = 0;
  uint32_t wk_depth = 0;
  bool wk_done = false;
  int cur = 0;
  uint64_t n = 0, E = 0, arena_words = 0, arena_cap = 0, C = 0, ct_cap = 0;
  uint64_t ext_bases = 0, ct_bases = 0;
  int rounds = 0;
  int L = 0;
  bool wide = false;
  bool done = false;
  uint32_t* d_err = nullptr;
  uint4* h_tot = nullptr;  // pinned
};

}  // namespace pk

namespace {

pk_status cp_alloc(pk_job* j, DevBuf& b, size_t bytes) { return job_alloc(j, b, bytes); }

// grows b to at least `bytes`, keeping its first `keep` bytes
pk_status cp_grow(pk_job* j, DevBuf& b, size_t bytes, size_t keep) {
  if (b.p && b.bytes >= bytes) return PK_OK;
  DevBuf nb;
  PK_TRY(job_alloc(j, nb, bytes));
  if (keep && b.p) PK_CUDA(cudaMemcpyAsync(nb.p, b.p, keep, cudaMemcpyDeviceToDevice, j->stream));
  if (b.p) {
    cudaFreeAsync(b.p, j->stream);
    j->ctx->used -= b.bytes;
  }
  b = nb;
  return PK_OK;
}

template <typename KeyT>
Side<KeyT> side_of(CpState& c, int s) {
  DevBuf* d = c.side[s];
  return Side<KeyT>{(KeyT*)d[CpState::KEY].p,  (uint32_t*)d[CpState::EOFF].p, (uint32_t*)d[CpState::NPRE].p,
                    (uint64_t*)d[CpState::XOFF].p, (uint32_t*)d[CpState::XLEN].p, (int32_t*)d[CpState::CNT].p,
                    (int32_t*)d[CpState::VIS].p, (KeyT*)d[CpState::NBR].p, (int2*)d[CpState::BEG].p,
                    (int3*)d[CpState::WIRE].p};
}

template <typename KeyT>
pk_status alloc_side(pk_job* j, CpState& c, int s, uint64_t n, uint64_t E) {
  DevBuf* d = c.side[s];
  PK_TRY(cp_alloc(j, d[CpState::KEY], sizeof(KeyT) * (n + 1)));
  PK_TRY(cp_alloc(j, d[CpState::EOFF], 4 * (n + 1)));
  PK_TRY(cp_alloc(j, d[CpState::NPRE], 4 * (n + 1)));
  PK_TRY(cp_alloc(j, d[CpState::XOFF], 8 * (E + 1)));
  PK_TRY(cp_alloc(j, d[CpState::XLEN], 4 * (E + 1)));
  PK_TRY(cp_alloc(j, d[CpState::CNT], 4 * (E + 1)));
  PK_TRY(cp_alloc(j, d[CpState::VIS], 4 * (E + 1)));
  PK_TRY(cp_alloc(j, d[CpState::NBR], sizeof(KeyT) * (E + 1)));
  PK_TRY(cp_alloc(j, d[CpState::BEG], 8 * (E + 1)));
  PK_TRY(cp_alloc(j, d[CpState::WIRE], 12 * (E + n + 1)));
  return PK_OK;
}

// exclusive scan of n uint4 (in place allowed: in == out is not; out holds n+1)
pk_status scan4(pk_job* j, CpState& c, const uint4* in, uint4* out, uint64_t n) {
  const uint32_t tiles = (uint32_t)((n + kScanTile - 1) / kScanTile);
  PK_TRY(cp_alloc(j, c.part, sizeof(uint4) * (tiles + 1)));
  uint4* part = (uint4*)c.part.p;
  if (tiles) pk::note_launch(), k_scan_tiles<<<tiles, kScanT, 0, j->stream>>>(in, out, part, (uint32_t)n);
  pk::note_launch(), k_scan_parts<<<1, kScanT, 0, j->stream>>>(part, tiles, out, (uint32_t)n);
  if (n) pk::note_launch(), k_scan_add<<<(uint32_t)((n + 255) / 256), 256, 0, j->stream>>>(out, part, (uint32_t)n);
  PK_CUDA(cudaGetLastError());
  return PK_OK;
}

pk_status read_total(pk_job* j, CpState& c, const uint4* at, uint4* out) {
  PK_CUDA(cudaMemcpyAsync(c.h_tot, at, sizeof(uint4), cudaMemcpyDeviceToHost, j->stream));
  PK_CUDA(cudaMemcpyAsync(c.h_tot + 1, c.d_err, 4, cudaMemcpyDeviceToHost, j->stream));
  PK_CUDA(cudaStreamSynchronize(j->stream));
  *out = c.h_tot[0];
  return PK_OK;
}

pk_status check_err(CpState& c) {
  const uint32_t e = c.h_tot[1].x;
  if (!e) return PK_OK;
  std::string m = "compaction: ";
  if (e & CE_LIST) m += "a prefix or suffix list grew past 32 entries; ";
  if (e & CE_TARGET) m += "a transfer names a node that is not in the map (the reference exits); ";
  if (e & CE_BALANCE) m += "a node's visits do not balance (the reference asserts); ";
  if (e & CE_TERMINAL) m += "a node lost its terminal entry; ";
  if (e & CE_BOUNDS) m += "an index fell outside its buffer; ";
  if (e & CE_WALK_PREFIX) m += "walk: no prefix of a successor matches (the reference exits); ";
  if (e & CE_WALK_SHARE) m += "walk: a wire's share of the visits is empty (the reference asserts); ";
  if (e & CE_WALK_LONG) m += "walk: a contig reached 500000 bases (the reference asserts); ";
  if (e & CE_WALK_DEPTH) m += "walk: a path went deeper than the walk stack; ";
  return set_error(PK_ERR_DEVICE, m);
}

inline uint32_t blocks(uint64_t n, int t) { return (uint32_t)((n + t - 1) / t); }

template <typename KeyT>
pk_status cp_init(pk_job* j, CpState& c, int32_t cov) {
  const uint64_t m = j->h_sc->n_nodes;
  PK_TRY(cp_alloc(j, c.col, sizeof(uint4) * (m + 1)));
  PK_TRY(cp_alloc(j, c.off, sizeof(uint4) * (m + 1)));
  if (m) pk::note_launch(), k_cp_init_count<<<blocks(m, 256), 256, 0, j->stream>>>((const uint4*)j->nsuf.p, (const uint4*)j->npre.p,
                                                                  (uint32_t)m, (uint4*)c.col.p);
  PK_TRY(scan4(j, c, (const uint4*)c.col.p, (uint4*)c.off.p, m));
  uint4 tot;
  PK_TRY(read_total(j, c, (const uint4*)c.off.p + m, &tot));
  c.n = m;
  c.E = tot.x;
  c.cur = 0;
  PK_TRY(alloc_side<KeyT>(j, c, 0, m, c.E));
  // arena: word 0 holds the one-base extensions A, C, T, G; one zero word of padding
  c.arena_cap = std::max<uint64_t>(1024, (c.E + 1) * 4);
  PK_TRY(cp_alloc(j, c.arena, 8 * (c.arena_cap + 1)));
  const uint64_t w0 = 0x1B00000000000000ull;
  PK_CUDA(cudaMemsetAsync(c.arena.p, 0, 16, j->stream));
  PK_CUDA(cudaMemcpyAsync(c.arena.p, &w0, 8, cudaMemcpyHostToDevice, j->stream));
  c.arena_words = 1;
  pk::note_launch(), k_cp_init<KeyT><<<blocks(m + 1, 128), 128, 0, j->stream>>>((const KeyT*)j->nkeys.p, (const uint4*)j->nsuf.p,
                                                              (const uint4*)j->npre.p, (uint32_t)m, c.L, cov,
                                                              (const uint4*)c.off.p, side_of<KeyT>(c, 0), c.d_err);
  PK_CUDA(cudaGetLastError());
  // the pageable 8-byte copy above must land before the host value goes away
  PK_CUDA(cudaStreamSynchronize(j->stream));
  return PK_OK;
}

template <typename KeyT>
pk_status cp_round(pk_job* j, CpState& c) {
  const uint64_t n = c.n;
  Side<KeyT> a = side_of<KeyT>(c, c.cur);
  PK_TRY(cp_alloc(j, c.col, sizeof(uint4) * (n + 1)));
  PK_TRY(cp_alloc(j, c.off, sizeof(uint4) * (n + 1)));
  PK_TRY(cp_alloc(j, c.is_id, n + 1));
  pk::note_launch(), k_cp_mark<KeyT><<<blocks(n, 256), 256, 0, j->stream>>>(a, (uint32_t)n, c.L, (uint4*)c.col.p, (uint8_t*)c.is_id.p);
  PK_TRY(scan4(j, c, (const uint4*)c.col.p, (uint4*)c.off.p, n));
  uint4 tot;
  PK_TRY(read_total(j, c, (const uint4*)c.off.p + n, &tot));
  PK_TRY(check_err(c));
  const uint64_t T = tot.x, C = tot.y, WB = tot.z, n2 = tot.w;
  // capacities: transfers, contigs (kept across rounds), arena (kept), next side
  PK_TRY(cp_alloc(j, c.tkey, sizeof(KeyT) * (T + 1)));
  PK_TRY(cp_alloc(j, c.tr, sizeof(Tr) * (T + 1)));
  PK_TRY(cp_alloc(j, c.tgt, 4 * (T + 1)));
  PK_TRY(cp_alloc(j, c.inlist, 4 * (T + 1)));
  if (c.C + C > c.ct_cap) {
    const uint64_t cap = std::max<uint64_t>(c.C + C, c.ct_cap + c.ct_cap / 2 + 1024);
    PK_TRY(cp_grow(j, c.ct, sizeof(Ct) * cap, sizeof(Ct) * c.C));
    c.ct_cap = cap;
  }
  if (c.arena_words + WB > c.arena_cap) {
    const uint64_t cap = std::max<uint64_t>(c.arena_words + WB, c.arena_cap + c.arena_cap / 2);
    PK_TRY(cp_grow(j, c.arena, 8 * (cap + 1), 8 * c.arena_words));
    c.arena_cap = cap;
  }
  const int nb = 1 - c.cur;
  PK_TRY(alloc_side<KeyT>(j, c, nb, n2, c.E + T));
  PK_TRY(cp_alloc(j, c.old_of, 4 * (n2 + 1)));
  Side<KeyT> b = side_of<KeyT>(c, nb);
  pk::note_launch(), k_cp_emit<KeyT><<<blocks(n, 256), 256, 0, j->stream>>>(
      a, (uint32_t)n, c.L, (const uint4*)c.off.p, (const uint8_t*)c.is_id.p, (uint64_t*)c.arena.p, c.arena_words,
      c.arena_cap, (KeyT*)c.tkey.p, (Tr*)c.tr.p, (Ct*)c.ct.p, c.C, b.key, (uint32_t*)c.old_of.p, c.d_err);
  PK_CUDA(cudaGetLastError());
  PK_TRY(cp_alloc(j, c.incnt, sizeof(uint4) * (n2 + 1)));
  PK_TRY(cp_alloc(j, c.inoff, sizeof(uint4) * (n2 + 1)));
  PK_TRY(cp_alloc(j, c.fill, 4 * (n2 + 1)));
  PK_TRY(cp_alloc(j, c.ecol, sizeof(uint4) * (n2 + 1)));
  PK_TRY(cp_alloc(j, c.eoff2, sizeof(uint4) * (n2 + 1)));
  PK_CUDA(cudaMemsetAsync(c.incnt.p, 0, sizeof(uint4) * (n2 + 1), j->stream));
  PK_CUDA(cudaMemsetAsync(c.fill.p, 0, 4 * (n2 + 1), j->stream));
  if (T)
    pk::note_launch(), k_cp_resolve<KeyT><<<blocks(T, 256), 256, 0, j->stream>>>((const KeyT*)c.tkey.p, (uint32_t)T, b.key,
                                                               (uint32_t)n2, (uint32_t*)c.tgt.p, (uint4*)c.incnt.p,
                                                               c.d_err);
  PK_TRY(scan4(j, c, (const uint4*)c.incnt.p, (uint4*)c.inoff.p, n2));
  if (T)
    pk::note_launch(), k_cp_fill<<<blocks(T, 256), 256, 0, j->stream>>>((const uint32_t*)c.tgt.p, (uint32_t)T,
                                                     (const uint4*)c.inoff.p, (uint32_t*)c.fill.p,
                                                     (uint32_t*)c.inlist.p);
  pk::note_launch(), k_cp_apply<KeyT, 0><<<blocks(n2 + 1, 128), 128, 0, j->stream>>>(
      a, b, (uint32_t)n2, c.L, (const uint32_t*)c.old_of.p, (const uint4*)c.inoff.p, (uint32_t*)c.inlist.p,
      (const Tr*)c.tr.p, (const uint64_t*)c.arena.p, (uint4*)c.ecol.p, c.d_err);
  PK_TRY(scan4(j, c, (const uint4*)c.ecol.p, (uint4*)c.eoff2.p, n2));
  pk::note_launch(), k_cp_apply<KeyT, 1><<<blocks(n2 + 1, 128), 128, 0, j->stream>>>(
      a, b, (uint32_t)n2, c.L, (const uint32_t*)c.old_of.p, (const uint4*)c.inoff.p, (uint32_t*)c.inlist.p,
      (const Tr*)c.tr.p, (const uint64_t*)c.arena.p, (uint4*)c.eoff2.p, c.d_err);
  PK_CUDA(cudaGetLastError());
  uint4 etot;
  PK_TRY(read_total(j, c, (const uint4*)c.eoff2.p + n2, &etot));
  PK_TRY(check_err(c));
  c.arena_words += WB;
  c.C += C;
  c.n = n2;
  c.E = etot.x;
  c.cur = nb;
  c.rounds++;
  return PK_OK;
}

template <typename KeyT>
pk_status cp_finish(pk_job* j, CpState& c) {
  PK_TRY(cp_alloc(j, c.col, sizeof(uint4) * (std::max(c.E, c.C) + 1)));
  PK_TRY(cp_alloc(j, c.epos, sizeof(uint4) * (c.E + 1)));
  PK_TRY(cp_alloc(j, c.cpos, sizeof(uint4) * (c.C + 1)));
  Side<KeyT> a = side_of<KeyT>(c, c.cur);
  if (c.E) pk::note_launch(), k_cp_lengths<<<blocks(c.E, 256), 256, 0, j->stream>>>(a.xlen, (uint32_t)c.E, (uint4*)c.col.p);
  PK_TRY(scan4(j, c, (const uint4*)c.col.p, (uint4*)c.epos.p, c.E));
  uint4 t1, t2;
  PK_TRY(read_total(j, c, (const uint4*)c.epos.p + c.E, &t1));
  if (c.C) pk::note_launch(), k_cp_ct_lengths<<<blocks(c.C, 256), 256, 0, j->stream>>>((const Ct*)c.ct.p, (uint32_t)c.C, (uint4*)c.col.p);
  PK_TRY(scan4(j, c, (const uint4*)c.col.p, (uint4*)c.cpos.p, c.C));
  PK_TRY(read_total(j, c, (const uint4*)c.cpos.p + c.C, &t2));
  PK_TRY(check_err(c));
  c.ext_bases = t1.x;
  c.ct_bases = t2.x;
  c.done = true;
  return PK_OK;
}

template <typename KeyT>
pk_status cp_walk(pk_job* j, CpState& c) {
  Side<KeyT> a = side_of<KeyT>(c, c.cur);
  const uint64_t n = c.n;
  cudaStream_t st = j->stream;
  PK_TRY(cp_alloc(j, c.col, sizeof(uint4) * (n + 1)));
  PK_TRY(cp_alloc(j, c.off, sizeof(uint4) * (n + 1)));
  if (n) pk::note_launch(), k_wk_begin_count<<<blocks(n, 256), 256, 0, st>>>(a.eoff, a.npre, a.xlen, a.vis, (uint32_t)n, (uint4*)c.col.p);
  PK_TRY(scan4(j, c, (const uint4*)c.col.p, (uint4*)c.off.p, n));
  uint4 t;
  PK_TRY(read_total(j, c, (const uint4*)c.off.p + n, &t));
  const uint64_t B = t.x;
  PK_TRY(cp_alloc(j, c.wk_begins, sizeof(uint2) * (B + 1)));
  PK_TRY(cp_alloc(j, c.wk_links, sizeof(uint2) * (c.E + 1)));
  if (n) {
    pk::note_launch(), k_wk_begins<<<blocks(n, 256), 256, 0, st>>>(a.eoff, a.npre, a.xlen, a.vis, (uint32_t)n, (const uint4*)c.off.p,
                                                (uint2*)c.wk_begins.p);
    pk::note_launch(), k_wk_links<KeyT><<<blocks(n, 256), 256, 0, st>>>(a, (uint32_t)n, c.L, (const uint64_t*)c.arena.p,
                                                     (uint2*)c.wk_links.p);
  }
  // frames per walk: 2^26 over all walks, at least 256 and at most 2^20 each
  const uint64_t cap = std::min<uint64_t>(1u << 20, std::max<uint64_t>(256, (1ull << 26) / std::max<uint64_t>(B, 1)));
  PK_TRY(cp_alloc(j, c.wk_stack, sizeof(WFrame) * cap * std::max<uint64_t>(B, 1)));
  PK_TRY(cp_alloc(j, c.wk_col, sizeof(uint4) * (B + 1)));
  PK_TRY(cp_alloc(j, c.wk_pos, sizeof(uint4) * (B + 1)));
  if (B)
    pk::note_launch(), k_walk<KeyT, 0><<<blocks(B * 32, 128), 128, 0, st>>>(a, c.L, (const uint2*)c.wk_begins.p, (uint32_t)B,
                                                   (const uint2*)c.wk_links.p, (WFrame*)c.wk_stack.p, (uint32_t)cap,
                                                   (uint4*)c.wk_col.p, nullptr, nullptr, nullptr, nullptr, c.d_err);
  PK_TRY(scan4(j, c, (const uint4*)c.wk_col.p, (uint4*)c.wk_pos.p, B));
  PK_TRY(read_total(j, c, (const uint4*)c.wk_pos.p + B, &t));
  PK_TRY(check_err(c));
  const uint64_t NC = t.x, NB = t.y, NP = t.z;
  PK_TRY(cp_alloc(j, c.wk_off, 8 * (NC + 1)));
  PK_TRY(cp_alloc(j, c.wk_out, NB + 1));
  PK_TRY(cp_alloc(j, c.wk_pieces, sizeof(WPiece) * (NP + 1)));
  if (B)
    pk::note_launch(), k_walk<KeyT, 1><<<blocks(B * 32, 128), 128, 0, st>>>(a, c.L, (const uint2*)c.wk_begins.p, (uint32_t)B,
                                                   (const uint2*)c.wk_links.p, (WFrame*)c.wk_stack.p, (uint32_t)cap,
                                                   nullptr, (const uint4*)c.wk_pos.p, (uint64_t*)c.wk_off.p,
                                                   (WPiece*)c.wk_pieces.p, (uint8_t*)c.wk_out.p, c.d_err);
  if (NP)
    pk::note_launch(), k_wk_expand<<<blocks(NP * 32, 256), 256, 0, st>>>((const WPiece*)c.wk_pieces.p, (uint32_t)NP,
                                                       (const uint64_t*)c.arena.p, (uint8_t*)c.wk_out.p);
  PK_CUDA(cudaMemcpyAsync((uint64_t*)c.wk_off.p + NC, &NB, 8, cudaMemcpyHostToDevice, st));
  PK_CUDA(cudaGetLastError());
  PK_TRY(read_total(j, c, (const uint4*)c.wk_pos.p + B, &t));
  PK_TRY(check_err(c));
  c.wk_begins_n = B;
  c.wk_n = NC;
  c.wk_bases = NB;
  c.wk_depth = (uint32_t)cap;
  c.wk_done = true;
  return PK_OK;
}

}  // namespace

void pk::cp_free(pk_job* j) {
  CpState* c = j->cp;
  if (!c) return;
  for (int s = 0; s < 2; s++)
    for (int b = 0; b < CpState::NSIDE; b++) {
      DevBuf& d = c->side[s][b];
      if (d.p) {
        cudaFreeAsync(d.p, j->stream);
        j->ctx->used -= d.bytes;
      }
    }
  DevBuf* rest[] = {&c->arena,  &c->col,      &c->off,    &c->part,   &c->is_id,  &c->tkey,
                    &c->tr,     &c->tgt,      &c->incnt,  &c->inoff,  &c->fill,   &c->inlist,
                    &c->ecol,   &c->eoff2,    &c->old_of, &c->ct,     &c->tot,    &c->epos,
                    &c->cpos,   &c->ubuf,     &c->wk_begins, &c->wk_stack, &c->wk_col, &c->wk_pos,
                    &c->wk_off, &c->wk_out, &c->wk_links, &c->wk_pieces};
  for (DevBuf* d : rest)
    if (d->p) {
      cudaFreeAsync(d->p, j->stream);
      j->ctx->used -= d->bytes;
    }
  cudaStreamSynchronize(j->stream);
  if (c->d_err) cudaFree(c->d_err);
  if (c->h_tot) cudaFreeHost(c->h_tot);
  delete c;
  j->cp = nullptr;
}

static pk_status fill_info(CpState& c, pk_compaction_info* o) {
  if (!o) return PK_OK;
  memset(o, 0, sizeof(*o));
  o->n_nodes = c.n;
  o->n_entries = c.E;
  o->n_contigs = c.C;
  o->ext_bases = c.ext_bases;
  o->contig_bases = c.ct_bases;
  o->rounds = c.rounds;
  o->key_bytes = c.wide ? 16 : 8;
  return PK_OK;
}

extern "C" pk_status pk_compact(pk_job* j, uint64_t threshold, int32_t coverage, pk_compaction_info* info) {
  if (!j) return set_error(PK_ERR_INVALID, "job is null");
  if (j->stage < 3) return set_error(PK_ERR_STATE, "no macro-nodes: call pk_build_macro_nodes first");
  const int32_t cov = coverage ? coverage : j->params.coverage;
  if (cov <= 0) return set_error(PK_ERR_INVALID, "coverage must be >= 1");
  PK_TRY(set_device(j->ctx));
  PK_TRY(sync_scalars(j));
  cp_free(j);
  j->cp = new CpState();
  CpState& c = *j->cp;
  c.wide = j->wide != 0;
  c.L = j->params.k - 1;
  PK_CUDA(cudaMalloc(&c.d_err, 16));
  PK_CUDA(cudaMemsetAsync(c.d_err, 0, 16, j->stream));
  PK_CUDA(cudaHostAlloc(&c.h_tot, 2 * sizeof(uint4), cudaHostAllocDefault));
  mark_begin(j, ST_COMPACT);
  pk_status s = c.wide ? cp_init<u128>(j, c, cov) : cp_init<uint64_t>(j, c, cov);
  while (s == PK_OK && c.n > threshold) {
    const uint64_t before = c.n;
    s = c.wide ? cp_round<u128>(j, c) : cp_round<uint64_t>(j, c);
    // the node with the largest key is always in the ID set, so every round shrinks
    // the map; a round that does not is a fault, not a reason to loop on
    if (s == PK_OK && c.n >= before)
      s = set_error(PK_ERR_DEVICE, "a compaction round merged no node (" + std::to_string(before) +
                                       " nodes before and after)");
  }
  if (s == PK_OK) s = c.wide ? cp_finish<u128>(j, c) : cp_finish<uint64_t>(j, c);
  mark_end(j, ST_COMPACT);
  if (s != PK_OK) {
    cp_free(j);
    return s;
  }
  j->compacted = true;
  return fill_info(c, info);
}

extern "C" pk_status pk_compaction_get_info(pk_job* j, pk_compaction_info* info) {
  if (!j || !info) return set_error(PK_ERR_INVALID, "null argument");
  if (!j->cp || !j->cp->done || !j->compacted)
    return set_error(PK_ERR_STATE, "no compaction of the current macro-nodes: call pk_compact first");
  return fill_info(*j->cp, info);
}

extern "C" pk_status pk_copy_compacted(pk_job* j, void* keys, uint64_t* entry_offsets, uint32_t* n_prefixes,
                                       pk_compact_entry* entries, int32_t* wires, uint8_t* ext_bases) {
  if (!j) return set_error(PK_ERR_INVALID, "job is null");
  if (!j->cp || !j->cp->done || !j->compacted)
    return set_error(PK_ERR_STATE, "no compaction of the current macro-nodes: call pk_compact first");
  CpState& c = *j->cp;
  PK_TRY(set_device(j->ctx));
  DevBuf* d = c.side[c.cur];
  const uint64_t n = c.n, E = c.E;
  cudaStream_t st = j->stream;
  if (keys && n) PK_CUDA(cudaMemcpyAsync(keys, d[CpState::KEY].p, (c.wide ? 16 : 8) * n, cudaMemcpyDeviceToHost, st));
  if (n_prefixes && n) PK_CUDA(cudaMemcpyAsync(n_prefixes, d[CpState::NPRE].p, 4 * n, cudaMemcpyDeviceToHost, st));
  if (wires && E + n) PK_CUDA(cudaMemcpyAsync(wires, d[CpState::WIRE].p, 12 * (E + n), cudaMemcpyDeviceToHost, st));
  std::vector<uint32_t> eo;
  if (entry_offsets) {
    eo.resize(n + 1);
    PK_CUDA(cudaMemcpyAsync(eo.data(), d[CpState::EOFF].p, 4 * (n + 1), cudaMemcpyDeviceToHost, st));
  }
  if (entries && E) {
    PK_TRY(cp_alloc(j, c.ubuf, sizeof(pk_compact_entry) * E));
    pk::note_launch(), k_cp_entries<<<blocks(E, 256), 256, 0, st>>>((const uint32_t*)d[CpState::XLEN].p,
                                                  (const int32_t*)d[CpState::CNT].p, (const int32_t*)d[CpState::VIS].p,
                                                  (const int2*)d[CpState::BEG].p, (const uint4*)c.epos.p, (uint32_t)E,
                                                  (pk_compact_entry*)c.ubuf.p);
    PK_CUDA(cudaMemcpyAsync(entries, c.ubuf.p, sizeof(pk_compact_entry) * E, cudaMemcpyDeviceToHost, st));
    PK_CUDA(cudaStreamSynchronize(st));
  }
  if (ext_bases && c.ext_bases) {
    PK_TRY(cp_alloc(j, c.ubuf, c.ext_bases));
    pk::note_launch(), k_cp_unpack<<<blocks(E * 32, 256), 256, 0, st>>>((const uint64_t*)c.arena.p, (const uint64_t*)d[CpState::XOFF].p,
                                                      (const uint32_t*)d[CpState::XLEN].p, nullptr,
                                                      (const uint4*)c.epos.p, (uint32_t)E, (uint8_t*)c.ubuf.p);
    PK_CUDA(cudaMemcpyAsync(ext_bases, c.ubuf.p, c.ext_bases, cudaMemcpyDeviceToHost, st));
  }
  PK_CUDA(cudaGetLastError());
  PK_CUDA(cudaStreamSynchronize(st));
  if (entry_offsets)
    for (uint64_t i = 0; i <= n; i++) entry_offsets[i] = eo[i];
  return PK_OK;
}

extern "C" pk_status pk_copy_partial_contigs(pk_job* j, uint64_t* offsets, uint8_t* bases) {
  if (!j) return set_error(PK_ERR_INVALID, "job is null");
  if (!j->cp || !j->cp->done || !j->compacted)
    return set_error(PK_ERR_STATE, "no compaction of the current macro-nodes: call pk_compact first");
  CpState& c = *j->cp;
  PK_TRY(set_device(j->ctx));
  cudaStream_t st = j->stream;
  std::vector<uint4> pos;
  if (offsets) {
    pos.resize(c.C + 1);
    PK_CUDA(cudaMemcpyAsync(pos.data(), c.cpos.p, sizeof(uint4) * (c.C + 1), cudaMemcpyDeviceToHost, st));
  }
  if (bases && c.ct_bases) {
    PK_TRY(cp_alloc(j, c.ubuf, c.ct_bases));
    pk::note_launch(), k_cp_unpack<<<blocks(c.C * 32, 256), 256, 0, st>>>((const uint64_t*)c.arena.p, nullptr, nullptr,
                                                        (const Ct*)c.ct.p, (const uint4*)c.cpos.p, (uint32_t)c.C,
                                                        (uint8_t*)c.ubuf.p);
    PK_CUDA(cudaMemcpyAsync(bases, c.ubuf.p, c.ct_bases, cudaMemcpyDeviceToHost, st));
  }
  PK_CUDA(cudaGetLastError());
  PK_CUDA(cudaStreamSynchronize(st));
  if (offsets)
    for (uint64_t i = 0; i <= c.C; i++) offsets[i] = pos[i].x;
  return PK_OK;
}

extern "C" pk_status pk_walk(pk_job* j, pk_walk_info* info) {
  if (!j) return set_error(PK_ERR_INVALID, "job is null");
  if (!j->cp || !j->cp->done || !j->compacted)
    return set_error(PK_ERR_STATE, "no compaction of the current macro-nodes: call pk_compact first");
  CpState& c = *j->cp;
  PK_TRY(set_device(j->ctx));
  c.wk_done = false;
  mark_begin(j, ST_WALK);
  const pk_status s = c.wide ? cp_walk<u128>(j, c) : cp_walk<uint64_t>(j, c);
  mark_end(j, ST_WALK);
  PK_TRY(s);
  if (info) {
    memset(info, 0, sizeof(*info));
    info->n_begins = c.wk_begins_n;
    info->n_contigs = c.wk_n;
    info->contig_bases = c.wk_bases;
    info->max_depth = c.wk_depth;
  }
  return PK_OK;
}

extern "C" pk_status pk_copy_walk_contigs(pk_job* j, uint64_t* offsets, uint8_t* bases) {
  if (!j) return set_error(PK_ERR_INVALID, "job is null");
  if (!j->cp || !j->cp->wk_done || !j->compacted)
    return set_error(PK_ERR_STATE, "no walk of the current compaction: call pk_walk first");
  CpState& c = *j->cp;
  PK_TRY(set_device(j->ctx));
  cudaStream_t st = j->stream;
  if (offsets) PK_CUDA(cudaMemcpyAsync(offsets, c.wk_off.p, 8 * (c.wk_n + 1), cudaMemcpyDeviceToHost, st));
  if (bases && c.wk_bases) PK_CUDA(cudaMemcpyAsync(bases, c.wk_out.p, c.wk_bases, cudaMemcpyDeviceToHost, st));
  PK_CUDA(cudaStreamSynchronize(st));
  return PK_OK;
}
