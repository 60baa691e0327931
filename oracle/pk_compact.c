/*
 * pk_compact.c -- C restatement of PaKman's iterative compaction and walk, the same
 * algorithm as oracle/pk_compact.py (which is pinned to the reference's own runs),
 * written for speed: the bench's CPU baseline for compaction runs it, and tests pin
 * it to the Python restatement through a hash of the whole result.
 *
 * TEST INFRASTRUCTURE ONLY.  Only the tests and the bench's CPU baseline load it; the
 * GPU product never links or calls it.
 *
 * Restated (file:line in the reference tree):
 *   begin_iterative_compaction   src/iterative_compaction.cpp:131-464
 *   generate_id_set              src/merge_mn.cpp:289-432
 *   iterate_and_pack_mn          src/merge_mn.cpp:433-550
 *   push_to_pred / push_to_succ  src/merge_mn.cpp:1325-1411
 *   MacroNode::setup_wiring      includes/distribute_kmers.h:550-657, with
 *                                libstdc++'s std::sort (introsort) for the ranking
 *   identify_begin_kmers, walk   src/iterative_compaction.cpp:65-93, src/walk.cpp:268-399
 * Extensions are byte strings of base codes (A=0 C=1 T=2 G=3); a node's key is its
 * (k-1)-mer, first base in the top bits.  The start is the wired map with lists in
 * ascending base order (initiate_mnode_wiring, src/wire.cpp:66-121).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

enum { PKC_OK = 0, PKC_EMEM = 1, PKC_EBALANCE = 2, PKC_ETARGET = 3, PKC_EWALK = 4 };

typedef struct {
  uint8_t* b;
  uint32_t n;
  int32_t cnt, vis;
  uint8_t term;
  u128 nbr;
} entry_t;

typedef struct {
  entry_t* v;
  int n, cap;
} elist_t;

typedef struct {
  u128 key;
  elist_t pre, suf;
  int32_t* w; /* 3 per slot, np + ns + 1 slots */
  int nw;
  int32_t* beg; /* 2 per prefix */
} node_t;

typedef struct {
  uint64_t rounds, n_nodes, n_contigs, walk_contigs, walk_bases, contig_bases;
  uint64_t hash; /* FNV-1a over the map, the partial contigs and the walk contigs */
} pkc_result;

static int L_;

static u128 str_key(const uint8_t* s, int n) {
  u128 v = 0;
  for (int i = 0; i < n; i++) v = (v << 2) | s[i];
  return v;
}

static void key_bases(u128 key, int n, uint8_t* out) {
  for (int i = 0; i < n; i++) out[i] = (uint8_t)((key >> (2 * (n - 1 - i))) & 3);
}

static uint8_t* dup_bytes(const uint8_t* s, uint32_t n) {
  uint8_t* p = (uint8_t*)malloc(n ? n : 1);
  if (p && n) memcpy(p, s, n);
  return p;
}

static int push_entry(elist_t* l, entry_t e) {
  if (l->n == l->cap) {
    int cap = l->cap ? 2 * l->cap : 4;
    entry_t* v = (entry_t*)realloc(l->v, sizeof(entry_t) * cap);
    if (!v) return PKC_EMEM;
    l->v = v;
    l->cap = cap;
  }
  l->v[l->n++] = e;
  return PKC_OK;
}

static void free_node(node_t* nd) {
  for (int i = 0; i < nd->pre.n; i++) free(nd->pre.v[i].b);
  for (int i = 0; i < nd->suf.n; i++) free(nd->suf.v[i].b);
  free(nd->pre.v);
  free(nd->suf.v);
  free(nd->w);
  free(nd->beg);
}

/* neighbour keys: first L of ext + key (prefix), last L of key + ext (suffix) */
static u128 pred_nbr(const uint8_t* e, uint32_t n, u128 key) {
  if (!n) return 0;
  if ((int)n >= L_) return str_key(e, L_);
  return (str_key(e, (int)n) << (2 * (L_ - (int)n))) | (key >> (2 * n));
}

static u128 succ_nbr(const uint8_t* e, uint32_t n, u128 key) {
  if (!n) return 0;
  if ((int)n >= L_) return str_key(e + n - L_, L_);
  const u128 mask = (((u128)1) << (2 * L_)) - 1;
  return ((key << (2 * n)) | str_key(e, (int)n)) & mask;
}

/* ---- std::sort (libstdc++ introsort) on int indices ranked by (visit, count) desc */
typedef struct {
  const entry_t* v;
} rank_t;

static int rless(const rank_t* r, int i, int j) {
  return r->v[i].vis > r->v[j].vis || (r->v[i].vis == r->v[j].vis && r->v[i].cnt > r->v[j].cnt);
}

static void heap_adjust(int* a, int hole, int len, int value, const rank_t* r) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (rless(r, a[child], a[child - 1])) child--;
    a[hole] = a[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    a[hole] = a[child - 1];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top && rless(r, a[parent], value)) {
    a[hole] = a[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  a[hole] = value;
}

static void heap_sort(int* a, int len, const rank_t* r) {
  if (len >= 2)
    for (int parent = (len - 2) / 2;; parent--) {
      heap_adjust(a, parent, len, a[parent], r);
      if (parent == 0) break;
    }
  for (int last = len; last > 1;) {
    last--;
    const int v = a[last];
    a[last] = a[0];
    heap_adjust(a, 0, last, v, r);
  }
}

static void swp(int* a, int i, int j) {
  int t = a[i];
  a[i] = a[j];
  a[j] = t;
}

static void introsort(int* a, int first, int last, int depth, const rank_t* r) {
  while (last - first > 16) {
    if (depth == 0) {
      heap_sort(a + first, last - first, r);
      return;
    }
    depth--;
    const int mid = first + (last - first) / 2, x = first + 1, y = mid, z = last - 1;
    if (rless(r, a[x], a[y])) {
      if (rless(r, a[y], a[z])) swp(a, first, y);
      else if (rless(r, a[x], a[z])) swp(a, first, z);
      else swp(a, first, x);
    } else if (rless(r, a[x], a[z])) {
      swp(a, first, x);
    } else if (rless(r, a[y], a[z])) {
      swp(a, first, z);
    } else {
      swp(a, first, y);
    }
    int lo = first + 1, hi = last;
    for (;;) {
      while (rless(r, a[lo], a[first])) lo++;
      hi--;
      while (rless(r, a[first], a[hi])) hi--;
      if (!(lo < hi)) break;
      swp(a, lo, hi);
      lo++;
    }
    introsort(a, lo, last, depth, r);
    last = lo;
  }
}

static void std_sort(int* a, int n, const rank_t* r) {
  if (n < 2) return;
  int lg = 0;
  while ((1 << (lg + 1)) <= n) lg++;
  introsort(a, 0, n, 2 * lg, r);
  const int lim = n > 16 ? 16 : n;
  for (int i = 1; i < lim; i++) {
    const int v = a[i];
    if (rless(r, v, a[0])) {
      memmove(a + 1, a, sizeof(int) * i);
      a[0] = v;
    } else {
      int j = i - 1;
      while (rless(r, v, a[j])) {
        a[j + 1] = a[j];
        j--;
      }
      a[j + 1] = v;
    }
  }
  for (int i = 16; i < n; i++) {
    const int v = a[i];
    int j = i - 1;
    while (rless(r, v, a[j])) {
      a[j + 1] = a[j];
      j--;
    }
    a[j + 1] = v;
  }
}

/* The ranking alone, for pinning against libstdc++: out = indices 0..n-1 sorted by
   (visit, count) descending the way std::sort leaves them. */
int pko_rank_std_sort(const int32_t* vis, const int32_t* cnt, int n, int* out) {
  entry_t* e = (entry_t*)calloc(n ? n : 1, sizeof(entry_t));
  if (!e) return PKC_EMEM;
  for (int i = 0; i < n; i++) {
    e[i].vis = vis[i];
    e[i].cnt = cnt[i];
    out[i] = i;
  }
  rank_t r = {e};
  std_sort(out, n, &r);
  free(e);
  return PKC_OK;
}

/* MacroNode::setup_wiring after wiring_info / prefix_begin_info were cleared */
static int setup_wiring(node_t* nd) {
  const int np = nd->pre.n, ns = nd->suf.n, nw = np + ns + 1;
  entry_t *pre = nd->pre.v, *suf = nd->suf.v;
  free(nd->w);
  free(nd->beg);
  nd->w = (int32_t*)calloc(3 * nw, sizeof(int32_t));
  nd->beg = (int32_t*)calloc(2 * (np ? np : 1), sizeof(int32_t));
  if (!nd->w || !nd->beg) return PKC_EMEM;
  nd->nw = nw;
  int pc = 0, sc = 0, ns_id = -1, np_id = -1;
  for (int i = 0; i < ns; i++)
    if (suf[i].n) sc += suf[i].vis;
  for (int i = 0; i < np; i++)
    if (pre[i].n) pc += pre[i].vis;
  for (int i = 0; i < ns; i++)
    if (!suf[i].n) {
      ns_id = i;
      if (suf[i].cnt == -1) {
        suf[i].cnt = 1;
        suf[i].vis = pc - sc > 0 ? pc - sc : 0;
      }
    }
  for (int i = 0; i < np; i++)
    if (!pre[i].n) {
      np_id = i;
      if (pre[i].cnt == -1) {
        pre[i].cnt = 1;
        pre[i].vis = sc - pc > 0 ? sc - pc : 0;
      }
    }
  if (ns_id < 0 || np_id < 0 || sc + suf[ns_id].vis != pc + pre[np_id].vis) return PKC_EBALANCE;
  int* ip = (int*)malloc(sizeof(int) * (np + ns + 2));
  int* is = ip + np + 1;
  int* offs = (int*)calloc(ns + 1, sizeof(int));
  if (!ip || !offs) return PKC_EMEM;
  for (int i = 0; i < np; i++) ip[i] = i;
  for (int i = 0; i < ns; i++) is[i] = i;
  rank_t rp = {pre}, rs = {suf};
  std_sort(ip, np, &rp);
  std_sort(is, ns, &rs);
  int leftover = sc + suf[ns_id].vis;
  int top_p = 0, top_s = 0, var_p = 0, var_s = 0, wi = 0, p_size = 0, last_pid = -1, begin_pos = -1;
  int st = PKC_OK;
  while (leftover > 0) {
    if (top_p >= np || top_s >= ns || wi >= nw) {
      st = PKC_EBALANCE;
      break;
    }
    const int sid = is[top_s], pid = ip[top_p];
    const int a = pre[pid].vis - var_p, b = suf[sid].vis - var_s, c = a < b ? a : b;
    nd->w[3 * wi] = sid;
    nd->w[3 * wi + 1] = offs[sid];
    nd->w[3 * wi + 2] = c;
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
    if (var_p == pre[pid].vis) {
      var_p = 0;
      top_p++;
      nd->beg[2 * pid] = begin_pos;
      nd->beg[2 * pid + 1] = p_size;
      p_size = 0;
    }
    if (var_s == suf[sid].vis) {
      var_s = 0;
      top_s++;
    }
  }
  free(ip);
  free(offs);
  return st;
}

/* ---- one round's transfers (TransferNode, src/merge_mn.cpp:483-525) ------------ */
typedef struct {
  u128 target;
  const uint8_t* w; /* W = P + K + S (owned by the round) */
  uint32_t pl, sl;
  int32_t c0, c1;
  uint8_t term, to_pred;
} xfer_t;

typedef struct {
  xfer_t* v;
  size_t n, cap;
} xlist_t;

typedef struct {
  uint8_t** v;
  uint32_t* len;
  size_t n, cap;
} slist_t;

static int slist_push(slist_t* s, uint8_t* p, uint32_t n) {
  if (s->n == s->cap) {
    size_t cap = s->cap ? 2 * s->cap : 64;
    uint8_t** v = (uint8_t**)realloc(s->v, sizeof(uint8_t*) * cap);
    uint32_t* l = (uint32_t*)realloc(s->len, sizeof(uint32_t) * cap);
    if (!v || !l) return PKC_EMEM;
    s->v = v;
    s->len = l;
    s->cap = cap;
  }
  s->v[s->n] = p;
  s->len[s->n++] = n;
  return PKC_OK;
}

static int xlist_push(xlist_t* x, xfer_t t) {
  if (x->n == x->cap) {
    size_t cap = x->cap ? 2 * x->cap : 1024;
    xfer_t* v = (xfer_t*)realloc(x->v, sizeof(xfer_t) * cap);
    if (!v) return PKC_EMEM;
    x->v = v;
    x->cap = cap;
  }
  x->v[x->n++] = t;
  return PKC_OK;
}

static long find_node(const node_t* nodes, size_t n, u128 key) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    if (nodes[mid].key < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && nodes[lo].key == key) ? (long)lo : -1;
}

static int push_transfer(node_t* nd, const xfer_t* t) {
  elist_t* l = t->to_pred ? &nd->suf : &nd->pre;
  const uint8_t* se = t->to_pred ? t->w + L_ : t->w + t->pl;
  const uint32_t sl = t->to_pred ? t->pl : t->sl;
  const uint8_t* ne = t->to_pred ? t->w + L_ : t->w;
  const uint32_t nl = t->pl + t->sl;
  int hit = -1;
  for (int j = 0; j < l->n; j++)
    if (l->v[j].n == sl && memcmp(l->v[j].b, se, sl) == 0) {
      hit = j;
      break;
    }
  entry_t e;
  e.b = dup_bytes(ne, nl);
  if (!e.b) return PKC_EMEM;
  e.n = nl;
  e.cnt = t->c0;
  e.vis = t->c1;
  e.term = t->term;
  e.nbr = t->term ? 0 : (t->to_pred ? succ_nbr(e.b, nl, nd->key) : pred_nbr(e.b, nl, nd->key));
  if (hit < 0 || l->v[hit].term) return push_entry(l, e);
  free(l->v[hit].b);
  l->v[hit] = e;
  return PKC_OK;
}

/* ---- hashing (FNV-1a 64) -------------------------------------------------------- */
static void fnv(uint64_t* h, const void* p, size_t n) {
  const uint8_t* b = (const uint8_t*)p;
  for (size_t i = 0; i < n; i++) {
    *h ^= b[i];
    *h *= 1099511628211ull;
  }
}

static void hash_u32(uint64_t* h, uint32_t v) { fnv(h, &v, 4); }
static void hash_i32(uint64_t* h, int32_t v) { fnv(h, &v, 4); }

static void hash_list(uint64_t* h, const elist_t* l) {
  hash_u32(h, (uint32_t)l->n);
  for (int i = 0; i < l->n; i++) {
    hash_u32(h, l->v[i].n);
    fnv(h, l->v[i].b, l->v[i].n);
    hash_i32(h, l->v[i].cnt);
    hash_i32(h, l->v[i].vis);
    fnv(h, &l->v[i].term, 1);
  }
}

/* ---- walk (iterative depth-first, src/walk.cpp:268-399) ------------------------- */
typedef struct {
  long node;
  int p, oip, wi, off, rem, share;
  uint32_t lenb;
} wframe_t;

static int walk_all(node_t* nodes, size_t n, uint64_t* h, uint64_t* ncontigs, uint64_t* nbases) {
  size_t cap = 1024, bcap = 4096;
  wframe_t* st = (wframe_t*)malloc(sizeof(wframe_t) * cap);
  uint8_t* buf = (uint8_t*)malloc(bcap);
  if (!st || !buf) return PKC_EMEM;
  int status = PKC_OK;
  for (size_t bi = 0; bi < n && status == PKC_OK; bi++)
    for (int bp = 0; bp < nodes[bi].pre.n && status == PKC_OK; bp++) {
      const entry_t* be = &nodes[bi].pre.v[bp];
      if (!(be->vis > 0 && be->term)) continue;
      uint32_t len = be->n + (uint32_t)L_;
      if (len > bcap) {
        bcap = 2 * len;
        buf = (uint8_t*)realloc(buf, bcap);
        if (!buf) return PKC_EMEM;
      }
      memcpy(buf, be->b, be->n);
      key_bases(nodes[bi].key, L_, buf + be->n);
      size_t d = 0;
      st[0] = (wframe_t){(long)bi, bp, 0, 0, 0, be->vis, -1, len};
      for (;;) {
        wframe_t* f = &st[d];
        node_t* cur = &nodes[f->node];
        const int bpos = cur->beg[2 * f->p], num = cur->beg[2 * f->p + 1];
        if (f->share >= 0) {
          f->rem -= f->share;
          f->share = -1;
          len = f->lenb;
          f->off += cur->w[3 * (bpos + f->wi) + 2];
          f->wi++;
          continue;
        }
        if (f->wi >= num) {
          if (d == 0) break;
          d--;
          continue;
        }
        const int32_t* w = &cur->w[3 * (bpos + f->wi)];
        const int sid = w[0], ois = w[1], sz = w[2];
        if (f->off + sz <= f->oip || f->off > f->oip + f->rem) {
          f->off += sz;
          f->wi++;
          continue;
        }
        const int oiw = f->oip <= f->off ? 0 : f->oip - f->off;
        const int next_off = ois + oiw;
        const int share = f->rem < sz - oiw ? f->rem : sz - oiw;
        const entry_t* S = &cur->suf.v[sid];
        f->lenb = len;
        if (len + S->n > bcap) {
          bcap = 2 * (len + S->n);
          buf = (uint8_t*)realloc(buf, bcap);
          if (!buf) return PKC_EMEM;
        }
        memcpy(buf + len, S->b, S->n);
        len += S->n;
        if (S->term) {
          hash_u32(h, len);
          fnv(h, buf, len);
          (*ncontigs)++;
          *nbases += len;
          f->rem -= share;
          len = f->lenb;
          f->off += sz;
          f->wi++;
          continue;
        }
        const long nx = find_node(nodes, n, S->nbr);
        if (nx < 0) {
          status = PKC_ETARGET;
          break;
        }
        /* the successor's first prefix equal to the first |S| bases of key + S */
        const uint8_t* srch = buf + f->lenb - L_;
        int q = -1;
        for (int j = 0; j < nodes[nx].pre.n; j++)
          if (nodes[nx].pre.v[j].n == S->n && memcmp(nodes[nx].pre.v[j].b, srch, S->n) == 0) {
            q = j;
            break;
          }
        if (q < 0 || share <= 0 || len >= 500000) {
          status = PKC_EWALK;
          break;
        }
        f->share = share;
        if (d + 1 == cap) {
          cap *= 2;
          st = (wframe_t*)realloc(st, sizeof(wframe_t) * cap);
          if (!st) return PKC_EMEM;
        }
        d++;
        st[d] = (wframe_t){nx, q, next_off, 0, 0, share, -1, len};
      }
    }
  free(st);
  free(buf);
  return status;
}

/*
 * Compaction from the macro-node table (keys: 2 x uint64 per node, lo then hi;
 * suf / pre: 4 counts per node by extension base) down to `threshold` nodes, then the
 * walk.  out->hash covers, in order: every node (key lo, hi; suffixes then prefixes as
 * n, then per entry len, bases, count, visit, terminal; wire slots; begin slots), the
 * partial contigs (count, then len + bases each) and the walk contigs (count, then
 * len + bases each).  max_rounds < 0: no limit.
 */
int pko_compact_walk(const uint64_t* keys, const uint32_t* suf, const uint32_t* pre, size_t m, int k,
                     int coverage, uint64_t threshold, pkc_result* out) {
  L_ = k - 1;
  memset(out, 0, sizeof(*out));
  node_t* nodes = (node_t*)calloc(m ? m : 1, sizeof(node_t));
  if (!nodes) return PKC_EMEM;
  int st = PKC_OK;
  for (size_t i = 0; i < m && st == PKC_OK; i++) {
    node_t* nd = &nodes[i];
    nd->key = ((u128)keys[2 * i + 1] << 64) | keys[2 * i];
    for (int side = 0; side < 2; side++) {
      const uint32_t* c = side ? &suf[4 * i] : &pre[4 * i];
      elist_t* l = side ? &nd->suf : &nd->pre;
      for (int b = 0; b < 4 && st == PKC_OK; b++)
        if (c[b]) {
          entry_t e;
          uint8_t base = (uint8_t)b;
          e.b = dup_bytes(&base, 1);
          e.n = 1;
          e.cnt = (int32_t)c[b];
          e.vis = (int32_t)((c[b] + (uint32_t)coverage - 1) / (uint32_t)coverage);
          e.term = 0;
          e.nbr = side ? succ_nbr(e.b, 1, nd->key) : pred_nbr(e.b, 1, nd->key);
          st = push_entry(l, e);
        }
      entry_t t = {dup_bytes(NULL, 0), 0, -1, -1, 1, 0};
      if (st == PKC_OK) st = push_entry(l, t);
    }
    if (st == PKC_OK) st = setup_wiring(nd);
  }
  size_t n = m;
  slist_t contigs = {0};
  xlist_t xs = {0};
  slist_t wbufs = {0};
  uint8_t kb[64];
  uint8_t* is_id = (uint8_t*)malloc(m ? m : 1);
  uint8_t* touched = (uint8_t*)malloc(m ? m : 1);
  if (!is_id || !touched) st = PKC_EMEM;
  while (st == PKC_OK && n > threshold) {
    out->rounds++;
    for (size_t i = 0; i < n; i++) {
      const node_t* nd = &nodes[i];
      int id = 1;
      for (int j = 0; j < nd->pre.n && id; j++)
        if (!nd->pre.v[j].term && nd->pre.v[j].nbr > nd->key) id = 0;
      for (int j = 0; j < nd->suf.n && id; j++)
        if (!nd->suf.v[j].term && nd->suf.v[j].nbr > nd->key) id = 0;
      is_id[i] = (uint8_t)id;
    }
    xs.n = 0;
    for (size_t i = 0; i < n && st == PKC_OK; i++) {
      if (!is_id[i]) continue;
      node_t* nd = &nodes[i];
      key_bases(nd->key, L_, kb);
      for (int p = 0; p < nd->pre.n && st == PKC_OK; p++) {
        const int bpos = nd->beg[2 * p], num = nd->beg[2 * p + 1];
        const entry_t* P = &nd->pre.v[p];
        const int self_p = !P->term && P->nbr == nd->key;
        for (int t = 0; t < num && st == PKC_OK; t++) {
          const int32_t* w = &nd->w[3 * (bpos + t)];
          const entry_t* S = &nd->suf.v[w[0]];
          const int self_s = !S->term && S->nbr == nd->key;
          const int ep = !P->term && !self_p, es = !S->term && !self_s;
          const int contig = P->term && S->term;
          if (!contig && !ep && !es) continue;
          const uint32_t wl = P->n + (uint32_t)L_ + S->n;
          uint8_t* W = (uint8_t*)malloc(wl);
          if (!W) {
            st = PKC_EMEM;
            break;
          }
          memcpy(W, P->b, P->n);
          memcpy(W + P->n, kb, L_);
          memcpy(W + P->n + L_, S->b, S->n);
          if (contig) {
            st = slist_push(&contigs, W, wl);
            continue;
          }
          st = slist_push(&wbufs, W, wl);
          const int32_t c0 = P->cnt < S->cnt ? P->cnt : S->cnt;
          if (st == PKC_OK && ep)
            st = xlist_push(&xs, (xfer_t){P->nbr, W, P->n, S->n, c0, w[2], (uint8_t)(S->term || self_s), 1});
          if (st == PKC_OK && es)
            st = xlist_push(&xs, (xfer_t){S->nbr, W, P->n, S->n, c0, w[2], (uint8_t)(P->term || self_p), 0});
        }
      }
    }
    size_t n2 = 0;
    for (size_t i = 0; i < n; i++) {
      if (is_id[i]) free_node(&nodes[i]);
      else nodes[n2++] = nodes[i];
    }
    n = n2;
    memset(touched, 0, n);
    for (size_t t = 0; t < xs.n && st == PKC_OK; t++) {
      const long j = find_node(nodes, n, xs.v[t].target);
      if (j < 0) {
        st = PKC_ETARGET;
        break;
      }
      st = push_transfer(&nodes[j], &xs.v[t]);
      touched[j] = 1;
    }
    for (size_t i = 0; i < n && st == PKC_OK; i++)
      if (touched[i]) st = setup_wiring(&nodes[i]);
    for (size_t i = 0; i < wbufs.n; i++) free(wbufs.v[i]);
    wbufs.n = 0;
  }
  uint64_t h = 1469598103934665603ull;
  if (st == PKC_OK) {
    for (size_t i = 0; i < n; i++) {
      const node_t* nd = &nodes[i];
      const uint64_t lo = (uint64_t)nd->key, hi = (uint64_t)(nd->key >> 64);
      fnv(&h, &lo, 8);
      fnv(&h, &hi, 8);
      hash_list(&h, &nd->suf);
      hash_list(&h, &nd->pre);
      hash_u32(&h, (uint32_t)nd->nw);
      fnv(&h, nd->w, 12 * (size_t)nd->nw);
      hash_u32(&h, (uint32_t)nd->pre.n);
      fnv(&h, nd->beg, 8 * (size_t)nd->pre.n);
    }
    const uint64_t nc = contigs.n;
    fnv(&h, &nc, 8);
    for (size_t c = 0; c < contigs.n; c++) {
      hash_u32(&h, contigs.len[c]);
      fnv(&h, contigs.v[c], contigs.len[c]);
      out->contig_bases += contigs.len[c];
    }
    out->n_nodes = n;
    out->n_contigs = contigs.n;
    /* the walk's contigs are hashed after their count, which is only known at the
       end: hash them into a separate stream and fold it in */
    uint64_t hw = 1469598103934665603ull;
    st = walk_all(nodes, n, &hw, &out->walk_contigs, &out->walk_bases);
    fnv(&h, &out->walk_contigs, 8);
    fnv(&h, &hw, 8);
    out->hash = h;
  }
  for (size_t i = 0; i < n; i++) free_node(&nodes[i]);
  free(nodes);
  for (size_t c = 0; c < contigs.n; c++) free(contigs.v[c]);
  free(contigs.v);
  free(contigs.len);
  for (size_t i = 0; i < wbufs.n; i++) free(wbufs.v[i]);
  free(wbufs.v);
  free(wbufs.len);
  free(xs.v);
  free(is_id);
  free(touched);
  return st;
}
