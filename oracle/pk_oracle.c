/*
 * pk_oracle.c -- CPU restatement of PaKman's k-mer counting, frequency-histogram
 * cutoff and macro-node construction, used as the CHECKER for the GPU path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only the tests, the smoke check and the bench's CPU
 * baseline load this library; the GPU product never links or calls it.  It is
 * pinned against the reference's own binaries (built from the reference sources by
 * oracle/ref/Makefile) on the committed fixtures under tests/golden/.
 *
 * Semantics restated (file:line refer to the reference tree):
 *  - record layout: the buffer is scanned from its first '>'; every record is a
 *    header line starting with '>' followed by exactly one sequence line
 *    (src/kmer_counting.cpp:2920-2935, 3144).  A record start that is not '>' is
 *    an assertion failure in the reference; here it returns PKO_EFORMAT.  Once a
 *    sequence line would start with fewer than k bytes left in the buffer, the
 *    reference stops (src/kmer_counting.cpp:2935) -- no later record is checked.
 *  - base codes: code(c) = (c >> 1) & 7 (char_to_el, includes/distribute_kmers.h:
 *    784-786): A=0 C=1 T=2 G=3, lowercase alike, 'N' = 7.  The window is rolled as
 *    kmer = ((kmer << 2) | code) & KMER_MASK (kmer_shift, :798-805), so an 'N' ORs
 *    into the previous base's low bit and windows spanning 'N' are still counted.
 *    No reverse complement is taken anywhere.
 *  - every window of k bytes inside one sequence line is one k-mer instance
 *    (src/kmer_counting.cpp:2967-3017).  The table is sorted ascending by k-mer
 *    and unique, with the number of instances as its count (transfer_kmers +
 *    SortAndAggregate, src/kmer_counting.cpp:254-352, 169-250).
 *  - drop_n (an extension used for the long-k workload): windows containing
 *    'N' or 'n' are skipped.  It equals running the reference on the same reads
 *    split into separate records at every 'N'.
 *  - histogram: hist[c] = #entries with count c, for c < t; cutoff = position of
 *    the first minimum of hist[1..t) (std::min_element, src/kmer_histogram.cpp:
 *    84-115); t == 1 gives cutoff 1.  Entries with count >= cutoff are kept
 *    (src/kmer_histogram.cpp:140).  No kept entry -> PKO_EEMPTY (the reference
 *    calls MPI_Abort, src/kmer_histogram.cpp:189-200).
 *  - macro-nodes: node set = sorted unique {x >> 2, x & SUCC_MASK} over kept x
 *    (src/mn_construct.cpp:225-285; the "^1" at :234 is shifted out).  Node P gets
 *    a suffix entry (ext = last base of x, count) for each kept x with x >> 2 == P
 *    (:346-391); node S gets a prefix entry (ext = first base of x, count) for each
 *    kept x with x & SUCC_MASK == S (:407-457).  Suffixes come out in ascending ext
 *    order in the reference; prefix order is unspecified there (unstable sort by
 *    suffix only, :303) and is ascending ext here.  Output per node: key and four
 *    u32 counts per side indexed by ext, 0 meaning absent.
 *  - visit value (:75-79) = ceil(count / coverage), exact in integers.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

typedef struct {
  uint64_t lo, hi;
} pko_key;

enum { PKO_OK = 0, PKO_EFORMAT = -1, PKO_EARG = -2, PKO_ENOMEM = -3, PKO_EEMPTY = -4 };

static inline u128 key_mask(int bits) {
  return bits >= 128 ? ~(u128)0 : (((u128)1 << bits) - 1);
}

/* ---------------------------------------------------------------- sorting ---- */
/* Stable LSD radix sort of (key, aux) records on the low `bits` bits of key. */
typedef struct {
  u128 key;
  uint32_t aux;
} rec_t;

static int radix_sort_recs(rec_t* a, size_t n, int bits) {
  if (n < 2 || bits <= 0) return PKO_OK;
  rec_t* b = (rec_t*)malloc(n * sizeof(rec_t));
  if (!b) return PKO_ENOMEM;
  size_t* cnt = (size_t*)malloc(65536 * sizeof(size_t));
  if (!cnt) { free(b); return PKO_ENOMEM; }
  rec_t *src = a, *dst = b;
  for (int sh = 0; sh < bits; sh += 16) {
    memset(cnt, 0, 65536 * sizeof(size_t));
    for (size_t i = 0; i < n; i++) cnt[(unsigned)(src[i].key >> sh) & 0xffff]++;
    size_t s = 0;
    for (int d = 0; d < 65536; d++) { size_t c = cnt[d]; cnt[d] = s; s += c; }
    for (size_t i = 0; i < n; i++) dst[cnt[(unsigned)(src[i].key >> sh) & 0xffff]++] = src[i];
    rec_t* t = src; src = dst; dst = t;
  }
  if (src != a) memcpy(a, src, n * sizeof(rec_t));
  free(b);
  free(cnt);
  return PKO_OK;
}

static int radix_sort_u64(uint64_t* a, size_t n, int bits) {
  if (n < 2 || bits <= 0) return PKO_OK;
  uint64_t* b = (uint64_t*)malloc(n * sizeof(uint64_t));
  size_t* cnt = (size_t*)malloc(65536 * sizeof(size_t));
  if (!b || !cnt) { free(b); free(cnt); return PKO_ENOMEM; }
  uint64_t *src = a, *dst = b;
  for (int sh = 0; sh < bits; sh += 16) {
    memset(cnt, 0, 65536 * sizeof(size_t));
    for (size_t i = 0; i < n; i++) cnt[(src[i] >> sh) & 0xffff]++;
    size_t s = 0;
    for (int d = 0; d < 65536; d++) { size_t c = cnt[d]; cnt[d] = s; s += c; }
    for (size_t i = 0; i < n; i++) dst[cnt[(src[i] >> sh) & 0xffff]++] = src[i];
    uint64_t* t = src; src = dst; dst = t;
  }
  if (src != a) memcpy(a, src, n * sizeof(uint64_t));
  free(b);
  free(cnt);
  return PKO_OK;
}

/* ------------------------------------------------------------ extraction ---- */
/*
 * Walk the records exactly as the reference's sliding window does and hand every
 * k-mer instance to `emit`.  Returns PKO_OK or PKO_EFORMAT.
 */
typedef void (*emit_fn)(void* ctx, u128 kmer);

static int walk_kmers(const uint8_t* buf, size_t n, int k, int drop_n, emit_fn emit, void* ctx,
                      size_t* n_reads) {
  const u128 mask = key_mask(2 * k);
  size_t p = 0, reads = 0;
  while (p < n && buf[p] != '>') p++;
  for (size_t i = p; i < n; i++) reads += (buf[i] == '>');
  if (n_reads) *n_reads = reads;
  while (p < n) {
    if (buf[p] != '>') return PKO_EFORMAT;
    while (p < n && buf[p] != '\n') p++; /* skip the header line */
    p++;
    if (p + (size_t)k > n) break;
    u128 kmer = 0;
    int run = 0; /* bases since the last dropped 'N' (drop_n only) */
    for (int i = 0; i < k - 1 && buf[p] != '\n'; i++, p++) {
      uint8_t c = buf[p];
      kmer = ((kmer << 2) | (u128)((c >> 1) & 7)) & mask;
      run = (drop_n && (c == 'N' || c == 'n')) ? 0 : run + 1;
    }
    while (p < n && buf[p] != '\n') {
      uint8_t c = buf[p++];
      kmer = ((kmer << 2) | (u128)((c >> 1) & 7)) & mask;
      run = (drop_n && (c == 'N' || c == 'n')) ? 0 : run + 1;
      if (!drop_n || run >= k) emit(ctx, kmer);
    }
    p++; /* skip the newline */
  }
  return PKO_OK;
}

typedef struct {
  uint64_t* k64;
  rec_t* k128;
  size_t n, cap;
  int wide;
  int oom;
} collect_t;

static void collect_emit(void* c_, u128 kmer) {
  collect_t* c = (collect_t*)c_;
  if (c->oom) return;
  if (c->n == c->cap) {
    size_t nc = c->cap ? 2 * c->cap : (1u << 20);
    void* p = c->wide ? realloc(c->k128, nc * sizeof(rec_t)) : realloc(c->k64, nc * sizeof(uint64_t));
    if (!p) { c->oom = 1; return; }
    if (c->wide) c->k128 = (rec_t*)p; else c->k64 = (uint64_t*)p;
    c->cap = nc;
  }
  if (c->wide) { c->k128[c->n].key = kmer; c->k128[c->n].aux = 0; }
  else c->k64[c->n] = (uint64_t)kmer;
  c->n++;
}

static void count_emit(void* c_, u128 kmer) {
  (void)kmer;
  (*(size_t*)c_)++;
}

/* Number of k-mer instances (windows) without building the table. */
int pko_count_windows(const uint8_t* buf, size_t n, int k, int drop_n, size_t* n_windows,
                      size_t* n_reads) {
  if (k < 2 || k > 64) return PKO_EARG;
  size_t w = 0;
  int rc = walk_kmers(buf, n, k, drop_n, count_emit, &w, n_reads);
  *n_windows = w;
  return rc;
}

/*
 * Build the sorted unique (k-mer, count) table.  keys/counts are malloc'd here and
 * released with pko_free.
 */
int pko_count(const uint8_t* buf, size_t n, int k, int drop_n, pko_key** keys_out,
              uint32_t** counts_out, size_t* n_unique, size_t* n_windows, size_t* n_reads) {
  if (k < 2 || k > 64) return PKO_EARG;
  collect_t c;
  memset(&c, 0, sizeof(c));
  c.wide = k > 32;
  int rc = walk_kmers(buf, n, k, drop_n, collect_emit, &c, n_reads);
  if (c.oom) rc = PKO_ENOMEM;
  if (rc != PKO_OK) { free(c.k64); free(c.k128); return rc; }
  *n_windows = c.n;
  if (c.wide) rc = radix_sort_recs(c.k128, c.n, 2 * k);
  else rc = radix_sort_u64(c.k64, c.n, 2 * k);
  if (rc != PKO_OK) { free(c.k64); free(c.k128); return rc; }
  /* run-length aggregation (SortAndAggregate_InPlace, src/kmer_counting.cpp:169-190) */
  size_t u = 0;
  pko_key* keys = (pko_key*)malloc((c.n ? c.n : 1) * sizeof(pko_key));
  uint32_t* cnts = (uint32_t*)malloc((c.n ? c.n : 1) * sizeof(uint32_t));
  if (!keys || !cnts) { free(keys); free(cnts); free(c.k64); free(c.k128); return PKO_ENOMEM; }
  for (size_t i = 0; i < c.n;) {
    u128 key = c.wide ? c.k128[i].key : (u128)c.k64[i];
    size_t j = i + 1;
    while (j < c.n && (c.wide ? c.k128[j].key : (u128)c.k64[j]) == key) j++;
    keys[u].lo = (uint64_t)key;
    keys[u].hi = (uint64_t)(key >> 64);
    cnts[u] = (uint32_t)(j - i);
    u++;
    i = j;
  }
  free(c.k64);
  free(c.k128);
  *keys_out = keys;
  *counts_out = cnts;
  *n_unique = u;
  return PKO_OK;
}

/*
 * Multi-threaded counting with the reference's distributed structure on threads
 * instead of MPI ranks: each thread walks a contiguous run of whole records
 * (DivideReads, src/input_reading.cpp:69-243), its k-mers are routed to an owner
 * by key range (the exchange of transfer_kmers, src/kmer_counting.cpp:254-352),
 * and each owner sorts and run-length aggregates what it received
 * (SortAndAggregate, :169-250).  Owners hold disjoint, ordered key ranges, so their
 * tables concatenate into the same sorted unique table as pko_count.  Valid input
 * only: record boundaries are found by "\n>"; a malformed record is reported by
 * the serial pko_count.
 */
typedef struct {
  const uint8_t* buf;
  size_t begin, end;
  int k, drop_n, wide, pbits, nparts;
  collect_t c;
  size_t reads;
  size_t* part_n;    /* [nparts] keys per owner range */
  void* routed;      /* keys grouped by owner range */
  size_t* part_off;  /* [nparts + 1] */
  int rc;
} mt_walker;

typedef struct {
  mt_walker* w;
  int nthreads, nparts, wide;
  int next_part; /* shared work counter */
  pthread_mutex_t mu;
  pko_key** out_keys;   /* [nparts] */
  uint32_t** out_cnts;  /* [nparts] */
  size_t* out_u;        /* [nparts] */
  size_t* out_n;        /* [nparts] */
  int rc;
} mt_job;

static inline int part_of(u128 key, int k, int pbits) {
  return (int)(key >> (2 * k - pbits));
}

static void* mt_walk(void* arg) {
  mt_walker* w = (mt_walker*)arg;
  memset(&w->c, 0, sizeof(w->c));
  w->c.wide = w->wide;
  w->rc = walk_kmers(w->buf + w->begin, w->end - w->begin, w->k, w->drop_n, collect_emit, &w->c,
                     &w->reads);
  if (w->c.oom) w->rc = PKO_ENOMEM;
  if (w->rc != PKO_OK) return NULL;
  /* route to owner ranges (counting pass, then a stable scatter) */
  w->part_n = (size_t*)calloc((size_t)w->nparts, sizeof(size_t));
  w->part_off = (size_t*)calloc((size_t)w->nparts + 1, sizeof(size_t));
  const size_t esz = w->wide ? sizeof(rec_t) : sizeof(uint64_t);
  w->routed = malloc((w->c.n ? w->c.n : 1) * esz);
  if (!w->part_n || !w->part_off || !w->routed) { w->rc = PKO_ENOMEM; return NULL; }
  for (size_t i = 0; i < w->c.n; i++) {
    u128 key = w->wide ? w->c.k128[i].key : (u128)w->c.k64[i];
    w->part_n[part_of(key, w->k, w->pbits)]++;
  }
  size_t acc = 0;
  for (int p = 0; p < w->nparts; p++) { w->part_off[p] = acc; acc += w->part_n[p]; }
  w->part_off[w->nparts] = acc;
  size_t* fill = (size_t*)calloc((size_t)w->nparts, sizeof(size_t));
  if (!fill) { w->rc = PKO_ENOMEM; return NULL; }
  for (size_t i = 0; i < w->c.n; i++) {
    u128 key = w->wide ? w->c.k128[i].key : (u128)w->c.k64[i];
    int p = part_of(key, w->k, w->pbits);
    size_t d = w->part_off[p] + fill[p]++;
    if (w->wide) ((rec_t*)w->routed)[d] = w->c.k128[i];
    else ((uint64_t*)w->routed)[d] = w->c.k64[i];
  }
  free(fill);
  free(w->c.k64);
  free(w->c.k128);
  w->c.k64 = NULL;
  w->c.k128 = NULL;
  return NULL;
}

static void* mt_owner(void* arg) {
  mt_job* J = (mt_job*)arg;
  const size_t esz = J->wide ? sizeof(rec_t) : sizeof(uint64_t);
  while (1) {
    pthread_mutex_lock(&J->mu);
    int p = J->next_part++;
    pthread_mutex_unlock(&J->mu);
    if (p >= J->nparts) break;
    size_t n = 0;
    for (int t = 0; t < J->nthreads; t++) n += J->w[t].part_n[p];
    unsigned char* a = (unsigned char*)malloc((n ? n : 1) * esz);
    pko_key* keys = (pko_key*)malloc((n ? n : 1) * sizeof(pko_key));
    uint32_t* cnts = (uint32_t*)malloc((n ? n : 1) * sizeof(uint32_t));
    if (!a || !keys || !cnts) {
      free(a); free(keys); free(cnts);
      J->rc = PKO_ENOMEM;
      continue;
    }
    size_t o = 0;
    for (int t = 0; t < J->nthreads; t++) {
      memcpy(a + o * esz, (unsigned char*)J->w[t].routed + J->w[t].part_off[p] * esz, J->w[t].part_n[p] * esz);
      o += J->w[t].part_n[p];
    }
    int k = J->w[0].k;
    int rc = J->wide ? radix_sort_recs((rec_t*)a, n, 2 * k) : radix_sort_u64((uint64_t*)a, n, 2 * k);
    if (rc != PKO_OK) J->rc = rc;
    size_t u = 0;
    for (size_t i = 0; i < n;) {
      u128 key = J->wide ? ((rec_t*)a)[i].key : (u128)((uint64_t*)a)[i];
      size_t j = i + 1;
      while (j < n && (J->wide ? ((rec_t*)a)[j].key : (u128)((uint64_t*)a)[j]) == key) j++;
      keys[u].lo = (uint64_t)key;
      keys[u].hi = (uint64_t)(key >> 64);
      cnts[u] = (uint32_t)(j - i);
      u++;
      i = j;
    }
    free(a);
    J->out_keys[p] = keys;
    J->out_cnts[p] = cnts;
    J->out_u[p] = u;
    J->out_n[p] = n;
  }
  return NULL;
}

int pko_count_mt(const uint8_t* buf, size_t n, int k, int drop_n, int threads, pko_key** keys_out,
                 uint32_t** counts_out, size_t* n_unique, size_t* n_windows, size_t* n_reads) {
  if (k < 2 || k > 64 || threads < 1) return PKO_EARG;
  if (threads > 256) threads = 256;
  int pbits = 0;
  while ((1 << pbits) < 8 * threads && pbits < 2 * k && pbits < 16) pbits++;
  const int nparts = 1 << pbits;
  size_t first = 0;
  while (first < n && buf[first] != '>') first++;
  /* chunk starts: whole records ("\n>") */
  size_t* st = (size_t*)malloc(((size_t)threads + 1) * sizeof(size_t));
  mt_walker* w = (mt_walker*)calloc((size_t)threads, sizeof(mt_walker));
  pthread_t* th = (pthread_t*)malloc((size_t)threads * sizeof(pthread_t));
  if (!st || !w || !th) { free(st); free(w); free(th); return PKO_ENOMEM; }
  st[0] = first;
  for (int t = 1; t < threads; t++) {
    size_t p = first + (n - first) / (size_t)threads * (size_t)t;
    if (p < st[t - 1]) p = st[t - 1];
    while (p < n && !(buf[p] == '>' && p > 0 && buf[p - 1] == '\n')) p++;
    st[t] = p;
  }
  st[threads] = n;
  for (int t = 0; t < threads; t++) {
    w[t].buf = buf;
    w[t].begin = st[t];
    w[t].end = st[t + 1];
    w[t].k = k;
    w[t].drop_n = drop_n;
    w[t].wide = k > 32;
    w[t].pbits = pbits;
    w[t].nparts = nparts;
    pthread_create(&th[t], NULL, mt_walk, &w[t]);
  }
  int rc = PKO_OK;
  size_t reads = 0;
  for (int t = 0; t < threads; t++) {
    pthread_join(th[t], NULL);
    if (w[t].rc != PKO_OK) rc = w[t].rc;
    reads += w[t].reads;
  }
  mt_job J;
  memset(&J, 0, sizeof(J));
  J.w = w;
  J.nthreads = threads;
  J.nparts = nparts;
  J.wide = k > 32;
  pthread_mutex_init(&J.mu, NULL);
  J.out_keys = (pko_key**)calloc((size_t)nparts, sizeof(pko_key*));
  J.out_cnts = (uint32_t**)calloc((size_t)nparts, sizeof(uint32_t*));
  J.out_u = (size_t*)calloc((size_t)nparts, sizeof(size_t));
  J.out_n = (size_t*)calloc((size_t)nparts, sizeof(size_t));
  if (!J.out_keys || !J.out_cnts || !J.out_u || !J.out_n) rc = PKO_ENOMEM;
  if (rc == PKO_OK) {
    for (int t = 0; t < threads; t++) pthread_create(&th[t], NULL, mt_owner, &J);
    for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
    rc = J.rc;
  }
  size_t u = 0, nw = 0;
  if (rc == PKO_OK)
    for (int p = 0; p < nparts; p++) { u += J.out_u[p]; nw += J.out_n[p]; }
  pko_key* keys = NULL;
  uint32_t* cnts = NULL;
  if (rc == PKO_OK) {
    keys = (pko_key*)malloc((u ? u : 1) * sizeof(pko_key));
    cnts = (uint32_t*)malloc((u ? u : 1) * sizeof(uint32_t));
    if (!keys || !cnts) rc = PKO_ENOMEM;
  }
  size_t o = 0;
  for (int p = 0; p < nparts; p++) {
    if (rc == PKO_OK && J.out_u[p]) {
      memcpy(keys + o, J.out_keys[p], J.out_u[p] * sizeof(pko_key));
      memcpy(cnts + o, J.out_cnts[p], J.out_u[p] * sizeof(uint32_t));
      o += J.out_u[p];
    }
    if (J.out_keys) free(J.out_keys[p]);
    if (J.out_cnts) free(J.out_cnts[p]);
  }
  for (int t = 0; t < threads; t++) {
    free(w[t].part_n);
    free(w[t].part_off);
    free(w[t].routed);
    free(w[t].c.k64);
    free(w[t].c.k128);
  }
  free(J.out_keys); free(J.out_cnts); free(J.out_u); free(J.out_n);
  pthread_mutex_destroy(&J.mu);
  free(st); free(w); free(th);
  if (rc != PKO_OK) { free(keys); free(cnts); return rc; }
  *keys_out = keys;
  *counts_out = cnts;
  *n_unique = u;
  *n_windows = nw;
  if (n_reads) *n_reads = reads;
  return PKO_OK;
}

/* Frequency histogram over [0, t) and the first-minimum cutoff over [1, t). */
int pko_cutoff(const uint32_t* counts, size_t u, int t, uint64_t* hist, int* cutoff) {
  if (t < 1) return PKO_EARG;
  memset(hist, 0, (size_t)t * sizeof(uint64_t));
  for (size_t i = 0; i < u; i++)
    if (counts[i] < (uint32_t)t) hist[counts[i]]++;
  int best = 1;
  for (int c = 2; c < t; c++)
    if (hist[c] < hist[best]) best = c;
  *cutoff = best; /* t == 1: empty range, std::min_element returns the end -> 1 */
  return PKO_OK;
}

/*
 * Macro-nodes from the table.  node_keys: M keys; suf/pre: 4*M counts indexed by
 * ext code (0 = absent).  Returns PKO_EEMPTY when no entry reaches the cutoff.
 */
int pko_macro_nodes(const pko_key* keys, const uint32_t* counts, size_t u, int k,
                    uint32_t cutoff, pko_key** node_keys, uint32_t** suf_out, uint32_t** pre_out,
                    size_t* n_nodes, size_t* n_kept) {
  if (k < 2 || k > 64) return PKO_EARG;
  const int nb = 2 * (k - 1);
  const u128 succ_mask = key_mask(nb);
  size_t v = 0;
  for (size_t i = 0; i < u; i++) v += counts[i] >= cutoff;
  *n_kept = v;
  if (v == 0) return PKO_EEMPTY;
  /* suffix-side items in key order (grouped by x >> 2, ext ascending) */
  rec_t* sfx = (rec_t*)malloc(v * sizeof(rec_t));
  rec_t* pfx = (rec_t*)malloc(v * sizeof(rec_t));
  uint32_t* sc = (uint32_t*)malloc(v * sizeof(uint32_t));
  uint32_t* pc = (uint32_t*)malloc(v * sizeof(uint32_t));
  if (!sfx || !pfx || !sc || !pc) { free(sfx); free(pfx); free(sc); free(pc); return PKO_ENOMEM; }
  size_t j = 0;
  for (size_t i = 0; i < u; i++) {
    if (counts[i] < cutoff) continue;
    u128 x = ((u128)keys[i].hi << 64) | keys[i].lo;
    sfx[j].key = x >> 2;
    sfx[j].aux = (uint32_t)(x & 3); /* last base */
    sc[j] = counts[i];
    pfx[j].key = x & succ_mask;
    pfx[j].aux = (uint32_t)(x >> nb) | ((uint32_t)j << 2); /* first base, original slot */
    j++;
  }
  /* prefix-side items sorted by suffix (k-1)-mer; stable, so ties stay in ext order */
  int rc = radix_sort_recs(pfx, v, nb);
  if (rc != PKO_OK) { free(sfx); free(pfx); free(sc); free(pc); return rc; }
  for (size_t i = 0; i < v; i++) pc[i] = sc[pfx[i].aux >> 2];
  /* merge the two key-ordered streams into nodes */
  pko_key* nk = (pko_key*)malloc(2 * v * sizeof(pko_key));
  uint32_t* ns = (uint32_t*)calloc(8 * v, sizeof(uint32_t));
  uint32_t* np = (uint32_t*)calloc(8 * v, sizeof(uint32_t));
  if (!nk || !ns || !np) {
    free(sfx); free(pfx); free(sc); free(pc); free(nk); free(ns); free(np);
    return PKO_ENOMEM;
  }
  size_t a = 0, b = 0, m = 0;
  while (a < v || b < v) {
    u128 ka = a < v ? sfx[a].key : ~(u128)0;
    u128 kb = b < v ? pfx[b].key : ~(u128)0;
    u128 node = (a < v && (b >= v || ka <= kb)) ? ka : kb;
    nk[m].lo = (uint64_t)node;
    nk[m].hi = (uint64_t)(node >> 64);
    while (a < v && sfx[a].key == node) { ns[4 * m + sfx[a].aux] = sc[a]; a++; }
    while (b < v && pfx[b].key == node) { np[4 * m + (pfx[b].aux & 3)] = pc[b]; b++; }
    m++;
  }
  free(sfx); free(pfx); free(sc); free(pc);
  *node_keys = nk;
  *suf_out = ns;
  *pre_out = np;
  *n_nodes = m;
  return PKO_OK;
}

/* visit value (src/mn_construct.cpp:75-79): (int)ceil((double)count / coverage). */
int pko_visit(int count, int coverage) {
  int q = count / coverage, r = count % coverage;
  if (r != 0 && ((r > 0) == (coverage > 0))) q++;
  return q;
}

/*
 * Initial wiring of macro-nodes (src/wire.cpp:66-121 with MacroNode::setup_wiring,
 * includes/distribute_kmers.h:549-655).  Per node the suffix list holds the present
 * extensions in ascending base code then one terminal entry, the prefix list likewise
 * (the reference's suffix lists come out in that order; its prefix order is left to an
 * unstable sort, so ties below are broken in this canonical order).  Each entry has a
 * (count, visit) pair; a terminal gets count 1 and visit max(other side's visit sum -
 * own side's, 0).  Entries are ranked by visit, then count, both descending (Comp_rev,
 * :495-506; the lists have at most 5 entries, where std::sort is an insertion sort and
 * keeps equal entries in list order), and a two-pointer walk pairs prefix visits with
 * suffix visits: wire w = (suffix list index, offset into that suffix's visits, count);
 * when a prefix is used up, begin[prefix] = (index of its first wire, its wires).
 * Wires and begin entries that are never set stay 0, as in the reference.
 */
typedef struct {
  int32_t ns, np;             /* list sizes including the terminal entry */
  int32_t term_suf, term_pre; /* visits of the terminal entries */
  int32_t nw;                 /* wires written */
  int32_t wire[9][3];         /* suffix_id, offset_in_suffix, count */
  int32_t begin[5][2];        /* prefix_pos, num_wires */
} pko_wire;

static void rank_entries(const int32_t* cnt, const int32_t* vis, int n, int* order) {
  for (int i = 0; i < n; i++) order[i] = i;
  for (int i = 1; i < n; i++) { /* insertion sort, equal entries keep their order */
    int x = order[i], j = i - 1;
    while (j >= 0 && (vis[x] > vis[order[j]] || (vis[x] == vis[order[j]] && cnt[x] > cnt[order[j]]))) {
      order[j + 1] = order[j];
      j--;
    }
    order[j + 1] = x;
  }
}

int pko_wire_nodes(const uint32_t* suf, const uint32_t* pre, size_t m, int coverage, pko_wire* out) {
  if (coverage == 0) return PKO_EARG;
  for (size_t nidx = 0; nidx < m; nidx++) {
    pko_wire* w = &out[nidx];
    memset(w, 0, sizeof(*w));
    int32_t scnt[5], svis[5], pcnt[5], pvis[5];
    int ns = 0, np = 0, sc = 0, pc = 0;
    for (int e = 0; e < 4; e++) {
      const uint32_t c = suf[4 * nidx + e];
      if (c) { scnt[ns] = (int32_t)c; svis[ns] = pko_visit((int)c, coverage); sc += svis[ns]; ns++; }
    }
    for (int e = 0; e < 4; e++) {
      const uint32_t c = pre[4 * nidx + e];
      if (c) { pcnt[np] = (int32_t)c; pvis[np] = pko_visit((int)c, coverage); pc += pvis[np]; np++; }
    }
    scnt[ns] = 1; svis[ns] = pc - sc > 0 ? pc - sc : 0; ns++;
    pcnt[np] = 1; pvis[np] = sc - pc > 0 ? sc - pc : 0; np++;
    w->ns = ns; w->np = np; w->term_suf = svis[ns - 1]; w->term_pre = pvis[np - 1];
    int os[5], op[5];
    rank_entries(scnt, svis, ns, os);
    rank_entries(pcnt, pvis, np, op);
    int leftover = sc + svis[ns - 1];
    int off_s[5] = {0, 0, 0, 0, 0};
    int top_p = 0, top_s = 0, var_p = 0, var_s = 0, wi = 0, p_size = 0, last_pid = -1, begin_pos = -1;
    while (leftover > 0 && wi < 9) {
      const int sid = os[top_s], pid = op[top_p];
      const int a = pvis[pid] - var_p, b = svis[sid] - var_s;
      const int cnt = a < b ? a : b;
      w->wire[wi][0] = sid; w->wire[wi][1] = off_s[sid]; w->wire[wi][2] = cnt;
      if (last_pid != pid) { begin_pos = wi; last_pid = pid; }
      p_size++; wi++;
      leftover -= cnt; var_p += cnt; var_s += cnt; off_s[sid] += cnt;
      if (var_p == pvis[pid]) {
        var_p = 0; top_p++;
        w->begin[pid][0] = begin_pos; w->begin[pid][1] = p_size;
        p_size = 0;
      }
      if (var_s == svis[sid]) { var_s = 0; top_s++; }
    }
    w->nw = wi;
  }
  return PKO_OK;
}

void pko_free(void* p) { free(p); }
