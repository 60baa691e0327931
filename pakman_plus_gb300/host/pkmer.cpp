// pkmer: command-line driver of the GB300 counting -> cutoff -> macro-node path.
//
// Options, defaults, messages and exit behaviour follow the reference's
// parseCommandLine (src/distribute_kmers.cpp:217-313) and input reading
// (src/input_reading.cpp:246-266):
//   -f FILE  input FASTA (required; "Must specify an input FASTA file name with -f")
//   -b N     batch size MAX_KMER_COUNT (default 100000000, with the reference's notice):
//            an input that does not fit the GPU's memory budget at once is counted in
//            record-aligned pieces of at most N bytes (so at most N k-mer windows) whose
//            tables are merged on the device -- the reference's batch flush -- and the
//            table is the same for any N
//   -r N     read length (required, 100..250)
//   -c N     coverage (required)
//   -t N     histogram buckets num_buckets (default 21)
//   -n N     node threshold (default 100000)
//   -i, -p V select CPU counting variants in the reference; every variant builds the
//            same table, so they are accepted and have no effect here
// The reference's build knobs ksize and LMER_LENGTH are run-time options here:
//   -k K     k-mer length, 2..64 (default 32)
//   -l L     LMER_LENGTH (default 8)
// and five options of this driver:
//   -o PFX   write PFX.table ("PKT1") and PFX.mn ("PKM1") binary dumps
//   -d DEV   CUDA device (default 0)
//   -N       drop k-mers spanning N (default: the reference's behaviour, kept)
//   -M BYTES HBM budget of the run (default: the whole device); counting switches to -b
//            pieces when the input does not fit it at once
//   -g       contig generation, as the reference's PERFORM_CONTIG_GENERATION build
//            (src/distribute_kmers.cpp:156-203): iterative compaction down to the -n
//            threshold, the walk, and the contig files that build writes into the
//            working directory -- contigs_par_r0.fa (partial contigs of the rounds)
//            and contigs_out_r0.fa (walk contigs), each contig longer than 400 bases
//            as ">contig_<i>_l_<length>_r_0" and its bases, i counting across both
//            files (src/walk.cpp:198-227, 488-515)
// A failed requirement prints the reference's message and exits with status 157
// (MPI_Abort(MPI_COMM_WORLD, -99) of a single process); an unreadable input exits 2.
#include <getopt.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <string>
#include <vector>

#include "pakman_gb300.h"

namespace {

constexpr int kAbortStatus = 157;  // (unsigned char)-99

double now_s() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

[[noreturn]] void abort_run(const char* msg) {
  fflush(stdout);
  fprintf(stderr, "%s\n", msg);
  exit(kAbortStatus);
}

[[noreturn]] void die_pk(const char* what, pk_status s) {
  fflush(stdout);
  fprintf(stderr, "%s: %s (%s)\n", what, pk_status_string(s), pk_last_error());
  if (s == PK_ERR_EMPTY || s == PK_ERR_FORMAT) exit(kAbortStatus);
  exit(1);
}

void put_key(FILE* f, const uint64_t* keys, uint64_t i, int wide) {
  uint64_t lo = wide ? keys[2 * i] : keys[i];
  uint64_t hi = wide ? keys[2 * i + 1] : 0;
  fwrite(&lo, 8, 1, f);
  fwrite(&hi, 8, 1, f);
}

// one side of a node: entries in ascending extension code
void put_side(FILE* f, const uint32_t* cnt, int coverage) {
  uint32_t n = 0;
  for (int e = 0; e < 4; e++) n += cnt[e] != 0;
  fwrite(&n, 4, 1, f);
  for (int e = 0; e < 4; e++) {
    if (!cnt[e]) continue;
    uint8_t ext = (uint8_t)e, term = 0;
    int32_t c = (int32_t)cnt[e];
    int32_t v = (int32_t)((cnt[e] + (uint32_t)coverage - 1) / (uint32_t)coverage);
    fwrite(&ext, 1, 1, f);
    fwrite(&c, 4, 1, f);
    fwrite(&v, 4, 1, f);
    fwrite(&term, 1, 1, f);
  }
}

}  // namespace

int main(int argc, char** argv) {
  std::string input, out_prefix;
  unsigned long max_kmer_count = 0;
  int read_length = 0, coverage = 0, num_buckets = 0, node_threshold = 0;
  int k = 32, lmer = 8, device = 0, drop_n = 0, gen = 0;
  unsigned long long budget = 0;
  int ret;
  while ((ret = getopt(argc, argv, "f:b:r:c:t:n:ip:k:l:o:d:NgM:")) != -1) {
    switch (ret) {
      case 'f': input.assign(optarg); break;
      case 'b':
        if (sscanf(optarg, "%lu", &max_kmer_count) != 1) {
          fprintf(stderr, "[Invalid option of -b %s\n", optarg);
          abort();  // the reference throws std::logic_error here
        }
        break;
      case 'r': read_length = atoi(optarg); break;
      case 'c': coverage = atoi(optarg); break;
      case 't': num_buckets = atoi(optarg); break;
      case 'n': node_threshold = atoi(optarg); break;
      case 'i': break;
      case 'p': break;
      case 'k': k = atoi(optarg); break;
      case 'l': lmer = atoi(optarg); break;
      case 'o': out_prefix.assign(optarg); break;
      case 'd': device = atoi(optarg); break;
      case 'N': drop_n = 1; break;
      case 'g': gen = 1; break;
      case 'M':
        if (sscanf(optarg, "%llu", &budget) != 1) abort_run("-M takes a byte count");
        break;
      default:
        fprintf(stderr, "Should not reach here!!\n");
        abort();  // the reference asserts
    }
  }
  if (input.empty()) abort_run("Must specify an input FASTA file name with -f");
  if (!max_kmer_count) {
    max_kmer_count = 100000000;
    printf("batch size not specified with -b, set to default value MAX_KMER_COUNT=100000000\n");
  }
  if (!read_length) abort_run("Must specify read_length with -r");
  if (!coverage) abort_run("Must specify coverage of the input data with -c");
  if (read_length > 250 || read_length < 100)
    abort_run("Must provide short reads of length >100 and <=250 with -r");
  if (!num_buckets) {
    num_buckets = 21;
    printf("num_buckets not specified with -t, set to default value num_buckets=21\n");
  }
  if (!node_threshold) {
    node_threshold = 100000;
    printf("node_threashold not specified with -n, set to default value node_threashold=100K\n");
  }
  if (k < 2 || k > 64) abort_run("k-mer size must be in 2..64 with -k");
  printf("K-mer size: %d, L-mer size: %d, Number of Processes: %d, MAX_KMER_COUNT: %ld Coverage: %d,",
         k, lmer, 1, (long)max_kmer_count, coverage);
  printf("Avg read length: %d, Num buckets: %d, Node threshold: %d\n", read_length, num_buckets,
         node_threshold);
  fflush(stdout);

  // ---- input reading (perform_input_reading): the file is streamed to the device
  // by pk_count_file below; an unreadable file ends the run as the reference's does
  FILE* fin = fopen(input.c_str(), "rb");
  if (!fin) {
    fprintf(stderr, "Couldn't open the input FASTA file\n");
    exit(2);
  }
  fclose(fin);
  pk_status st = PK_OK;

  pk_ctx* ctx = nullptr;
  pk_job* job = nullptr;
  if ((st = pk_ctx_create(device, (uint64_t)budget, &ctx)) != PK_OK) die_pk("pk_ctx_create", st);
  if ((st = pk_job_create(ctx, nullptr, &job)) != PK_OK) die_pk("pk_job_create", st);
  pk_params p;
  pk_params_default(&p);
  p.k = k;
  p.lmer_length = lmer;
  p.num_buckets = num_buckets;
  p.coverage = coverage;
  p.read_length = read_length;
  p.drop_n = drop_n;
  p.batch_kmers = max_kmer_count;

  // ---- input reading streamed into counting (perform_kmer_counting)
  double t2 = now_s();
  st = pk_count_file(job, input.c_str(), 0, 1, &p);
  if (st == PK_ERR_IO) {
    fprintf(stderr, "Couldn't open the input FASTA file\n");
    exit(2);
  }
  if (st != PK_OK) die_pk("k-mer counting", st);
  uint64_t u = 0, nwin = 0, nreads = 0;
  pk_table_info(job, &u, &nwin, &nreads);
  uint32_t pieces = 1;
  pk_count_pieces(job, &pieces);
  double t3 = now_s();
  printf("input reading and k-mer counting (secs): %f, reads: %llu, k-mer instances: %llu, unique k-mers: %llu\n",
         t3 - t2, (unsigned long long)nreads, (unsigned long long)nwin, (unsigned long long)u);
  printf("Number of batch iterations: %u\n", pieces);
  const int wide = k > 32;
  if (!out_prefix.empty()) {
    std::vector<uint64_t> keys((size_t)u * (wide ? 2 : 1) + 2);
    std::vector<uint32_t> cnts((size_t)u + 1);
    if ((st = pk_copy_table(job, keys.data(), cnts.data(), u)) != PK_OK) die_pk("pk_copy_table", st);
    FILE* f = fopen((out_prefix + ".table").c_str(), "wb");
    if (!f) abort_run("cannot write the table dump");
    uint32_t kk = (uint32_t)k;
    fwrite("PKT1", 1, 4, f);
    fwrite(&kk, 4, 1, f);
    fwrite(&u, 8, 1, f);
    for (uint64_t i = 0; i < u; i++) {
      put_key(f, keys.data(), i, wide);
      int32_t c = (int32_t)cnts[i];
      fwrite(&c, 4, 1, f);
    }
    fclose(f);
  }

  // ---- histogram cutoff + macro-nodes (begin_mnode_construction)
  double t4 = now_s();
  uint32_t cutoff = 0;
  uint64_t kept = 0;
  std::vector<uint64_t> hist((size_t)num_buckets);
  st = pk_cutoff(job, num_buckets, &cutoff, hist.data(), &kept);
  printf("histogram cutoff: %u, kept k-mers: %llu\n", cutoff, (unsigned long long)kept);
  if (st == PK_ERR_EMPTY) {
    fflush(stdout);
    fprintf(stderr, "No k-mers left after the frequency cutoff\n");
    exit(kAbortStatus);
  }
  if (st != PK_OK) die_pk("pk_cutoff", st);
  uint64_t m = 0;
  if ((st = pk_build_macro_nodes(job, 0, &m)) != PK_OK) die_pk("macro-node construction", st);
  double t5 = now_s();
  printf("MN node construction (secs): %f, macro-nodes: %llu\n", t5 - t4, (unsigned long long)m);
  if (!out_prefix.empty()) {
    std::vector<uint64_t> keys((size_t)m * (wide ? 2 : 1) + 2);
    std::vector<uint32_t> suf((size_t)m * 4 + 4), pre((size_t)m * 4 + 4);
    if ((st = pk_copy_macro_nodes(job, keys.data(), suf.data(), pre.data(), m)) != PK_OK)
      die_pk("pk_copy_macro_nodes", st);
    FILE* f = fopen((out_prefix + ".mn").c_str(), "wb");
    if (!f) abort_run("cannot write the macro-node dump");
    uint32_t kk = (uint32_t)k, kl = (uint32_t)(k - 1);
    fwrite("PKM1", 1, 4, f);
    fwrite(&kk, 4, 1, f);
    fwrite(&m, 8, 1, f);
    for (uint64_t i = 0; i < m; i++) {
      put_key(f, keys.data(), i, wide);
      fwrite(&kl, 4, 1, f);
      const uint64_t lo = wide ? keys[2 * i] : keys[i];
      const uint64_t hi = wide ? keys[2 * i + 1] : 0;
      for (int b = (int)kl - 1; b >= 0; b--) {  // the node's bases, first base first
        const int sh = 2 * b;
        uint8_t base = (uint8_t)(sh >= 64 ? (hi >> (sh - 64)) & 3 : (lo >> sh) & 3);
        fwrite(&base, 1, 1, f);
      }
      put_side(f, &suf[4 * i], coverage);
      put_side(f, &pre[4 * i], coverage);
    }
    fclose(f);
  }
  if (gen) {
    double t6 = now_s();
    pk_compaction_info ci;
    if ((st = pk_compact(job, (uint64_t)node_threshold, coverage, &ci)) != PK_OK) die_pk("iterative compaction", st);
    std::vector<uint64_t> poff(ci.n_contigs + 1);
    std::vector<uint8_t> pb(ci.contig_bases + 1);
    if ((st = pk_copy_partial_contigs(job, poff.data(), pb.data())) != PK_OK) die_pk("pk_copy_partial_contigs", st);
    double t7 = now_s();
    printf("iterative compaction (secs): %f, rounds: %d, macro-nodes left: %llu, partial contigs: %llu\n",
           t7 - t6, ci.rounds, (unsigned long long)ci.n_nodes, (unsigned long long)ci.n_contigs);
    pk_walk_info wi;
    if ((st = pk_walk(job, &wi)) != PK_OK) die_pk("walk", st);
    std::vector<uint64_t> woff(wi.n_contigs + 1);
    std::vector<uint8_t> wb(wi.contig_bases + 1);
    if ((st = pk_copy_walk_contigs(job, woff.data(), wb.data())) != PK_OK) die_pk("pk_copy_walk_contigs", st);
    double t8 = now_s();
    printf("walk (secs): %f, begin k-mers: %llu, contigs: %llu\n", t8 - t7, (unsigned long long)wi.n_begins,
           (unsigned long long)wi.n_contigs);
    int num_contigs = 0;
    auto write_fa = [&](const char* name, const std::vector<uint64_t>& off, const std::vector<uint8_t>& b) {
      FILE* f = fopen(name, "w");
      if (!f) abort_run("Error opening output contig file!");
      static const char sym[4] = {'A', 'C', 'T', 'G'};
      std::string seq;
      for (size_t c = 0; c + 1 < off.size(); c++) {
        const uint64_t len = off[c + 1] - off[c];
        if (len <= 400) continue;
        seq.resize(len);
        for (uint64_t i = 0; i < len; i++) seq[i] = sym[b[off[c] + i] & 3];
        fprintf(f, ">contig_%d_l_%llu_r_0\n%s\n", ++num_contigs, (unsigned long long)len, seq.c_str());
      }
      fclose(f);
    };
    write_fa("contigs_par_r0.fa", poff, pb);
    write_fa("contigs_out_r0.fa", woff, wb);
    t5 = now_s();
  }
  printf("pakman-gb300-elapsed-time-no-io (secs): %f\n", t5 - t2);
  pk_job_destroy(job);
  pk_ctx_destroy(ctx);
  return 0;
}
