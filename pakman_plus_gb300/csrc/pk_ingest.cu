// File ingest behind pk_fasta_slice / pk_count_file (include/pakman_gb300.h): the
// slice rule of the reference's DivideReads (src/input_reading.cpp:68-243) and a
// streamed load of that slice into the job's device buffer.  Reader threads pread
// 16 MiB pieces into pinned staging buffers; each piece is copied to the device on
// the job's stream and its 64 KiB tiles are line-scanned right behind the copy, so
// file reads, host-to-device copies and the line scan overlap.  Counting then starts
// at the tile prefix (count_impl with lines_ready).
#include <cuda_runtime.h>
#include <errno.h>
#include <fcntl.h>
#include <stdint.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pakman_gb300.h"
#include "pk_internal.h"
#include "pk_runtime.h"

using namespace pk;

namespace {

constexpr uint64_t kPiece = 16ull << 20;  // bytes per staged piece
static_assert(kPiece % kTileBytes == 0, "a piece must end on a line-scan tile boundary");
constexpr int kReaders = pk_job::kIngestBufs / 2;  // two staging buffers per reader

struct Fd {
  int fd = -1;
  ~Fd() {
    if (fd >= 0) close(fd);
  }
};

// n bytes at file offset off (short reads are continued)
bool read_at(int fd, void* dst, uint64_t n, uint64_t off) {
  char* p = static_cast<char*>(dst);
  while (n) {
    const ssize_t r = pread(fd, p, (size_t)std::min<uint64_t>(n, 1ull << 30), (off_t)off);
    if (r < 0) {
      if (errno == EINTR) continue;
      return false;
    }
    if (r == 0) return false;  // the file ended early (it shrank)
    p += r;
    n -= (uint64_t)r;
    off += (uint64_t)r;
  }
  return true;
}

// First '>' at or after byte `from`; the file size when there is none.
bool next_record(int fd, uint64_t size, uint64_t from, uint64_t* at) {
  std::vector<char> buf(1 << 16);
  for (uint64_t pos = from; pos < size;) {
    const uint64_t n = std::min<uint64_t>(buf.size(), size - pos);
    if (!read_at(fd, buf.data(), n, pos)) return false;
    const void* q = memchr(buf.data(), '>', (size_t)n);
    if (q) {
      *at = pos + (uint64_t)(static_cast<const char*>(q) - buf.data());
      return true;
    }
    pos += n;
  }
  *at = size;
  return true;
}

pk_status open_file(const char* path, Fd& f, uint64_t* size) {
  f.fd = open(path, O_RDONLY);
  if (f.fd < 0)
    return set_error(PK_ERR_IO, std::string("Couldn't open the input FASTA file ") + path + ": " + strerror(errno));
  struct stat st;
  if (fstat(f.fd, &st) != 0 || !S_ISREG(st.st_mode))
    return set_error(PK_ERR_IO, std::string("the input FASTA file is not a readable regular file: ") + path);
  *size = (uint64_t)st.st_size;
  return PK_OK;
}

// DivideReads: rank r nominally owns [r * (S / n), (r + 1) * (S / n)) (the last rank to
// the end); its data run from the first '>' at or after its nominal start (rank 0:
// byte 0) to the first '>' at or after the next rank's nominal start (the last rank:
// the end of the file).
pk_status slice_of(int fd, uint64_t size, int rank, int n, uint64_t* off, uint64_t* len) {
  const uint64_t local = size / (uint64_t)n;
  uint64_t b = 0, e = size;
  if (rank != 0 && !next_record(fd, size, (uint64_t)rank * local, &b))
    return set_error(PK_ERR_IO, "reading the input FASTA file failed");
  if (rank != n - 1 && !next_record(fd, size, (uint64_t)(rank + 1) * local, &e))
    return set_error(PK_ERR_IO, "reading the input FASTA file failed");
  if (e < b) e = b;
  *off = b;
  *len = e - b;
  return PK_OK;
}

pk_status check_rank(int32_t rank, int32_t n_ranks) {
  if (n_ranks < 1 || rank < 0 || rank >= n_ranks)
    return set_error(PK_ERR_INVALID, "rank must lie in [0, n_ranks) and n_ranks must be >= 1");
  return PK_OK;
}

pk_status stream_and_count(pk_job* j, Fd& f, const char* path, uint64_t off, uint64_t len, const pk_params* p);

}  // namespace

extern "C" pk_status pk_fasta_slice(const char* path, int32_t rank, int32_t n_ranks, int32_t read_length,
                                    uint64_t* offset, uint64_t* length) {
  if (!path || !offset || !length) return set_error(PK_ERR_INVALID, "path, offset and length must not be null");
  if (read_length < 0) return set_error(PK_ERR_INVALID, "read_length must be >= 0");
  PK_TRY(check_rank(rank, n_ranks));
  Fd f;
  uint64_t size = 0;
  PK_TRY(open_file(path, f, &size));
  return slice_of(f.fd, size, rank, n_ranks, offset, length);
}

extern "C" pk_status pk_count_file(pk_job* j, const char* path, int32_t rank, int32_t n_ranks,
                                   const pk_params* p) {
  if (!j) return set_error(PK_ERR_INVALID, "job is null");
  if (!path) return set_error(PK_ERR_INVALID, "path is null");
  PK_TRY(check_params(p));
  PK_TRY(check_rank(rank, n_ranks));
  Fd f;
  uint64_t size = 0, off = 0, len = 0;
  PK_TRY(open_file(path, f, &size));
  PK_TRY(slice_of(f.fd, size, rank, n_ranks, &off, &len));
  PK_TRY(set_device(j->ctx));
  for (int i = 0; i < ST_COUNT_; i++) j->ev_rec[i] = false;
  // -b pieces (always, or when the slice does not fit at once): the slice is read into
  // host memory and counted piece by piece
  auto in_pieces = [&]() -> pk_status {
    std::vector<char> host(len ? len : 1);
    if (len && !read_at(f.fd, host.data(), len, off))
      return set_error(PK_ERR_IO, std::string("reading the input FASTA file failed: ") + path);
    const uint64_t b = p->batch_kmers ? p->batch_kmers : 100000000ull;
    return count_pieces(j, host.data(), len, p, p->chunking == 1 ? b : std::min<uint64_t>(b, (len + 1) / 2));
  };
  if (p->chunking == 1) return in_pieces();
  const pk_status whole = stream_and_count(j, f, path, off, len, p);
  if ((whole == PK_ERR_NOMEM || whole == PK_ERR_LIMIT) && p->chunking == 0 && len > 1) {
    PK_CUDA(cudaStreamSynchronize(j->stream));
    job_free_all(j);
    return in_pieces();
  }
  return whole;
}

namespace {

// The whole slice streamed to the device and counted at once.
pk_status stream_and_count(pk_job* j, Fd& f, const char* path, uint64_t off, uint64_t len, const pk_params* p) {
  PK_TRY(job_alloc(j, j->fasta, (size_t)len + 16));
  const uint64_t ntiles = (len + kTileBytes - 1) / kTileBytes;
  PK_TRY(job_alloc(j, j->tile_nl, sizeof(uint32_t) * (ntiles + 1)));
  for (int i = 0; i < pk_job::kIngestBufs; i++) {
    if (!j->ing_host[i]) PK_CUDA(cudaHostAlloc(&j->ing_host[i], kPiece, cudaHostAllocDefault));
    if (!j->ing_ev[i]) PK_CUDA(cudaEventCreateWithFlags(&j->ing_ev[i], cudaEventDisableTiming));
  }
  // the scalars as counting initialises them; every piece's scan adds to them
  Scalars init{};
  memset(&init, 0, sizeof(init));
  init.s0 = ~0ull;
  *j->h_sc = init;
  PK_CUDA(cudaMemcpyAsync(j->d_sc, j->h_sc, sizeof(Scalars), cudaMemcpyHostToDevice, j->stream));

  mark_begin(j, ST_H2D);
  const uint64_t npieces = (len + kPiece - 1) / kPiece;
  std::mutex mu;
  pk_status first = PK_OK;
  std::string first_msg;
  auto record = [&](pk_status s, const std::string& m) {
    std::lock_guard<std::mutex> g(mu);
    if (first == PK_OK) {
      first = s;
      first_msg = m;
    }
  };
  auto failed = [&]() {
    std::lock_guard<std::mutex> g(mu);
    return first != PK_OK;
  };
  // reader t takes pieces t, t + R, t + 2R, ... and alternates its two buffers; a
  // buffer is refilled only after the copy that last read it has completed
  auto reader = [&](int t) {
    cudaError_t e = cudaSetDevice(j->ctx->device);
    uint64_t m = 0;
    for (uint64_t i = (uint64_t)t; i < npieces && e == cudaSuccess; i += kReaders, m++) {
      if (failed()) return;
      const int b = 2 * t + (int)(m & 1);
      const uint64_t o = i * kPiece, n = std::min<uint64_t>(kPiece, len - o);
      e = cudaEventSynchronize(j->ing_ev[b]);
      if (e != cudaSuccess) break;
      if (!read_at(f.fd, j->ing_host[b], n, off + o)) {
        record(PK_ERR_IO, std::string("reading the input FASTA file failed: ") + path);
        return;
      }
      e = cudaMemcpyAsync(static_cast<char*>(j->fasta.p) + o, j->ing_host[b], n, cudaMemcpyHostToDevice,
                          j->stream);
      if (e == cudaSuccess) e = cudaEventRecord(j->ing_ev[b], j->stream);
      if (e == cudaSuccess)
        e = launch_line_tiles(static_cast<const uint8_t*>(j->fasta.p), len, static_cast<uint32_t*>(j->tile_nl.p),
                              j->d_sc, o / kTileBytes, (n + kTileBytes - 1) / kTileBytes, j->stream);
    }
    if (e != cudaSuccess) record(PK_ERR_CUDA, std::string("file ingest: ") + cudaGetErrorString(e));
  };
  const int nthreads = (int)std::min<uint64_t>((uint64_t)kReaders, npieces);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; t++) th.emplace_back(reader, t);
  for (auto& x : th) x.join();
  if (first != PK_OK) return set_error(first, first_msg);
  mark_end(j, ST_H2D);
  j->lines_ready = true;
  const pk_status s = count_impl(j, j->fasta.p, len, p);
  j->lines_ready = false;
  return s;
}

}  // namespace
