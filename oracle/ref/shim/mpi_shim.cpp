// Single-rank implementation of the MPI subset declared in mpi.h.
// TEST INFRASTRUCTURE ONLY (see mpi.h): it lets the reference's hot-path
// sources run unmodified as one rank so their outputs can pin the oracle.
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

extern "C" {

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) {
  fflush(stdout);
  fprintf(stderr, "[mpi-shim] MPI_Abort(%d)\n", code);
  fflush(stderr);
  exit(code == 0 ? 1 : (code & 0xff) ? (code & 0xff) : 1);
}
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out) {
  *out = (MPI_Datatype)count * old;
  return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype*) { return MPI_SUCCESS; }

int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  memmove(r, s, (size_t)count * (size_t)t);
  return MPI_SUCCESS;
}
int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  memmove(r, s, (size_t)count * (size_t)t);
  return MPI_SUCCESS;
}
int MPI_Alltoall(const void* s, int scount, MPI_Datatype st, void* r, int, MPI_Datatype,
                 MPI_Comm) {
  memmove(r, s, (size_t)scount * (size_t)st);
  return MPI_SUCCESS;
}
int MPI_Alltoallv(const void* s, const int* scounts, const int* sdispls, MPI_Datatype st, void* r,
                  const int*, const int* rdispls, MPI_Datatype rt, MPI_Comm) {
  memmove((char*)r + (size_t)rdispls[0] * (size_t)rt, (const char*)s + (size_t)sdispls[0] * (size_t)st,
          (size_t)scounts[0] * (size_t)st);
  return MPI_SUCCESS;
}

int MPI_Allgather(const void* s, int scount, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) {
  memmove(r, s, (size_t)scount * (size_t)st);
  return MPI_SUCCESS;
}
int MPI_Allgatherv(const void* s, int scount, MPI_Datatype st, void* r, const int*, const int* rdispls,
                   MPI_Datatype rt, MPI_Comm) {
  memmove((char*)r + (size_t)rdispls[0] * (size_t)rt, s, (size_t)scount * (size_t)st);
  return MPI_SUCCESS;
}

int MPI_File_open(MPI_Comm, const char* name, int, MPI_Info, MPI_File* fh) {
  fh->fp = fopen(name, "rb");
  return fh->fp ? MPI_SUCCESS : 1;
}
int MPI_File_get_size(MPI_File fh, MPI_Offset* size) {
  FILE* f = (FILE*)fh.fp;
  long cur = ftell(f);
  fseek(f, 0, SEEK_END);
  *size = (MPI_Offset)ftell(f);
  fseek(f, cur, SEEK_SET);
  return MPI_SUCCESS;
}
int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void* buf, int count, MPI_Datatype t,
                         MPI_Status*) {
  FILE* f = (FILE*)fh.fp;
  fseek(f, (long)off, SEEK_SET);
  size_t want = (size_t)count * (size_t)t;
  size_t got = fread(buf, 1, want, f);
  (void)got;
  return MPI_SUCCESS;
}
int MPI_File_close(MPI_File* fh) {
  if (fh->fp) fclose((FILE*)fh->fp);
  fh->fp = 0;
  return MPI_SUCCESS;
}

}  // extern "C"
