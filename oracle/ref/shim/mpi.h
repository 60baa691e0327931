/*
 * Single-rank stand-in for the MPI calls made by PaKman's k-mer counting,
 * histogram, macro-node and compaction translation units.
 *
 * TEST INFRASTRUCTURE ONLY: this header exists so the reference's own sources
 * (src/distribute_kmers.cpp, src/input_reading.cpp, src/kmer_counting.cpp,
 * src/kmer_histogram.cpp, src/mn_construct.cpp, src/timers.cpp, the compaction
 * units) compile
 * unmodified on a machine without MPI and run as one rank.  With one rank every
 * collective is a local copy: Allreduce/Reduce copy send to receive, Alltoall(v)
 * and Allgather(v) copy the rank-0 block, MPI-IO reads through stdio.  Nothing in the GPU
 * product includes or links this file.
 */
#ifndef PK_REF_MPI_SHIM_H
#define PK_REF_MPI_SHIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A datatype handle is simply the element size in bytes. */
typedef long MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef struct { void* fp; } MPI_File;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_INFO_NULL 0
#define MPI_MODE_RDONLY 1
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_UNSIGNED ((MPI_Datatype)4)
#define MPI_LONG ((MPI_Datatype)8)
#define MPI_UNSIGNED_LONG ((MPI_Datatype)8)
#define MPI_LONG_LONG ((MPI_Datatype)8)
#define MPI_UINT64_T ((MPI_Datatype)8)
#define MPI_INT64_T ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)8)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out);
int MPI_Type_commit(MPI_Datatype* t);
int MPI_Type_free(MPI_Datatype* t);

int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Alltoall(const void* s, int scount, MPI_Datatype st, void* r, int rcount, MPI_Datatype rt,
                 MPI_Comm c);
int MPI_Alltoallv(const void* s, const int* scounts, const int* sdispls, MPI_Datatype st, void* r,
                  const int* rcounts, const int* rdispls, MPI_Datatype rt, MPI_Comm c);
int MPI_Allgather(const void* s, int scount, MPI_Datatype st, void* r, int rcount, MPI_Datatype rt,
                  MPI_Comm c);
int MPI_Allgatherv(const void* s, int scount, MPI_Datatype st, void* r, const int* rcounts,
                   const int* rdispls, MPI_Datatype rt, MPI_Comm c);

int MPI_File_open(MPI_Comm c, const char* name, int mode, MPI_Info info, MPI_File* fh);
int MPI_File_get_size(MPI_File fh, MPI_Offset* size);
int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void* buf, int count, MPI_Datatype t,
                         MPI_Status* st);
int MPI_File_close(MPI_File* fh);

#ifdef __cplusplus
}
#endif
#endif
