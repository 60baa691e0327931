// Calls the reference's DivideReads (src/input_reading.cpp:68-243) once and writes
// the data it returns for that rank (TEST INFRASTRUCTURE ONLY; built from the
// reference sources by `make -C oracle/ref divide`).
//
//   divide_reads_ref FILE RANK SIZE OVERLAP OUT      stdout: "<'>' count> <bytes>"
#include <mpi.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

char* DivideReads(MPI_File* in, const int rank, const int size, const int overlap, uint64_t* nlines,
                  size_t* data_size);

int main(int argc, char** argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: %s FILE RANK SIZE OVERLAP OUT\n", argv[0]);
    return 2;
  }
  MPI_File in;
  if (MPI_File_open(MPI_COMM_WORLD, argv[1], MPI_MODE_RDONLY, MPI_INFO_NULL, &in)) return 3;
  uint64_t nlines = 0;
  size_t n = 0;
  char* data = DivideReads(&in, atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), &nlines, &n);
  MPI_File_close(&in);
  FILE* f = fopen(argv[5], "wb");
  if (!f) return 4;
  if (n) fwrite(data, 1, n, f);
  fclose(f);
  printf("%llu %zu\n", (unsigned long long)nlines, n);
  free(data);
  return 0;
}
