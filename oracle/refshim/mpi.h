/* mpi.h — single-rank stand-in so the reference's HAVE_MPI code paths compile
 * on the CPU checker build.  With one rank MPI_Allreduce is a copy, which
 * gives `fsMax` (src/cart3d.cpp:191-198) its initialised single-rank value.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef FST_MPI_SHIM_H
#define FST_MPI_SHIM_H
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_DOUBLE 8
#define MPI_FLOAT 4
#define MPI_INT 40
#define MPI_MAX 1
#define MPI_SUM 2
#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c) {
  (void)o; (void)c;
  memcpy(r, s, (size_t)n * (size_t)(t == MPI_INT ? 4 : t));
  return 0;
}
#endif
