/* Single-process stand-in for the four MPI calls the reference makes, so the
 * reference C sources compile without an MPI installation.  Rank 0 of 1;
 * MPI_Allreduce copies its send buffer (the sum over one rank).  Test
 * infrastructure only: used to build the reference checker in oracle/_ref. */
#ifndef EMMI_ORACLE_MPI_STUB_H
#define EMMI_ORACLE_MPI_STUB_H
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_SUM 0

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t,
                                MPI_Op op, MPI_Comm c)
{
  (void)op; (void)c;
  if (s != r) memmove(r, s, (size_t)n * (size_t)t);
  return 0;
}
#endif
