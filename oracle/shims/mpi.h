/* Single-rank stand-in for the MPI API subset the reference sources use.
 * TEST INFRASTRUCTURE ONLY: lets the unmodified reference (main.c, read_data.c,
 * read_params.c, vars.c) compile as the oracle binary oracle/_ref/capow_ref.
 * One rank: Comm_rank = 0, Comm_size = 1; reductions and gathers copy;
 * Sendrecv to/from self copies, MPI_PROC_NULL leaves the receive buffer untouched
 * (exactly the halo semantics of read_data.c:152-175 on one rank). */
#ifndef CAPOW_SHIM_MPI_H
#define CAPOW_SHIM_MPI_H
#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_UNSIGNED_LONG_LONG 3
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_PROC_NULL (-2)

int MPI_Init(int *argc, char ***argv);
int MPI_Comm_rank(MPI_Comm c, int *rank);
int MPI_Comm_size(MPI_Comm c, int *size);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm c, int code);
int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm c);
int MPI_Sendrecv(const void *s, int sc, MPI_Datatype st, int dest, int stag, void *r, int rc, MPI_Datatype rt,
                 int src, int rtag, MPI_Comm c, MPI_Status *status);
#endif
