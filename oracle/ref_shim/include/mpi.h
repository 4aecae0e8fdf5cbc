/* Single-rank stand-in for the MPI interface used by MG-PICOLA (reference
 * test build only).  Written from the MPI standard's semantics for one process:
 * reductions copy, self send/receive copies, everything else is a no-op. */
#ifndef REF_SHIM_MPI_H
#define REF_SHIM_MPI_H
#include <stddef.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef int MPI_Request;
#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
#define MPI_IN_PLACE ((void *)1)
#define MPI_TYPECLASS_REAL 1
enum { MPI_BYTE = 1, MPI_INT, MPI_UNSIGNED, MPI_DOUBLE, MPI_FLOAT, MPI_LONG_LONG, MPI_UNSIGNED_LONG_LONG,
       MPI_SHIM_FIRST_USER = 100 };
enum { MPI_SUM = 1, MPI_MAX, MPI_MIN };
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm c, int code);
int MPI_Comm_rank(MPI_Comm c, int *r);
int MPI_Comm_size(MPI_Comm c, int *s);
int MPI_Barrier(MPI_Comm c);
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Allgather(const void *s, int ns, MPI_Datatype ts, void *r, int nr, MPI_Datatype tr, MPI_Comm c);
int MPI_Sendrecv(const void *s, int ns, MPI_Datatype ts, int dest, int stag, void *r, int nr, MPI_Datatype tr,
                 int src, int rtag, MPI_Comm c, MPI_Status *st);
int MPI_Type_match_size(int typeclass, int size, MPI_Datatype *t);
int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *off, const MPI_Datatype *types, MPI_Datatype *t);
int MPI_Type_commit(MPI_Datatype *t);
#endif
