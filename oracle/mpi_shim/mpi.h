/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the reference's own
 * sources into the oracle harness (oracle/_ref).  One rank, a 1x1x1 periodic
 * Cartesian grid; the rank's grid coordinates can be set through
 * asg_shim_coords so that the periodic (global) mesh path can be exercised
 * with a non-zero cube offset.  Not part of the product.
 */
#ifndef ASG_MPI_SHIM_H
#define ASG_MPI_SHIM_H

#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int count_bytes; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ERR_TRUNCATE 15
#define MPI_INT 4
#define MPI_FLOAT 4
#define MPI_LONG 8
#define MPI_DOUBLE 8
#define MPI_SUM 0

extern int asg_shim_coords[3];

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* c) { *c = 0; return 0; }
static inline int MPI_Cart_get(MPI_Comm, int nd, int* dims, int* periods, int* coords)
{
    for (int i = 0; i < nd; ++i) { dims[i] = 1; periods[i] = 1; coords[i] = asg_shim_coords[i]; }
    return 0;
}
static inline int MPI_Cart_rank(MPI_Comm, const int*, int* r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); return 0; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    std::memmove(r, s, (size_t)n * (size_t)t);
    return 0;
}
static inline int MPI_Sendrecv(const void* sb, int ns, MPI_Datatype st, int, int, void* rb, int nr,
                               MPI_Datatype rt, int, int, MPI_Comm, MPI_Status* stat)
{
    int nb = ns * st;
    if (nb > nr * rt) return MPI_ERR_TRUNCATE;
    std::memmove(rb, sb, (size_t)nb);
    if (stat) stat->count_bytes = nb;
    return 0;
}
static inline int MPI_Get_count(const MPI_Status* stat, MPI_Datatype t, int* n)
{
    *n = stat->count_bytes / t;
    return 0;
}

#endif
