/*
 * Single-rank stand-in for <mpi.h>, used only to compile the reference GCGE
 * sources on a machine without MPI.  Test infrastructure: nothing in the
 * GPU library includes this file.
 *
 * The reference hard-wires OPS_USE_MPI=1 (src/ops_config.h:17).  With one
 * rank every collective it issues is an in-place no-op:
 *   - MPI_Allreduce(MPI_IN_PLACE, ...)   src/ops_multi_vec.c:214-223,
 *                                        src/ops_lin_sol.c:317,365
 *   - MPI_Allgatherv(MPI_IN_PLACE, ...)  src/ops_eig_sol_gcg.c:1171
 *   - MPI_Bcast                          src/ops_eig_sol_gcg.c:1123
 * Derived datatypes and user reduction ops (src/ops.c:266-318) are accepted
 * and ignored.  MPI_Wtime is a monotonic wall clock.
 */
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H

#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef void MPI_User_function(void *, void *, int *, MPI_Datatype *);

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 1
#define MPI_IN_PLACE ((void *)1)
#define MPI_SUCCESS 0

static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t,
                                MPI_Op o, MPI_Comm c)
{ (void)s; (void)r; (void)n; (void)t; (void)o; (void)c; return 0; }
static inline int MPI_Allgatherv(const void *s, int sc, MPI_Datatype st, void *r,
                                 const int *rc, const int *d, MPI_Datatype rt,
                                 MPI_Comm c)
{ (void)s; (void)sc; (void)st; (void)r; (void)rc; (void)d; (void)rt; (void)c; return 0; }
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Type_vector(int n, int bl, int st, MPI_Datatype o, MPI_Datatype *t)
{ (void)n; (void)bl; (void)st; (void)o; *t = 3; return 0; }
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Op_create(MPI_User_function *f, int commute, MPI_Op *o)
{ (void)f; (void)commute; *o = 2; return 0; }
static inline int MPI_Op_free(MPI_Op *o) { (void)o; return 0; }
static inline double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#endif
