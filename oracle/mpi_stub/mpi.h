/*
 * Single-rank MPI shim used ONLY to compile the reference's C sources into the
 * oracle (oracle/_ref).  Test infrastructure: nothing in the product links it.
 *
 * Semantics are those of one process in MPI_COMM_WORLD:
 *   - size 1, rank 0; MPI_Dims_create gives {1,1}; Cart coords {0,0};
 *   - MPI_Cart_shift returns MPI_PROC_NULL on both sides (fixed boundaries,
 *     period {0,0} as the reference requests in mpiTM_UPML.c:723);
 *   - point-to-point calls whose peer is MPI_PROC_NULL complete at once and
 *     move no data, which is what MPI specifies for MPI_PROC_NULL.  The halo
 *     cells of the one sub-domain therefore stay zero (PEC outside the PML).
 *   - Send/Recv to a real peer cannot occur with one rank; they abort loudly.
 */
#ifndef ORACLE_MPI_STUB_H
#define ORACLE_MPI_STUB_H
#include <stdio.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
#define MPI_SUCCESS 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_C_DOUBLE_COMPLEX 3

static inline void oracle_mpi_abort_(const char *what)
{
  fprintf(stderr, "oracle mpi shim: %s with a real peer is impossible with one rank\n", what);
  abort();
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Dims_create(int n, int nd, int *dims)
{
  for (int d = 0; d < nd; d++) if (dims[d] == 0) dims[d] = 1;
  (void)n; return 0;
}
static inline int MPI_Cart_create(MPI_Comm old, int nd, const int *dims, const int *period, int reorder, MPI_Comm *c)
{ (void)old; (void)nd; (void)dims; (void)period; (void)reorder; *c = 0; return 0; }
static inline int MPI_Cart_shift(MPI_Comm c, int dir, int disp, int *src, int *dst)
{ (void)c; (void)dir; (void)disp; *src = MPI_PROC_NULL; *dst = MPI_PROC_NULL; return 0; }
static inline int MPI_Cart_coords(MPI_Comm c, int rank, int nd, int *coords)
{ (void)c; (void)rank; for (int d = 0; d < nd; d++) coords[d] = 0; return 0; }
static inline int MPI_Type_vector(int cnt, int bl, int stride, MPI_Datatype old, MPI_Datatype *t)
{ (void)cnt; (void)bl; (void)stride; (void)old; *t = 100; return 0; }
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)tag; (void)c; *r = 0; if (dst != MPI_PROC_NULL) oracle_mpi_abort_("MPI_Isend"); return 0; }
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)tag; (void)c; *r = 0; if (src != MPI_PROC_NULL) oracle_mpi_abort_("MPI_Irecv"); return 0; }
static inline int MPI_Wait(MPI_Request *r, MPI_Status *s) { (void)r; (void)s; return 0; }
static inline int MPI_Sendrecv(const void *sb, int sn, MPI_Datatype st, int dst, int stag,
                               void *rb, int rn, MPI_Datatype rt, int src, int rtag, MPI_Comm c, MPI_Status *s)
{
  (void)sb; (void)sn; (void)st; (void)stag; (void)rb; (void)rn; (void)rt; (void)rtag; (void)c; (void)s;
  if (dst != MPI_PROC_NULL || src != MPI_PROC_NULL) oracle_mpi_abort_("MPI_Sendrecv");
  return 0;
}
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)dst; (void)tag; (void)c; oracle_mpi_abort_("MPI_Send"); return 0; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *s)
{ (void)b; (void)n; (void)t; (void)src; (void)tag; (void)c; (void)s; oracle_mpi_abort_("MPI_Recv"); return 0; }

#endif
