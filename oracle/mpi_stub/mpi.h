/* Single-rank stand-in for <mpi.h>, used only to compile the reference
 * library's own C sources into the CPU oracle (oracle/_ref).
 *
 * Test infrastructure: nothing in the product links this header.
 *
 * With one rank (P = {1,1,1,1}) every halo branch of the reference
 * (qcd_communication.c: `if(lL[b] < L[b])`) is skipped, so point-to-point
 * calls never run; reductions become copies of the local value.
 * Handle types are plain ints (the MPICH convention), which is also the
 * layout the GPU drop-in header assumes for qcd_geometry.
 */
#ifndef ORACLE_MPI_STUB_H
#define ORACLE_MPI_STUB_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

/* a datatype's value is its size in bytes (derived types are never sent) */
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_COMM_WORLD 0
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_MAX_PROCESSOR_NAME 64

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; return code; }
static inline int MPI_Comm_size(MPI_Comm c, int *n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Get_processor_name(char *name, int *len)
{ strcpy(name, "oracle"); *len = 6; return 0; }
static inline int MPI_Bcast(void *buf, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)buf; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Allreduce(const void *in, void *out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{ (void)op; (void)c; if (in != out) memmove(out, in, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Reduce(const void *in, void *out, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{ (void)op; (void)root; (void)c; if (in != out) memmove(out, in, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Type_vector(int n, int bl, int st, MPI_Datatype o, MPI_Datatype *t)
{ (void)n; (void)bl; (void)st; (void)o; *t = 0; return 0; }
static inline int MPI_Type_contiguous(int n, MPI_Datatype o, MPI_Datatype *t)
{ (void)n; (void)o; *t = 0; return 0; }
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; *r = 0; return 0; }
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; *r = 0; return 0; }
static inline int MPI_Waitall(int n, MPI_Request *r, MPI_Status *s) { (void)n; (void)r; (void)s; return 0; }

#endif
