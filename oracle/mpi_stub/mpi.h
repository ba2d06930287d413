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

/* Single-rank MPI-IO, enough for the reference's file readers (qcd_io.c).
 * With one rank every subarray type covers the whole array, so a file view
 * is contiguous from its displacement: a view keeps the displacement and the
 * elementary type's size (offsets of *_at calls count elementary types), and
 * the individual file pointer is the stdio position. */
#include <stdio.h>
#include <stdlib.h>

typedef long long MPI_Offset;
typedef int MPI_Info;
typedef struct oracle_mpi_file { FILE *f; MPI_Offset disp; int esize; } *MPI_File;

#define MPI_BYTE 1
#define MPI_FLOAT 4
#define MPI_LONG 8
#define MPI_INFO_NULL 0
#define MPI_ORDER_C 56
#define MPI_MODE_CREATE 1
#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4

static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Type_create_subarray(int nd, const int *sizes, const int *lsizes, const int *starts,
                                           int order, MPI_Datatype old, MPI_Datatype *t)
{ (void)nd; (void)sizes; (void)lsizes; (void)starts; (void)order; *t = old; return 0; }
static inline int MPI_File_open(MPI_Comm c, const char *name, int mode, MPI_Info info, MPI_File *fh)
{
  (void)c; (void)info;
  FILE *f = NULL;
  if (mode & MPI_MODE_RDONLY) f = fopen(name, "rb");
  else { f = fopen(name, "r+b"); if (!f && (mode & MPI_MODE_CREATE)) f = fopen(name, "w+b"); }
  *fh = NULL;
  if (!f) return 1;
  *fh = (MPI_File)calloc(1, sizeof(**fh));
  (*fh)->f = f;
  (*fh)->esize = 1;
  return 0;
}
static inline int MPI_File_close(MPI_File *fh)
{ if (*fh) { fclose((*fh)->f); free(*fh); *fh = NULL; } return 0; }
static inline int MPI_File_sync(MPI_File fh) { return fh ? fflush(fh->f) : 1; }
static inline int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype e, MPI_Datatype ft,
                                    const char *rep, MPI_Info info)
{
  (void)ft; (void)rep; (void)info;
  if (!fh) return 1;
  fh->disp = disp;
  fh->esize = e;
  return fseeko(fh->f, (off_t)disp, SEEK_SET);
}
static inline int MPI_File_read_all(MPI_File fh, void *buf, int n, MPI_Datatype t, MPI_Status *s)
{ (void)s; return fh && fread(buf, (size_t)t, (size_t)n, fh->f) == (size_t)n ? 0 : 1; }
static inline int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void *buf, int n, MPI_Datatype t, MPI_Status *s)
{
  if (!fh || fseeko(fh->f, (off_t)(fh->disp + off * fh->esize), SEEK_SET)) return 1;
  return MPI_File_read_all(fh, buf, n, t, s);
}
static inline int MPI_File_write_all(MPI_File fh, const void *buf, int n, MPI_Datatype t, MPI_Status *s)
{ (void)s; return fh && fwrite(buf, (size_t)t, (size_t)n, fh->f) == (size_t)n ? 0 : 1; }
static inline int MPI_File_write(MPI_File fh, const void *buf, int n, MPI_Datatype t, MPI_Status *s)
{ return MPI_File_write_all(fh, buf, n, t, s); }

#endif
