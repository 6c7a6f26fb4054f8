/*
 * Single-rank MPI stand-in used ONLY to compile the reference program
 * (the C files of UVaTRMM/src) as a CPU checker.  It is test infrastructure: nothing in
 * the product links it.
 *
 * With one rank every point-to-point call in the reference's broadcast relay
 * is skipped (UVaTRMM/src/mm_triangular.c:186 guards them with
 * `mpi_procs > 1`), derived datatypes only need a handle, and MPI_Reduce is a
 * copy of the send buffer (UVaTRMM/src/mm_triangular.c:423-424 and
 * UVaTRMM/src/mm_triangular_common.c:2972-2980 reduce MPI_DOUBLE only).
 */
#ifndef UVATRMM_ORACLE_MPI_STUB_H
#define UVATRMM_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_REQUEST_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_MAX_PROCESSOR_NAME 256

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; fflush(stdout); exit(code); }
static inline int MPI_Error_string(int code, char *msg, int *len) {
  *len = snprintf(msg, 64, "mpi stub error %d", code); return 0;
}
static inline int MPI_Get_processor_name(char *name, int *len) {
  strcpy(name, "local"); *len = 5; return 0;
}
static inline int mpi_stub_type_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 4; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  (void)op; (void)root; (void)c;
  memmove(r, s, (size_t)n * (size_t)mpi_stub_type_size(t));
  return 0;
}
/* Datatype constructors: a handle is all the single-rank path needs. */
static inline int MPI_Type_vector(int n, int bl, int st, MPI_Datatype old, MPI_Datatype *t) {
  (void)n; (void)bl; (void)st; (void)old; *t = 100; return 0;
}
static inline int MPI_Type_indexed(int n, const int *bl, const int *d, MPI_Datatype old, MPI_Datatype *t) {
  (void)n; (void)bl; (void)d; (void)old; *t = 101; return 0;
}
static inline int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *d, const MPI_Datatype *ts, MPI_Datatype *t) {
  (void)n; (void)bl; (void)d; (void)ts; *t = 102; return 0;
}
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { *t = 0; return 0; }
/* Point-to-point and collectives are unreachable with one rank. */
static inline int mpi_stub_unreachable(const char *what) {
  fprintf(stderr, "mpi stub: %s called with one rank\n", what); exit(97);
}
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return mpi_stub_unreachable("MPI_Send");
}
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st) {
  (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return mpi_stub_unreachable("MPI_Recv");
}
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r) {
  (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)r; return mpi_stub_unreachable("MPI_Isend");
}
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *r) {
  (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)r; return mpi_stub_unreachable("MPI_Irecv");
}
static inline int MPI_Ibcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c, MPI_Request *r) {
  (void)b; (void)n; (void)t; (void)root; (void)c; (void)r; return mpi_stub_unreachable("MPI_Ibcast");
}
static inline int MPI_Wait(MPI_Request *r, MPI_Status *s) { (void)r; (void)s; return 0; }
static inline int MPI_Waitall(int n, MPI_Request *r, MPI_Status *s) { (void)n; (void)r; (void)s; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm *out) {
  (void)color; (void)key; *out = c; return 0;
}

#endif
