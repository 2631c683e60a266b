/*
 * Single-rank stand-in for MPI, used only to compile the reference's host code into
 * the test checker (oracle/_ref).  Every communicator has one rank; collectives copy
 * the local contribution to the output; point-to-point calls have no partner and
 * are never reached at one rank.
 */
#ifndef SP_REF_SHIM_MPI_H
#define SP_REF_SHIM_MPI_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_REQUEST_NULL 0

#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_LONG_LONG_INT 3
#define MPI_FLOAT 4
#define MPI_DOUBLE 5

#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_PROD 4
#define MPI_LAND 5
#define MPI_LOR 6
#define MPI_LXOR 7

/* datatype sizes: the five predefined types, then contiguous derived types */
static size_t sp_mpi_type_size[4096] = {0, 1, 4, 8, 4, 8};
static int sp_mpi_ntypes = 6;
static inline size_t sp_mpi_sz(MPI_Datatype t) { return sp_mpi_type_size[t]; }
static inline void sp_mpi_copy(const void* s, void* r, int n, MPI_Datatype t) {
  if (s != MPI_IN_PLACE && n > 0 && s != r) memmove(r, s, (size_t)n * sp_mpi_sz(t));
}

static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code); }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }
static inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* n) { (void)c; *n = 2; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* n) {
  (void)c; (void)color; (void)key; *n = 2; return 0;
}
static inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
static inline int MPI_Comm_delete(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
static inline int MPI_Get_processor_name(char* name, int* len) {
  strcpy(name, "localhost"); *len = 9; return 0;
}
static inline int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype* t) {
  sp_mpi_type_size[sp_mpi_ntypes] = (size_t)n * sp_mpi_sz(old);
  *t = sp_mpi_ntypes++;
  return 0;
}
static inline int MPI_Type_commit(MPI_Datatype* t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype* t) { (void)t; return 0; }

static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)root; (void)c; return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, int root,
                             MPI_Comm c) {
  (void)o; (void)root; (void)c; if (r) sp_mpi_copy(s, r, n, t); return 0;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o,
                                MPI_Comm c) {
  (void)o; (void)c; sp_mpi_copy(s, r, n, t); return 0;
}
static inline int MPI_Iallreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o,
                                 MPI_Comm c, MPI_Request* q) {
  (void)o; (void)c; sp_mpi_copy(s, r, n, t); *q = 0; return 0;
}
static inline int MPI_Scan(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c) {
  (void)o; (void)c; sp_mpi_copy(s, r, n, t); return 0;
}
static inline int MPI_Gather(const void* s, int sn, MPI_Datatype st, void* r, int rn,
                             MPI_Datatype rt, int root, MPI_Comm c) {
  (void)rn; (void)rt; (void)root; (void)c; sp_mpi_copy(s, r, sn, st); return 0;
}
static inline int MPI_Gatherv(const void* s, int sn, MPI_Datatype st, void* r, const int* rn,
                              const int* rd, MPI_Datatype rt, int root, MPI_Comm c) {
  (void)rn; (void)rt; (void)root; (void)c;
  sp_mpi_copy(s, (char*)r + (size_t)rd[0] * sp_mpi_sz(st), sn, st); return 0;
}
static inline int MPI_Scatter(const void* s, int sn, MPI_Datatype st, void* r, int rn,
                              MPI_Datatype rt, int root, MPI_Comm c) {
  (void)sn; (void)st; (void)root; (void)c; sp_mpi_copy(s, r, rn, rt); return 0;
}
static inline int MPI_Scatterv(const void* s, const int* sn, const int* sd, MPI_Datatype st,
                               void* r, int rn, MPI_Datatype rt, int root, MPI_Comm c) {
  (void)sn; (void)root; (void)c; (void)st;
  sp_mpi_copy((const char*)s + (size_t)sd[0] * sp_mpi_sz(rt), r, rn, rt); return 0;
}
static inline int MPI_Allgather(const void* s, int sn, MPI_Datatype st, void* r, int rn,
                                MPI_Datatype rt, MPI_Comm c) {
  (void)rn; (void)rt; (void)c; sp_mpi_copy(s, r, sn, st); return 0;
}
static inline int MPI_Allgatherv(const void* s, int sn, MPI_Datatype st, void* r, const int* rn,
                                 const int* rd, MPI_Datatype rt, MPI_Comm c) {
  (void)rn; (void)rt; (void)c;
  sp_mpi_copy(s, (char*)r + (size_t)rd[0] * sp_mpi_sz(st), sn, st); return 0;
}
static inline int MPI_Alltoall(const void* s, int sn, MPI_Datatype st, void* r, int rn,
                               MPI_Datatype rt, MPI_Comm c) {
  (void)rn; (void)rt; (void)c; sp_mpi_copy(s, r, sn, st); return 0;
}
static inline int MPI_Alltoallv(const void* s, const int* sn, const int* sd, MPI_Datatype st,
                                void* r, const int* rn, const int* rd, MPI_Datatype rt,
                                MPI_Comm c) {
  (void)rn; (void)rt; (void)c;
  sp_mpi_copy((const char*)s + (size_t)sd[0] * sp_mpi_sz(st),
              (char*)r + (size_t)rd[0] * sp_mpi_sz(st), sn[0], st);
  return 0;
}
static inline int MPI_Ialltoallv(const void* s, const int* sn, const int* sd, MPI_Datatype st,
                                 void* r, const int* rn, const int* rd, MPI_Datatype rt,
                                 MPI_Comm c, MPI_Request* q) {
  *q = 0; return MPI_Alltoallv(s, sn, sd, st, r, rn, rd, rt, c);
}
static inline int sp_mpi_no_partner(const char* f, int n) {
  if (n > 0) { fprintf(stderr, "single-rank MPI stand-in: %s with data\n", f); abort(); }
  return 0;
}
static inline int MPI_Send(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  (void)b; (void)t; (void)d; (void)tag; (void)c; return sp_mpi_no_partner("MPI_Send", n);
}
static inline int MPI_Recv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c) {
  (void)b; (void)t; (void)s; (void)tag; (void)c; return sp_mpi_no_partner("MPI_Recv", n);
}
static inline int MPI_Isend(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c,
                            MPI_Request* q) {
  (void)b; (void)t; (void)d; (void)tag; (void)c; *q = 0; return sp_mpi_no_partner("MPI_Isend", n);
}
static inline int MPI_Irecv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c,
                            MPI_Request* q) {
  (void)b; (void)t; (void)s; (void)tag; (void)c; *q = 0; return sp_mpi_no_partner("MPI_Irecv", n);
}
static inline int MPI_Wait(MPI_Request* q, MPI_Status* s) { (void)q; (void)s; return 0; }
static inline int MPI_Waitall(int n, MPI_Request* q, MPI_Status* s) {
  (void)n; (void)q; (void)s; return 0;
}

#endif
