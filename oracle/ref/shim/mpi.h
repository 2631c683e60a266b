/*
 * Stand-in for MPI, used only to compile the reference's host code into the test
 * checker (oracle/_ref).  Two modes:
 *   - one rank (the default): every communicator has one rank, collectives copy the
 *     local contribution to the output, point-to-point calls have no partner;
 *   - several ranks as forked processes (sp_mpi_start, called by the checker's
 *     driver before it forks): ranks meet in a shared memory segment.  Collectives
 *     stage each rank's contribution in its own area between two process-shared
 *     barriers; sends are buffered into the destination's mailbox and receives wait
 *     (bounded) for the matching (communicator, source, tag) message.  Reductions combine the
 *     ranks' contributions in rank order, so every rank gets identical bits.
 * Non-blocking collectives complete at the call.  Test infrastructure only.
 */
#ifndef SP_REF_SHIM_MPI_H
#define SP_REF_SHIM_MPI_H

#include <execinfo.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

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
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)

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

/* ---- state shared by every translation unit (defined in ref_shim.cpp) */
#define SP_MPI_MAXRANKS 16
#define SP_MPI_MAXMSG 8192
#define SP_MPI_MAXREQ 4096

struct sp_mpi_msg { int src, tag, comm, consumed; size_t off, len; };
struct sp_mpi_box { int nmsg, live; size_t used; struct sp_mpi_msg msg[SP_MPI_MAXMSG]; };
struct sp_mpi_world {
  int size;
  pthread_barrier_t bar;
  pthread_mutex_t mtx;
  pthread_cond_t cv;
  size_t area_bytes, box_bytes;
  struct sp_mpi_box box[SP_MPI_MAXRANKS];
  /* then size staging areas, then size mailbox data areas */
};
struct sp_mpi_req { int used, done; long long seq; void* buf; size_t len; int src, tag, comm; };

extern struct sp_mpi_world* sp_mpi_w;   /* NULL: one rank */
extern int sp_mpi_rank;
extern size_t sp_mpi_type_size[4096];
extern int sp_mpi_ntypes;
extern struct sp_mpi_req sp_mpi_reqs[SP_MPI_MAXREQ];
extern int sp_mpi_ncomms; /* communicator ids handed out (the same sequence on every rank) */

/* creates the segment for `size` ranks; call before fork, then sp_mpi_set_rank */
int sp_mpi_start(int size, size_t area_bytes, size_t box_bytes);
void sp_mpi_set_rank(int rank);

static inline size_t sp_mpi_sz(MPI_Datatype t) { return sp_mpi_type_size[t]; }
static inline void sp_mpi_copy(const void* s, void* r, int n, MPI_Datatype t) {
  if (s != MPI_IN_PLACE && n > 0 && s != r) memmove(r, s, (size_t)n * sp_mpi_sz(t));
}
static inline void sp_mpi_die(const char* what) {
  fprintf(stderr, "MPI stand-in (rank %d): %s\n", sp_mpi_rank, what);
  void* bt[32];
  backtrace_symbols_fd(bt, backtrace(bt, 32), 2);
  abort();
}
static inline char* sp_mpi_area(int r) {
  return (char*)(sp_mpi_w + 1) + (size_t)r * sp_mpi_w->area_bytes;
}
static inline char* sp_mpi_boxdata(int r) {
  return (char*)(sp_mpi_w + 1) + (size_t)sp_mpi_w->size * sp_mpi_w->area_bytes +
         (size_t)r * sp_mpi_w->box_bytes;
}
static inline void sp_mpi_barrier(void) { pthread_barrier_wait(&sp_mpi_w->bar); }
/* stages n bytes (plus an optional header) in this rank's area */
static inline void sp_mpi_stage(const void* hdr, size_t hn, const void* data, size_t n) {
  if (hn + n > sp_mpi_w->area_bytes) sp_mpi_die("staging area too small");
  char* a = sp_mpi_area(sp_mpi_rank);
  if (hn) memcpy(a, hdr, hn);
  if (n) memcpy(a + hn, data, n);
}

/* element-wise reduction of one contribution into an accumulator */
#define SP_MPI_RED(T)                                                          \
  do {                                                                         \
    T* x = (T*)acc; const T* y = (const T*)in;                                 \
    for (int i = 0; i < n; ++i) switch (op) {                                  \
        case MPI_MAX: x[i] = x[i] > y[i] ? x[i] : y[i]; break;                 \
        case MPI_MIN: x[i] = x[i] < y[i] ? x[i] : y[i]; break;                 \
        case MPI_SUM: x[i] = x[i] + y[i]; break;                               \
        case MPI_PROD: x[i] = x[i] * y[i]; break;                              \
        case MPI_LAND: x[i] = (x[i] != 0) && (y[i] != 0); break;               \
        case MPI_LOR: x[i] = (x[i] != 0) || (y[i] != 0); break;                \
        default: x[i] = ((x[i] != 0) != (y[i] != 0)); break;                   \
      }                                                                        \
  } while (0)
static inline void sp_mpi_reduce_into(void* acc, const void* in, int n, MPI_Datatype t, MPI_Op op) {
  switch (t) {
    case MPI_CHAR: SP_MPI_RED(char); break;
    case MPI_INT: SP_MPI_RED(int); break;
    case MPI_LONG_LONG_INT: SP_MPI_RED(long long); break;
    case MPI_FLOAT: SP_MPI_RED(float); break;
    case MPI_DOUBLE: SP_MPI_RED(double); break;
    default: sp_mpi_die("reduction on a derived type");
  }
}
#undef SP_MPI_RED
/* ranks lo..hi combined in rank order into out (all staged) */
static inline void sp_mpi_combine(void* out, int lo, int hi, int n, MPI_Datatype t, MPI_Op op) {
  const size_t b = (size_t)n * sp_mpi_sz(t);
  if (b) memcpy(out, sp_mpi_area(lo), b);
  for (int r = lo + 1; r <= hi; ++r) sp_mpi_reduce_into(out, sp_mpi_area(r), n, t, op);
}

static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code); }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = sp_mpi_w ? sp_mpi_rank : 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = sp_mpi_w ? sp_mpi_w->size : 1; return 0; }
static inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* n) { (void)c; *n = ++sp_mpi_ncomms; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* n) {
  (void)c; (void)color; (void)key;
  if (sp_mpi_w) sp_mpi_die("MPI_Comm_split");
  *n = 2; return 0;
}
static inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
static inline int MPI_Comm_delete(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
static inline int MPI_Get_processor_name(char* name, int* len) {
  strcpy(name, "localhost"); *len = 9; return 0;
}
static inline int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype* t) {
  const size_t sz = (size_t)n * sp_mpi_sz(old);
  for (int i = 6; i < sp_mpi_ntypes; ++i)
    if (sp_mpi_type_size[i] == sz) { *t = i; return 0; }
  if (sp_mpi_ntypes >= 4096) sp_mpi_die("too many datatypes");
  sp_mpi_type_size[sp_mpi_ntypes] = sz;
  *t = sp_mpi_ntypes++;
  return 0;
}
static inline int MPI_Type_commit(MPI_Datatype* t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype* t) { (void)t; return 0; }

static inline int MPI_Barrier(MPI_Comm c) { (void)c; if (sp_mpi_w) sp_mpi_barrier(); return 0; }
static inline int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) return 0;
  const size_t bytes = (size_t)n * sp_mpi_sz(t);
  if (sp_mpi_rank == root) sp_mpi_stage(0, 0, b, bytes);
  sp_mpi_barrier();
  if (sp_mpi_rank != root && bytes) memcpy(b, sp_mpi_area(root), bytes);
  sp_mpi_barrier();
  return 0;
}
static inline int sp_mpi_reduce_to(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o,
                                   int root, int scan) {
  const size_t bytes = (size_t)n * sp_mpi_sz(t);
  sp_mpi_stage(0, 0, s == MPI_IN_PLACE ? r : s, bytes);
  sp_mpi_barrier();
  if (scan) sp_mpi_combine(r, 0, sp_mpi_rank, n, t, o);
  else if (root < 0 || sp_mpi_rank == root) sp_mpi_combine(r, 0, sp_mpi_w->size - 1, n, t, o);
  sp_mpi_barrier();
  return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, int root,
                             MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) { if (r) sp_mpi_copy(s, r, n, t); return 0; }
  return sp_mpi_reduce_to(s, r, n, t, o, root, 0);
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o,
                                MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) { sp_mpi_copy(s, r, n, t); return 0; }
  return sp_mpi_reduce_to(s, r, n, t, o, -1, 0);
}
static inline int MPI_Iallreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o,
                                 MPI_Comm c, MPI_Request* q) {
  *q = 0; return MPI_Allreduce(s, r, n, t, o, c);
}
static inline int MPI_Scan(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) { sp_mpi_copy(s, r, n, t); return 0; }
  return sp_mpi_reduce_to(s, r, n, t, o, -1, 1);
}
/* gathers: every rank stages [count][data]; readers copy what they need */
static inline int sp_mpi_gatherv(const void* s, int sn, MPI_Datatype st, void* r, const int* rd,
                                 MPI_Datatype rt, int root) {
  const size_t bytes = (size_t)sn * sp_mpi_sz(st);
  sp_mpi_stage(&bytes, sizeof bytes, s == MPI_IN_PLACE ? (const char*)r + (size_t)rd[sp_mpi_rank] * sp_mpi_sz(rt) : s, bytes);
  sp_mpi_barrier();
  if (root < 0 || sp_mpi_rank == root)
    for (int w = 0; w < sp_mpi_w->size; ++w) {
      size_t nb;
      memcpy(&nb, sp_mpi_area(w), sizeof nb);
      if (nb) memmove((char*)r + (size_t)rd[w] * sp_mpi_sz(rt), sp_mpi_area(w) + sizeof nb, nb);
    }
  sp_mpi_barrier();
  return 0;
}
static inline int MPI_Gather(const void* s, int sn, MPI_Datatype st, void* r, int rn,
                             MPI_Datatype rt, int root, MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) { sp_mpi_copy(s, r, sn, st); return 0; }
  int rd[SP_MPI_MAXRANKS];
  for (int w = 0; w < sp_mpi_w->size; ++w) rd[w] = w * rn;
  return sp_mpi_gatherv(s, sn, st, r, rd, rt, root);
}
static inline int MPI_Gatherv(const void* s, int sn, MPI_Datatype st, void* r, const int* rn,
                              const int* rd, MPI_Datatype rt, int root, MPI_Comm c) {
  (void)rn; (void)c;
  if (!sp_mpi_w) { sp_mpi_copy(s, (char*)r + (size_t)rd[0] * sp_mpi_sz(st), sn, st); return 0; }
  return sp_mpi_gatherv(s, sn, st, r, rd, rt, root);
}
static inline int MPI_Allgather(const void* s, int sn, MPI_Datatype st, void* r, int rn,
                                MPI_Datatype rt, MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) { sp_mpi_copy(s, r, sn, st); return 0; }
  int rd[SP_MPI_MAXRANKS];
  for (int w = 0; w < sp_mpi_w->size; ++w) rd[w] = w * rn;
  return sp_mpi_gatherv(s, sn, st, r, rd, rt, -1);
}
static inline int MPI_Allgatherv(const void* s, int sn, MPI_Datatype st, void* r, const int* rn,
                                 const int* rd, MPI_Datatype rt, MPI_Comm c) {
  (void)rn; (void)c;
  if (!sp_mpi_w) { sp_mpi_copy(s, (char*)r + (size_t)rd[0] * sp_mpi_sz(st), sn, st); return 0; }
  return sp_mpi_gatherv(s, sn, st, r, rd, rt, -1);
}
/* scatters and all-to-alls: the source stages [counts][displs][buffer] */
static inline int sp_mpi_alltoallv(const void* s, const int* sn, const int* sd, MPI_Datatype st,
                                   void* r, const int* rd, MPI_Datatype rt, int root) {
  const int P = sp_mpi_w->size;
  const size_t esz = sp_mpi_sz(st);
  if (root < 0 || sp_mpi_rank == root) {
    int hdr[2 * SP_MPI_MAXRANKS];
    size_t end = 0;
    for (int w = 0; w < P; ++w) {
      hdr[w] = sn[w];
      hdr[P + w] = sd[w];
      const size_t e = (size_t)(sd[w] + sn[w]) * esz;
      if (sn[w] > 0 && e > end) end = e;
    }
    sp_mpi_stage(hdr, sizeof(int) * 2 * P, s, end);
  }
  sp_mpi_barrier();
  for (int w = 0; w < P; ++w) {
    if (root >= 0 && w != root) continue;
    const int* hdr = (const int*)sp_mpi_area(w);
    const int cnt = hdr[sp_mpi_rank], dsp = hdr[P + sp_mpi_rank];
    const char* src = sp_mpi_area(w) + sizeof(int) * 2 * P + (size_t)dsp * esz;
    if (cnt > 0) memmove((char*)r + (size_t)rd[root < 0 ? w : 0] * sp_mpi_sz(rt), src, (size_t)cnt * esz);
  }
  sp_mpi_barrier();
  return 0;
}
static inline int MPI_Scatter(const void* s, int sn, MPI_Datatype st, void* r, int rn,
                              MPI_Datatype rt, int root, MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) { sp_mpi_copy(s, r, rn, rt); return 0; }
  int cnt[SP_MPI_MAXRANKS], dsp[SP_MPI_MAXRANKS], zero = 0;
  for (int w = 0; w < sp_mpi_w->size; ++w) { cnt[w] = sn; dsp[w] = w * sn; }
  return sp_mpi_alltoallv(s, cnt, dsp, st, r, &zero, rt, root);
}
static inline int MPI_Scatterv(const void* s, const int* sn, const int* sd, MPI_Datatype st,
                               void* r, int rn, MPI_Datatype rt, int root, MPI_Comm c) {
  (void)c; (void)st;
  if (!sp_mpi_w) { sp_mpi_copy((const char*)s + (size_t)sd[0] * sp_mpi_sz(rt), r, rn, rt); return 0; }
  int zero = 0;
  return sp_mpi_alltoallv(s, sn, sd, rt, r, &zero, rt, root);
}
static inline int MPI_Alltoall(const void* s, int sn, MPI_Datatype st, void* r, int rn,
                               MPI_Datatype rt, MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) { sp_mpi_copy(s, r, sn, st); return 0; }
  int cnt[SP_MPI_MAXRANKS], dsp[SP_MPI_MAXRANKS], rdsp[SP_MPI_MAXRANKS];
  for (int w = 0; w < sp_mpi_w->size; ++w) { cnt[w] = sn; dsp[w] = w * sn; rdsp[w] = w * rn; }
  return sp_mpi_alltoallv(s, cnt, dsp, st, r, rdsp, rt, -1);
}
static inline int MPI_Alltoallv(const void* s, const int* sn, const int* sd, MPI_Datatype st,
                                void* r, const int* rn, const int* rd, MPI_Datatype rt,
                                MPI_Comm c) {
  (void)rn; (void)c;
  if (!sp_mpi_w) {
    sp_mpi_copy((const char*)s + (size_t)sd[0] * sp_mpi_sz(st),
                (char*)r + (size_t)rd[0] * sp_mpi_sz(st), sn[0], st);
    return 0;
  }
  return sp_mpi_alltoallv(s, sn, sd, st, r, rd, rt, -1);
}
static inline int MPI_Ialltoallv(const void* s, const int* sn, const int* sd, MPI_Datatype st,
                                 void* r, const int* rn, const int* rd, MPI_Datatype rt,
                                 MPI_Comm c, MPI_Request* q) {
  *q = 0; return MPI_Alltoallv(s, sn, sd, st, r, rn, rd, rt, c);
}

/* ---- point to point: buffered sends; MPI's matching order (a message goes to the
 * earliest posted receive that matches it, receives take the earliest arrived
 * matching message); waits are bounded */
static inline void sp_mpi_post(const void* b, size_t len, int dst, int tag, int comm) {
  pthread_mutex_lock(&sp_mpi_w->mtx);
  struct sp_mpi_box* box = &sp_mpi_w->box[dst];
  if (box->nmsg >= SP_MPI_MAXMSG || box->used + len > sp_mpi_w->box_bytes) {
    pthread_mutex_unlock(&sp_mpi_w->mtx);
    sp_mpi_die("mailbox full");
  }
  struct sp_mpi_msg* m = &box->msg[box->nmsg++];
  m->src = sp_mpi_rank; m->tag = tag; m->comm = comm; m->consumed = 0; m->off = box->used; m->len = len;
  if (len) memcpy(sp_mpi_boxdata(dst) + box->used, b, len);
  box->used += (len + 15) & ~(size_t)15;
  box->live++;
  pthread_cond_broadcast(&sp_mpi_w->cv);
  pthread_mutex_unlock(&sp_mpi_w->mtx);
}
static inline int sp_mpi_matches(const struct sp_mpi_msg* m, int src, int tag, int comm) {
  return !m->consumed && m->comm == comm && (src == MPI_ANY_SOURCE || m->src == src) &&
         (tag == MPI_ANY_TAG || m->tag == tag);
}
/* delivers message m into request r (mutex held) */
static inline void sp_mpi_deliver(struct sp_mpi_msg* m, struct sp_mpi_req* r) {
  struct sp_mpi_box* box = &sp_mpi_w->box[sp_mpi_rank];
  if (m->len > r->len) {
    fprintf(stderr, "MPI stand-in (rank %d): message from %d tag %d has %zu bytes, receive %zu\n",
            sp_mpi_rank, m->src, m->tag, m->len, r->len);
    pthread_mutex_unlock(&sp_mpi_w->mtx);
    sp_mpi_die("message too long");
  }
  if (m->len) memcpy(r->buf, sp_mpi_boxdata(sp_mpi_rank) + m->off, m->len);
  m->consumed = 1;
  r->done = 1;
  if (--box->live == 0) { box->nmsg = 0; box->used = 0; }
}
/* hands arrived messages, in arrival order, to the earliest posted matching receive */
static inline void sp_mpi_progress(void) {
  struct sp_mpi_box* box = &sp_mpi_w->box[sp_mpi_rank];
  for (int i = 0; i < box->nmsg; ++i) {
    struct sp_mpi_msg* m = &box->msg[i];
    if (m->consumed) continue;
    struct sp_mpi_req* best = 0;
    for (int q = 1; q < SP_MPI_MAXREQ; ++q) {
      struct sp_mpi_req* r = &sp_mpi_reqs[q];
      if (r->used && !r->done && sp_mpi_matches(m, r->src, r->tag, r->comm) &&
          (!best || r->seq < best->seq))
        best = r;
    }
    if (best) {
      const int n = box->nmsg;
      sp_mpi_deliver(m, best);
      if (box->nmsg != n) return;  /* the mailbox emptied and was reset */
    }
  }
}
static inline int sp_mpi_irecv(void* b, size_t len, int src, int tag, int comm) {
  static long long seq = 0;
  int id = 0;
  for (int i = 1; i < SP_MPI_MAXREQ && !id; ++i)
    if (!sp_mpi_reqs[i].used) id = i;
  if (!id) sp_mpi_die("too many pending receives");
  struct sp_mpi_req* r = &sp_mpi_reqs[id];
  r->used = 1; r->done = 0; r->seq = ++seq; r->buf = b; r->len = len; r->src = src; r->tag = tag;
  r->comm = comm;
  pthread_mutex_lock(&sp_mpi_w->mtx);
  sp_mpi_progress();
  pthread_mutex_unlock(&sp_mpi_w->mtx);
  return id;
}
static inline void sp_mpi_wait(int id) {
  struct sp_mpi_req* r = &sp_mpi_reqs[id];
  struct timespec dl;
  clock_gettime(CLOCK_REALTIME, &dl);
  dl.tv_sec += 60;
  pthread_mutex_lock(&sp_mpi_w->mtx);
  for (;;) {
    sp_mpi_progress();
    if (r->done) break;
    if (pthread_cond_timedwait(&sp_mpi_w->cv, &sp_mpi_w->mtx, &dl) != 0) {
      pthread_mutex_unlock(&sp_mpi_w->mtx);
      sp_mpi_die("receive timed out");
    }
  }
  pthread_mutex_unlock(&sp_mpi_w->mtx);
  r->used = 0;
}
static inline int MPI_Send(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  if (!sp_mpi_w) { if (n > 0) sp_mpi_die("MPI_Send without a partner"); return 0; }
  sp_mpi_post(b, (size_t)n * sp_mpi_sz(t), d, tag, c);
  return 0;
}
static inline int MPI_Recv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c) {
  (void)c;
  if (!sp_mpi_w) { if (n > 0) sp_mpi_die("MPI_Recv without a partner"); return 0; }
  sp_mpi_wait(sp_mpi_irecv(b, (size_t)n * sp_mpi_sz(t), s, tag, c));
  return 0;
}
static inline int MPI_Isend(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c,
                            MPI_Request* q) {
  *q = 0;
  return MPI_Send(b, n, t, d, tag, c);
}
static inline int MPI_Irecv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c,
                            MPI_Request* q) {
  (void)c;
  *q = 0;
  if (!sp_mpi_w) { if (n > 0) sp_mpi_die("MPI_Irecv without a partner"); return 0; }
  *q = sp_mpi_irecv(b, (size_t)n * sp_mpi_sz(t), s, tag, c);
  return 0;
}
static inline int MPI_Wait(MPI_Request* q, MPI_Status* st) {
  (void)st;
  if (*q > 0 && *q < SP_MPI_MAXREQ && sp_mpi_reqs[*q].used) sp_mpi_wait(*q);
  *q = 0;
  return 0;
}
static inline int MPI_Waitall(int n, MPI_Request* q, MPI_Status* s) {
  (void)s;
  for (int i = 0; i < n; ++i) MPI_Wait(&q[i], MPI_STATUS_IGNORE);
  return 0;
}

#endif
