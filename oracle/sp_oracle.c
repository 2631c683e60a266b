/*
 * sp_oracle.c -- CPU restatement of streamParanumal's streaming hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see sp_oracle.h).  Pinned against the reference's own
 * host code compiled from its sources (oracle/ref/, outputs in tests/golden/).
 */
#include "sp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ BS1..BS5 */

void or_bs1(int64_t n, const double* a, double* b) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) b[i] = a[i];
}

/* y = alpha*x + beta*y.  CUDA mode contracts the first product into the add. */
void or_bs2(int64_t n, double alpha, const double* x, double beta, double* y, int fmad) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const double by = beta * y[i];
    y[i] = fmad ? fma(alpha, x[i], by) : (alpha * x[i] + by);
  }
}

void or_bs2_f32(int64_t n, float alpha, const float* x, float beta, float* y, int fmad) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const float by = beta * y[i];
    y[i] = fmad ? fmaf(alpha, x[i], by) : (alpha * x[i] + by);
  }
}

/* The halving tree of the OKL reduction kernels (bs3.okl:43-63): for h = bs/2 .. 2,
 * s[t] += s[t+h] for t < h (each @inner loop completes before the next one);
 * result s[0] + s[1]. */
static double tree(int bs, double* s) {
  for (int h = bs / 2; h >= 2; h /= 2)
    for (int t = 0; t < h; ++t) s[t] += s[t + h];
  return s[0] + s[1];
}

/* Stage 1 of bs3 (bs3.okl:33-63): lane t of block b sums a[id]^2 for
 * id = t + b*bs, stepping by bs*nblocks. */
void or_bs3_1(int bs, int nblocks, int64_t n, const double* a, double* partial, int fmad) {
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nblocks; ++b) {
    double* s = (double*)malloc(sizeof(double) * bs);
    for (int t = 0; t < bs; ++t) {
      double r = 0.0;
      for (int64_t id = t + (int64_t)b * bs; id < n; id += (int64_t)bs * nblocks)
        r = fmad ? fma(a[id], a[id], r) : r + a[id] * a[id];
      s[t] = r;
    }
    partial[b] = tree(bs, s);
    free(s);
  }
}

/* Stage 1 of bs4 (bs4.okl:34-64). */
void or_bs4_1(int bs, int nblocks, int64_t n, const double* a, const double* bb, double* partial,
              int fmad) {
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nblocks; ++b) {
    double* s = (double*)malloc(sizeof(double) * bs);
    for (int t = 0; t < bs; ++t) {
      double r = 0.0;
      for (int64_t id = t + (int64_t)b * bs; id < n; id += (int64_t)bs * nblocks)
        r = fmad ? fma(a[id], bb[id], r) : r + a[id] * bb[id];
      s[t] = r;
    }
    partial[b] = tree(bs, s);
    free(s);
  }
}

/* Stage 1 of bs5 (bs5.okl:34-66): r = r + alpha*Ap stored, partial sum of r^2. */
void or_bs5_1(int bs, int nblocks, int64_t n, const double* Ap, double alpha, double* r,
              double* partial, int fmad) {
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nblocks; ++b) {
    double* s = (double*)malloc(sizeof(double) * bs);
    for (int t = 0; t < bs; ++t) {
      double acc = 0.0;
      for (int64_t id = t + (int64_t)b * bs; id < n; id += (int64_t)bs * nblocks) {
        const double rr = fmad ? fma(alpha, Ap[id], r[id]) : r[id] + alpha * Ap[id];
        r[id] = rr;
        acc = fmad ? fma(rr, rr, acc) : acc + rr * rr;
      }
      s[t] = acc;
    }
    partial[b] = tree(bs, s);
    free(s);
  }
}

/* Stage 2 (bs3.okl:66-102): lane t takes 0.0 + partial[t] (the stride bs*nblocks
 * is at least nblocks, so one entry per lane), then the same tree. */
void or_finish(int bs, int nblocks, const double* partial, double* out) {
  double* s = (double*)malloc(sizeof(double) * bs);
  for (int t = 0; t < bs; ++t) {
    double r = 0.0;
    for (int64_t id = t; id < nblocks; id += (int64_t)bs * nblocks) r += partial[id];
    s[t] = r;
  }
  out[0] = tree(bs, s);
  free(s);
}

/* ---- double-double accumulation (Dekker/Knuth error-free transformations) */
typedef struct { double hi, lo; } dd;

static dd dd_add_d(dd a, double b) {
  const double s = a.hi + b;
  const double bb = s - a.hi;
  const double e = (a.hi - (s - bb)) + (b - bb);
  const double lo = a.lo + e;
  const double hi = s + lo;
  dd r = {hi, lo - (hi - s)};
  return r;
}

static dd dd_add_prod(dd a, double x, double y) {
  const double p = x * y;
  const double pe = fma(x, y, -p);
  a = dd_add_d(a, p);
  return dd_add_d(a, pe);
}

static dd dd_add(dd a, dd b) {
  a = dd_add_d(a, b.hi);
  return dd_add_d(a, b.lo);
}

double or_dot_dd(int64_t n, const double* a, const double* b) {
  dd total = {0.0, 0.0};
#pragma omp parallel
  {
    dd loc = {0.0, 0.0};
#pragma omp for schedule(static) nowait
    for (int64_t i = 0; i < n; ++i) loc = dd_add_prod(loc, a[i], b[i]);
#pragma omp critical
    total = dd_add(total, loc);
  }
  return total.hi + total.lo;
}

double or_dot_dd_f32(int64_t n, const float* a, const float* b) {
  dd total = {0.0, 0.0};
#pragma omp parallel
  {
    dd loc = {0.0, 0.0};
#pragma omp for schedule(static) nowait
    for (int64_t i = 0; i < n; ++i) loc = dd_add_prod(loc, (double)a[i], (double)b[i]);
#pragma omp critical
    total = dd_add(total, loc);
  }
  return total.hi + total.lo;
}

double or_cg_update(int64_t n, double alpha, const double* p, const double* Ap, double* x,
                    double* r) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    x[i] = fma(alpha, p[i], x[i]);
    r[i] = fma(-alpha, Ap[i], r[i]);
  }
  return or_dot_dd(n, r, r);
}

double or_cg_update_f32(int64_t n, float alpha, const float* p, const float* Ap, float* x,
                        float* r) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    x[i] = fmaf(alpha, p[i], x[i]);
    r[i] = fmaf(-alpha, Ap[i], r[i]);
  }
  return or_dot_dd_f32(n, r, r);
}

/* ------------------------------------------------------------------ inputs */

static uint64_t splitmix64(uint64_t* st) {
  uint64_t z = (*st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

void or_fill_uniform(int64_t n, uint64_t seed, double* x) {
  uint64_t st = seed;
  for (int64_t i = 0; i < n; ++i) {
    const double u = (double)(splitmix64(&st) >> 11) * 0x1.0p-53;
    x[i] = 2.0 * u - 1.0;
  }
}

/* ------------------------------------------------------------------ box mesh ids */

int or_box_hex_ids(int nx, int ny, int nz, int p, uint64_t perm_seed, int64_t* ids) {
  if (nx < 1 || ny < 1 || nz < 1 || p < 1) return 1;
  const int64_t Nq = p + 1, Np = Nq * Nq * Nq, E = (int64_t)nx * ny * nz;
  int64_t* slot = (int64_t*)malloc(sizeof(int64_t) * E);
  for (int64_t e = 0; e < E; ++e) slot[e] = e;
  if (perm_seed) {
    uint64_t st = perm_seed;
    for (int64_t i = E - 1; i > 0; --i) {
      const int64_t j = (int64_t)(splitmix64(&st) % (uint64_t)(i + 1));
      const int64_t t = slot[i];
      slot[i] = slot[j];
      slot[j] = t;
    }
  }
  for (int64_t l = 0; l < E * Np; ++l) ids[l] = 1 + l;  /* meshConnectNodes.cpp:47-54 */
  /* face pairs: element (ex,ey,ez) and its +x/+y/+z neighbour; node (i,j,k) on the
   * shared face.  Both directions are compared, as vmapM/vmapP list every face. */
  int changed = 1;
  while (changed) {
    changed = 0;
    for (int64_t ez = 0; ez < nz; ++ez)
      for (int64_t ey = 0; ey < ny; ++ey)
        for (int64_t ex = 0; ex < nx; ++ex) {
          const int64_t e = ex + ey * nx + ez * nx * ny;
          for (int dir = 0; dir < 3; ++dir) {
            int64_t f;
            if (dir == 0) { if (ex + 1 >= nx) continue; f = e + 1; }
            else if (dir == 1) { if (ey + 1 >= ny) continue; f = e + nx; }
            else { if (ez + 1 >= nz) continue; f = e + (int64_t)nx * ny; }
            for (int64_t b = 0; b < Nq; ++b)
              for (int64_t a = 0; a < Nq; ++a) {
                int64_t nM, nP;
                if (dir == 0) { nM = p + a * Nq + b * Nq * Nq; nP = 0 + a * Nq + b * Nq * Nq; }
                else if (dir == 1) { nM = a + p * Nq + b * Nq * Nq; nP = a + 0 * Nq + b * Nq * Nq; }
                else { nM = a + b * Nq + p * Nq * Nq; nP = a + b * Nq + 0; }
                const int64_t lM = slot[e] * Np + nM, lP = slot[f] * Np + nP;
                if (ids[lP] < ids[lM]) { ids[lM] = ids[lP]; changed = 1; }
                if (ids[lM] < ids[lP]) { ids[lP] = ids[lM]; changed = 1; }
              }
          }
        }
  }
  free(slot);
  return 0;
}

/* ------------------------------------------------------------------ ogs setup */

typedef struct { int64_t key; int32_t pos; } kp;

static int cmp_kp(const void* x, const void* y) {  /* stable by (key, pos) */
  const kp* a = (const kp*)x;
  const kp* b = (const kp*)y;
  if (a->key != b->key) return a->key < b->key ? -1 : 1;
  return (a->pos > b->pos) - (a->pos < b->pos);
}

static int64_t iabs64(int64_t v) { return v < 0 ? -v : v; }

int or_ogs_setup(int32_t N, int64_t* ids, int kind, int unique, int32_t* NrowsT,
                 int32_t* rowStartsT, int32_t* colIdsT, int32_t* NrowsN, int32_t* rowStartsN,
                 int32_t* colIdsN) {
  if ((kind == 0 && unique) || (kind == 2 && unique)) return 1; /* ogsSetup.cpp:113-116 */
  /* compress out zero ids (ogsSetup.cpp:119-137): colIds ascending local index */
  int32_t Nids = 0;
  for (int32_t l = 0; l < N; ++l) Nids += (ids[l] != 0);
  int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (Nids + 1));
  int64_t* base = (int64_t*)malloc(sizeof(int64_t) * (Nids + 1));
  for (int32_t l = 0, m = 0; l < N; ++l)
    if (ids[l] != 0) { col[m] = l; base[m] = ids[l]; ++m; }

  kp* srt = (kp*)malloc(sizeof(kp) * (Nids + 1));
  for (int32_t i = 0; i < Nids; ++i) { srt[i].key = iabs64(base[i]); srt[i].pos = i; }
  qsort(srt, Nids, sizeof(kp), cmp_kp);
  int32_t* goff = (int32_t*)malloc(sizeof(int32_t) * (Nids + 2));
  int32_t ng = 0;
  goff[0] = 0;
  for (int32_t i = 1; i <= Nids; ++i)
    if (i == Nids || srt[i].key != srt[i - 1].key) goff[++ng] = i;

  if (unique) { /* FindSharedGroups at one rank (ogsSetup.cpp:361-382) */
    const uint64_t A = 6364136223846793005ULL;
    uint64_t x = A * (~0ULL ^ 0ULL) + 1ULL;  /* seedRNG(rank=0) */
    for (int32_t g = 0; g < ng; ++g) {
      int32_t v = (int32_t)(uint32_t)x;
      x = A * x + 1ULL;
      if (v < 0) v = (int32_t)(0u - (uint32_t)v);
      const int32_t size = goff[g + 1] - goff[g];
      const int32_t m = v % size;
      for (int32_t i = goff[g]; i < goff[g + 1]; ++i) base[srt[i].pos] = -srt[i].key;
      if (m >= 0) base[srt[goff[g] + m].pos] = srt[goff[g]].key;
    }
    for (int32_t i = 0; i < Nids; ++i) ids[col[i]] = base[i]; /* ogsSetup.cpp:145-147 */
  }

  /* EnumerateGatherGroups (ogsSetup.cpp:492-559): the first member of each group
   * in the stable order marks the group with its sign; rows are numbered over
   * positive marks, then negative marks, each in original order. */
  int32_t* gids = (int32_t*)calloc(Nids + 1, sizeof(int32_t));
  for (int32_t g = 0; g < ng; ++g) {
    int sign = -1;
    for (int32_t i = goff[g]; i < goff[g + 1]; ++i)
      if (base[srt[i].pos] > 0) { sign = 1; break; }
    gids[srt[goff[g]].pos] = sign;
  }
  int32_t NP = 0;
  for (int32_t i = 0; i < Nids; ++i) NP += (gids[i] == 1);
  int32_t* first = (int32_t*)malloc(sizeof(int32_t) * (ng + 1));
  int32_t c = 0;
  for (int32_t i = 0; i < Nids; ++i) if (gids[i] == 1) first[c++] = i;
  for (int32_t i = 0; i < Nids; ++i) if (gids[i] == -1) first[c++] = i;
  for (int32_t n = 0; n < ng; ++n) gids[first[n]] = n;
  for (int32_t g = 0; g < ng; ++g) {
    const int32_t row = gids[srt[goff[g]].pos];
    for (int32_t i = goff[g] + 1; i < goff[g + 1]; ++i) gids[srt[i].pos] = row;
  }

  /* SortByRow (stable) and run-length row starts (ogsSetup.cpp:561-579,
   * ogsOperator.cpp:609-611) */
  int32_t* cnt = (int32_t*)calloc(ng + 1, sizeof(int32_t));
  for (int32_t i = 0; i < Nids; ++i) cnt[gids[i] + 1]++;
  rowStartsT[0] = 0;
  for (int32_t r = 0; r < ng; ++r) rowStartsT[r + 1] = rowStartsT[r] + cnt[r + 1];
  int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * (ng + 1));
  for (int32_t r = 0; r < ng; ++r) fill[r] = rowStartsT[r];
  for (int32_t i = 0; i < Nids; ++i) colIdsT[fill[gids[i]]++] = col[i];
  *NrowsT = ng;

  /* N operator (ogsOperator.cpp:617-643): positive entries only for Signed kinds */
  *NrowsN = NP;
  rowStartsN[0] = 0;
  int32_t nn = 0;
  for (int32_t r = 0; r < NP; ++r) {
    for (int32_t i = rowStartsT[r]; i < rowStartsT[r + 1]; ++i) {
      const int32_t l = colIdsT[i];
      if (kind == 0 || ids[l] > 0) colIdsN[nn++] = l;
    }
    rowStartsN[r + 1] = nn;
  }
  free(col); free(base); free(srt); free(goff); free(gids); free(first); free(cnt); free(fill);
  return 0;
}

/* ------------------------------------------------------------------ ogs host loops */

#define OR_DEF_OPS(T, BIG)                                                         \
  static T init_##T(int op) {                                                      \
    return op == 0 ? (T)0 : op == 1 ? (T)1 : op == 2 ? (T)(-(BIG)) : (T)(BIG);    \
  }                                                                                \
  static T apply_##T(int op, T a, T b) {                                           \
    if (op == 0) return add_##T(a, b);                                             \
    if (op == 1) return mul_##T(a, b);                                             \
    if (op == 2) return (b > a) ? b : a;                                           \
    return (b < a) ? b : a;                                                        \
  }

typedef long long ll;
static float add_float(float a, float b) { return a + b; }
static float mul_float(float a, float b) { return a * b; }
static double add_double(double a, double b) { return a + b; }
static double mul_double(double a, double b) { return a * b; }
static int32_t add_int32_t(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static int32_t mul_int32_t(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
static ll add_ll(ll a, ll b) { return (ll)((unsigned long long)a + (unsigned long long)b); }
static ll mul_ll(ll a, ll b) { return (ll)((unsigned long long)a * (unsigned long long)b); }

OR_DEF_OPS(float, 3.402823466e+38f)
OR_DEF_OPS(double, 1.7976931348623157e+308)
OR_DEF_OPS(int32_t, 2147483647)
OR_DEF_OPS(ll, 9223372036854775807LL)

#define OR_GATHER(T)                                                                \
  do {                                                                              \
    T* g = (T*)gv;                                                                  \
    const T* x = (const T*)v;                                                       \
    _Pragma("omp parallel for schedule(static)")                                    \
    for (int32_t n = 0; n < Nrows; ++n)                                             \
      for (int f = 0; f < k; ++f) {                                                 \
        T val = init_##T(op);                                                       \
        for (int32_t c = rowStarts[n]; c < rowStarts[n + 1]; ++c)                   \
          val = apply_##T(op, val, x[f + (int64_t)colIds[c] * k]);                  \
        g[f + (int64_t)n * k] = val;                                                \
      }                                                                             \
  } while (0)

void or_ogs_gather(int type, int op, int32_t Nrows, const int32_t* rowStarts,
                   const int32_t* colIds, int k, void* gv, const void* v) {
  switch (type) {
    case 0: OR_GATHER(float); break;
    case 1: OR_GATHER(double); break;
    case 2: OR_GATHER(int32_t); break;
    default: OR_GATHER(ll); break;
  }
}

#define OR_SCATTER(T)                                                               \
  do {                                                                              \
    T* x = (T*)v;                                                                   \
    const T* g = (const T*)gv;                                                      \
    _Pragma("omp parallel for schedule(static)")                                    \
    for (int32_t n = 0; n < Nrows; ++n)                                             \
      for (int32_t c = rowStarts[n]; c < rowStarts[n + 1]; ++c)                     \
        for (int f = 0; f < k; ++f) x[f + (int64_t)colIds[c] * k] = g[f + (int64_t)n * k]; \
  } while (0)

void or_ogs_scatter(int type, int32_t Nrows, const int32_t* rowStarts, const int32_t* colIds,
                    int k, void* v, const void* gv) {
  switch (type) {
    case 0: OR_SCATTER(float); break;
    case 1: OR_SCATTER(double); break;
    case 2: OR_SCATTER(int32_t); break;
    default: OR_SCATTER(ll); break;
  }
}

#define OR_GS(T)                                                                    \
  do {                                                                              \
    T* x = (T*)v;                                                                   \
    _Pragma("omp parallel for schedule(static)")                                    \
    for (int32_t n = 0; n < Nrows; ++n)                                             \
      for (int f = 0; f < k; ++f) {                                                 \
        T val = init_##T(op);                                                       \
        for (int32_t c = gRowStarts[n]; c < gRowStarts[n + 1]; ++c)                 \
          val = apply_##T(op, val, x[f + (int64_t)gColIds[c] * k]);                 \
        for (int32_t c = sRowStarts[n]; c < sRowStarts[n + 1]; ++c)                 \
          x[f + (int64_t)sColIds[c] * k] = val;                                     \
      }                                                                             \
  } while (0)

void or_ogs_gather_scatter(int type, int op, int32_t Nrows, const int32_t* gRowStarts,
                           const int32_t* gColIds, const int32_t* sRowStarts,
                           const int32_t* sColIds, int k, void* v) {
  switch (type) {
    case 0: OR_GS(float); break;
    case 1: OR_GS(double); break;
    case 2: OR_GS(int32_t); break;
    default: OR_GS(ll); break;
  }
}
