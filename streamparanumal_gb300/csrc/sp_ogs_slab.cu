// Lane-row slab gathers (kernel 7): each lane combines whole rows in registers.
//
// The kernels of sp_ogs.cu stage a chunk's gathered values in shared memory and
// let one lane per row combine them from there: every entry costs a shared store,
// a shared load, warp syncs and the row loop's bookkeeping, about two warp
// instructions per entry, between one chunk's memory round trip and the next.
// Here the plan lays the rows out so that no staging is needed (build_slabs):
// rows of equal size m run side by side, lane l holding rows (j, l) of the slab
// step by step, and the t-th members of the lanes' rows are neighbouring words of
// the id array.  A lane loads the ids of its rows' members (coalesced), gathers
// the values (up to KB of them in flight per lane), combines each row in its CSR
// order from the op's first step -- the order of ogsOperator.cpp:382-385 and
// ogsKernels.okl:64-67, hence the same bits as every other kernel here -- and
// writes the row result (gather) or stores it back to every member (gather+scatter,
// Sym).  A single-member row's result differs from its value only when the op's
// first step changes the bits (-0 under Add, -Inf and NaN under Max/Min), and only
// then is it stored back.
//
// Persistent warps take slabs s, s + W, s + 2W, ... (W warps in the grid), so the
// slabs in flight at any moment are a window of the walk, as for the chunk
// kernels.  A slab is worked in passes of KB members per lane; the ids of the next
// pass load while the current pass's values are in flight.  Slabs may carry their
// ids as 16-bit element-relative codes (compress_slabs), decoded through a table
// the warp keeps in shared memory, and the in-place gather+scatter may defer a
// pass's stores until the next pass's loads are issued.  Every choice computes the
// same bits.
#include <algorithm>

#include "sp_internal.h"
#include "sp_ogs_ops.cuh"
#include "sp_ogs_plan.h"
#include "sp_ogs_slab.h"

namespace sp {

// Resident CTAs of 256 lanes per SM each kernel shape is compiled for by default:
// 3 for 4-byte values at 8 members per lane, else 2 (the sweeps on GB300 of 1..4
// CTAs per shape; more CTAs spill, or, without spills, lowered the DRAM rate).
template <int BYTES, int KB>
struct SlabCtas {
  static constexpr int value = (BYTES == 4 && KB == 8) ? 3 : 2;
};

// Row steps [j0, j0 + P) of a slab of M-member rows (M, P known at compile time).
template <typename T, int OP, int MODE, int M, int P>
__device__ __forceinline__ void slab_steps(const int32_t* __restrict__ ids,
                                           const int32_t* __restrict__ rows, T* v, T* gv,
                                           int32_t eb, int32_t rb, int nl, int rem, int Re,
                                           int j0, int lane) {
  int32_t col[P * M];
  int32_t row[P];
  T val[P * M];
  bool ok[P];
#pragma unroll
  for (int jj = 0; jj < P; ++jj) {
    const int j = j0 + jj;
    const int w = (j == Re - 1) ? rem : nl;
    ok[jj] = (j < Re) && (lane < w);
    const int32_t* src = ids + eb + j * M * nl + lane;
#pragma unroll
    for (int t = 0; t < M; ++t) col[jj * M + t] = ok[jj] ? __ldg(src + t * w) : 0;
    if (MODE == 1) row[jj] = ok[jj] ? __ldg(rows + rb + j * nl + lane) : 0;
  }
#pragma unroll
  for (int u = 0; u < P * M; ++u)
    if (ok[u / M]) val[u] = v[col[u]];
#pragma unroll
  for (int jj = 0; jj < P; ++jj) {
    if (!ok[jj]) continue;
    T acc = Op<T, OP>::first(val[jj * M]);
#pragma unroll
    for (int t = 1; t < M; ++t) Op<T, OP>::apply(acc, val[jj * M + t]);
    if (MODE == 1) {
      gv[row[jj]] = acc;
    } else if (M == 1) {
      if (!same_bits(acc, val[jj])) v[col[jj]] = acc;
    } else {
#pragma unroll
      for (int t = 0; t < M; ++t) v[col[jj * M + t]] = acc;
    }
  }
}

// Any row size: one row step at a time, the members in batches of KB.  Rows
// without members (gather only) receive the op's identity.  (Sizes other than 1, 2,
// 4 and 8 -- not met on conforming hex boxes -- come through here.)
template <typename T, int OP, int MODE, int KB>
__device__ __forceinline__ void slab_any(const int32_t* __restrict__ ids,
                                      const int32_t* __restrict__ rows, T* v, T* gv, int32_t eb,
                                      int32_t rb, int m, int nl, int rem, int Re, int lane) {
  for (int j = 0; j < Re; ++j) {
    const int w = (j == Re - 1) ? rem : nl;
    const bool ok = lane < w;
    const int32_t* src = ids + eb + j * m * nl + lane;
    T acc = Op<T, OP>::init();
    for (int t0 = 0; t0 < m; t0 += KB) {
      int32_t col[KB];
      T val[KB];
#pragma unroll
      for (int u = 0; u < KB; ++u) col[u] = (ok && t0 + u < m) ? __ldg(src + (t0 + u) * w) : 0;
#pragma unroll
      for (int u = 0; u < KB; ++u)
        if (ok && t0 + u < m) val[u] = v[col[u]];
#pragma unroll
      for (int u = 0; u < KB; ++u)
        if (ok && t0 + u < m) {
          if (t0 + u == 0)
            acc = Op<T, OP>::first(val[u]);
          else
            Op<T, OP>::apply(acc, val[u]);
        }
    }
    if (!ok) continue;
    if (MODE == 1) {
      gv[__ldg(rows + rb + j * nl + lane)] = acc;
    } else if (m == 1) {
      const int32_t c = __ldg(src);
      if (!same_bits(acc, v[c])) v[c] = acc;
    } else {
      for (int t = 0; t < m; ++t) v[__ldg(src + t * w)] = acc;
    }
  }
}

// Row steps per pass of KB members per lane for rows of m members: KB / m when m
// is 1, 2, 4 or 8, else 0 (such slabs take the general path).
template <int KB>
__device__ __forceinline__ int pass_steps(int m) {
  return (m == 1 || m == 2 || m == 4 || m == 8) ? KB / m : 0;
}

// A full pass: P = KB / m row steps from step j0, all of 32 lanes.  Then lane l's
// u-th member id sits 32 u words after its first one whatever m is.
template <int KB>
__device__ __forceinline__ bool pass_full(int4 d, int j0) {
  const int m = d.z, nl = d.w & 255, rem = (d.w >> 8) & 255, Re = d.w >> 16;
  const int P = pass_steps<KB>(m);
  const int nfull = (nl == 32) ? (rem == 32 ? Re : Re - 1) : 0;
  return P > 0 && j0 + P <= nfull;
}

// Combines the KB gathered values of a full pass as rows of M members (M known at
// compile time) and writes them: gv[row] (gather) or every member (gather+scatter).
template <typename T, int OP, int MODE, int M, int KB>
__device__ __forceinline__ void pass_combine(const T (&val)[KB], const int32_t (&cid)[KB],
                                             const int32_t (&rw)[KB], T* v, T* gv) {
  constexpr int P = KB / M;
#pragma unroll
  for (int jj = 0; jj < P; ++jj) {
    T acc = Op<T, OP>::first(val[jj * M]);
#pragma unroll
    for (int t = 1; t < M; ++t) Op<T, OP>::apply(acc, val[jj * M + t]);
    if (MODE == 1) {
      gv[rw[jj]] = acc;
    } else if (M == 1) {
      if (!same_bits(acc, val[jj])) v[cid[jj]] = acc;
    } else {
#pragma unroll
      for (int t = 0; t < M; ++t) v[cid[jj * M + t]] = acc;
    }
  }
}

// The in-place gather+scatter's combine of a full pass with its stores deferred:
// the results and their columns are kept (pval, pcid, mask pm) and stored after the
// next pass's values have been requested.  Columns of different rows never
// coincide, so the later loads cannot see these stores early or late.
template <typename T, int OP, int M, int KB>
__device__ __forceinline__ void pass_defer(const T (&val)[KB], const int32_t (&cid)[KB],
                                           T (&pval)[KB], int32_t (&pcid)[KB], uint32_t& pm) {
  constexpr int P = KB / M;
#pragma unroll
  for (int jj = 0; jj < P; ++jj) {
    T acc = Op<T, OP>::first(val[jj * M]);
#pragma unroll
    for (int t = 1; t < M; ++t) Op<T, OP>::apply(acc, val[jj * M + t]);
#pragma unroll
    for (int t = 0; t < M; ++t) {
      const int u = jj * M + t;
      pval[u] = acc;
      pcid[u] = cid[u];
      if (M > 1 || !same_bits(acc, val[u])) pm |= 1u << u;
    }
  }
}

template <typename T, int KB>
__device__ __forceinline__ void flush_deferred(T* v, const T (&pval)[KB],
                                               const int32_t (&pcid)[KB], uint32_t& pm) {
#pragma unroll
  for (int u = 0; u < KB; ++u)
    if (pm & (1u << u)) v[pcid[u]] = pval[u];
  pm = 0u;
}

// The rest of a slab from step j0 (its last, partial step and any full steps that
// do not fill a pass), or a whole slab of another row size.
template <typename T, int OP, int MODE, int KB>
__device__ __forceinline__ void slab_rest(const int32_t* __restrict__ ids,
                                          const int32_t* __restrict__ rows, T* v, T* gv, int4 d,
                                          int j0, int lane) {
  const int m = d.z, nl = d.w & 255, rem = (d.w >> 8) & 255, Re = d.w >> 16;
  switch (m) {
    case 1: {
      constexpr int PT = KB >= 16 ? 4 : 2;
      for (; j0 < Re; j0 += PT)
        slab_steps<T, OP, MODE, 1, PT>(ids, rows, v, gv, d.x, d.y, nl, rem, Re, j0, lane);
      break;
    }
    case 2: {
      constexpr int PT = KB >= 16 ? 2 : 1;
      for (; j0 < Re; j0 += PT)
        slab_steps<T, OP, MODE, 2, PT>(ids, rows, v, gv, d.x, d.y, nl, rem, Re, j0, lane);
      break;
    }
    case 4:
      for (; j0 < Re; ++j0)
        slab_steps<T, OP, MODE, 4, 1>(ids, rows, v, gv, d.x, d.y, nl, rem, Re, j0, lane);
      break;
    case 8:
      for (; j0 < Re; ++j0)
        slab_steps<T, OP, MODE, 8, 1>(ids, rows, v, gv, d.x, d.y, nl, rem, Re, j0, lane);
      break;
    default:
      slab_any<T, OP, MODE, 4>(ids, rows, v, gv, d.x, d.y, m, nl, rem, Re, lane);
  }
}

// Persistent warps over slabs s, s + W, ...; each slab is a run of passes of KB
// members per lane.  The member ids of a lane's next full pass are loaded while
// the values of the current pass are in flight (one memory round trip per pass),
// the next slab's descriptor one slab ahead.  Row words are loaded beside the
// values they are stored with.
// Value load of a full pass: LD 0 plain (L1 and L2), 1 L2 only (ld.global.cg), 2
// evict-first (ld.global.cs), 3 through the read-only path (ld.global.nc; gathers
// only, whose v the kernel never writes).
template <int LD, int MODE, typename T>
__device__ __forceinline__ T load_val(const T* p) {
  if constexpr (LD == 1) return __ldcg(p);
  else if constexpr (LD == 2) return __ldcs(p);
  else if constexpr (LD == 3 && MODE == 1) return __ldg(p);
  else return *p;
}

// The member ids of a lane's full pass starting at step j of slab e: 32-bit ids, or
// the 16-bit codes of a compressed slab (decoded against its table later).
template <int KB>
__device__ __forceinline__ void load_raw(const int32_t* __restrict__ ids,
                                         const uint16_t* __restrict__ codes, int4 e, int j,
                                         bool coded, int lane, int32_t (&raw)[KB]) {
  const int32_t off = e.x + j * e.z * 32 + lane;
  if (coded) {
#pragma unroll
    for (int u = 0; u < KB; ++u) raw[u] = (int32_t)__ldg(codes + off + 32 * u);
  } else {
#pragma unroll
    for (int u = 0; u < KB; ++u) raw[u] = __ldg(ids + off + 32 * u);
  }
}

// DF = 1 (gather+scatter only): a full pass's stores are issued after the next
// pass's value loads.  With `codes` (ogs.slab_code_shift > 0) the slabs that
// compressed read 16-bit member codes, decoded through their table of high parts,
// which the warp keeps in shared memory (loaded one slab ahead into registers,
// stored when the slab begins); the other slabs read their 32-bit ids.  With
// RC = 1 (gathers with `rcodes`, ogs.slab_row_codes): the full passes of a slab
// whose row words compressed read 16-bit row codes likewise, decoded through the
// slab's row table (at most 32 entries, one per lane), which is prefetched and
// stored with the id table.  With RC = 0 the row words are the 32-bit ones, which
// every plan keeps.
template <typename T, int OP, int MODE, int KB, int CTAS, int LD = 0, int DF = 0, int RC = 0>
__global__ void __launch_bounds__(kOgsThreads, CTAS)
k_ogsl_gather(const int4* __restrict__ slabs, int32_t nslabs, const int32_t* __restrict__ ids,
              const int32_t* __restrict__ rows, T* v, T* gv, const uint16_t* __restrict__ codes,
              const int32_t* __restrict__ tabs, const int2* __restrict__ td, int sh,
              const uint16_t* __restrict__ rcodes, const int32_t* __restrict__ rtabs,
              const int2* __restrict__ rtd) {
  __shared__ int32_t stab[kWarpsPerCta][kSlabCodeTable];
  constexpr bool rcx = RC != 0 && MODE == 1;
  __shared__ int32_t rstab[kWarpsPerCta][rcx ? kSlabRowTable : 1];
  static_assert(kSlabRowTable <= 32, "a row table is one word per lane");
  constexpr bool defer = DF != 0 && MODE == 0;
  constexpr int TPL = kSlabCodeTable / 32;  // table words per lane
  T pval[KB];
  int32_t pcid[KB];
  uint32_t pm = 0u;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t W = gridDim.x * kWarpsPerCta;
  int32_t s = blockIdx.x * kWarpsPerCta + w;
  if (s >= nslabs) return;
  const int4 zero = make_int4(0, 0, 0, 0);
  const int2 plain = make_int2(-1, 0);
  const int32_t mask = (1 << sh) - 1;
  int4 d = __ldg(slabs + s);
  int4 dn = (s + W < nslabs) ? __ldg(slabs + s + W) : zero;
  int2 t = codes ? __ldg(td + s) : plain;
  int2 tn = (codes && s + W < nslabs) ? __ldg(td + s + W) : plain;
  const bool rc = rcx && rcodes != nullptr;
  int2 rt = rc ? __ldg(rtd + s) : plain;
  int2 rtn = (rc && s + W < nslabs) ? __ldg(rtd + s + W) : plain;
  int j0 = 0;
  bool full = pass_full<KB>(d, 0);
  int32_t raw[KB];
  if (full) {
    load_raw<KB>(ids, codes, d, 0, t.y > 0, lane, raw);
    if (t.y > 0) {
#pragma unroll
      for (int i = 0; i < TPL; ++i)
        if (lane + 32 * i < t.y) stab[w][lane + 32 * i] = __ldg(tabs + t.x + lane + 32 * i);
    }
    if (rcx && rt.y > 0 && lane < rt.y) rstab[w][lane] = __ldg(rtabs + rt.x + lane);
    if (t.y > 0 || (rcx && rt.y > 0)) __syncwarp();
  }
  while (true) {
    const int m = d.z, Re = d.w >> 16;
    const int P = pass_steps<KB>(m);
    // the pass after this one: the next steps of this slab, or the next slab
    const bool next_slab = !full || j0 + P >= Re;
    const int4 dx = next_slab ? dn : d;
    const int2 tx = next_slab ? tn : t;
    const int jx = next_slab ? 0 : j0 + P;
    const bool has_next = !next_slab || s + W < nslabs;
    const bool fullx = has_next && pass_full<KB>(dx, jx);
    int32_t nraw[KB];
    int32_t ntab[TPL];
    int32_t nrt = 0;  // this lane's word of the next slab's row table
    if (full) {
      int32_t cid[KB];
      if (t.y > 0) {
#pragma unroll
        for (int u = 0; u < KB; ++u) cid[u] = stab[w][raw[u] >> sh] | (raw[u] & mask);
      } else {
#pragma unroll
        for (int u = 0; u < KB; ++u) cid[u] = raw[u];
      }
      T val[KB];
      int32_t rw[KB];
      const bool rcoded = rcx && rt.y > 0;  // this slab's row words are codes
#pragma unroll
      for (int u = 0; u < KB; ++u) val[u] = load_val<LD, MODE>(v + cid[u]);
      if (MODE == 1) {
        if (rcoded) {
          const uint16_t* rsrc = rcodes + d.y + j0 * 32 + lane;
#pragma unroll
          for (int jj = 0; jj < KB; ++jj)
            if (jj < P) rw[jj] = (int32_t)__ldg(rsrc + 32 * jj);
        } else {
          const int32_t* rsrc = rows + d.y + j0 * 32 + lane;
#pragma unroll
          for (int jj = 0; jj < KB; ++jj)
            if (jj < P) rw[jj] = __ldg(rsrc + 32 * jj);
        }
      }
      if (fullx) {
        load_raw<KB>(ids, codes, dx, jx, tx.y > 0, lane, nraw);
        if (next_slab && tx.y > 0) {
#pragma unroll
          for (int i = 0; i < TPL; ++i)
            if (lane + 32 * i < tx.y) ntab[i] = __ldg(tabs + tx.x + lane + 32 * i);
        }
        if (rcx && next_slab && lane < rtn.y) nrt = __ldg(rtabs + rtn.x + lane);
      }
      if (rcoded) {
#pragma unroll
        for (int jj = 0; jj < KB; ++jj)
          if (jj < P) rw[jj] = rstab[w][rw[jj] >> sh] | (rw[jj] & mask);
      }
      if constexpr (defer) {
        flush_deferred<T, KB>(v, pval, pcid, pm);
        switch (m) {
          case 1: pass_defer<T, OP, 1, KB>(val, cid, pval, pcid, pm); break;
          case 2: pass_defer<T, OP, 2, KB>(val, cid, pval, pcid, pm); break;
          case 4: pass_defer<T, OP, 4, KB>(val, cid, pval, pcid, pm); break;
          default: pass_defer<T, OP, 8, KB>(val, cid, pval, pcid, pm);
        }
      } else {
        switch (m) {
          case 1: pass_combine<T, OP, MODE, 1, KB>(val, cid, rw, v, gv); break;
          case 2: pass_combine<T, OP, MODE, 2, KB>(val, cid, rw, v, gv); break;
          case 4: pass_combine<T, OP, MODE, 4, KB>(val, cid, rw, v, gv); break;
          default: pass_combine<T, OP, MODE, 8, KB>(val, cid, rw, v, gv);
        }
      }
    } else {
      if constexpr (defer) flush_deferred<T, KB>(v, pval, pcid, pm);
      slab_rest<T, OP, MODE, KB>(ids, rows, v, gv, d, j0, lane);
      if (fullx) {
        load_raw<KB>(ids, codes, dx, jx, tx.y > 0, lane, nraw);
        if (next_slab && tx.y > 0) {
#pragma unroll
          for (int i = 0; i < TPL; ++i)
            if (lane + 32 * i < tx.y) ntab[i] = __ldg(tabs + tx.x + lane + 32 * i);
        }
        if (rcx && next_slab && lane < rtn.y) nrt = __ldg(rtabs + rtn.x + lane);
      }
    }
    if (!has_next) break;
    if (next_slab) {
      s += W;
      d = dn;
      t = tn;
      rt = rtn;
      dn = (s + W < nslabs) ? __ldg(slabs + s + W) : zero;
      tn = (codes && s + W < nslabs) ? __ldg(td + s + W) : plain;
      rtn = (rc && s + W < nslabs) ? __ldg(rtd + s + W) : plain;
    }
    j0 = jx;
    full = fullx;
    if (full) {
#pragma unroll
      for (int u = 0; u < KB; ++u) raw[u] = nraw[u];
      const bool id_tab = next_slab && t.y > 0;
      const bool row_tab = rcx && next_slab && rt.y > 0;
      if (id_tab || row_tab) {
        __syncwarp();  // every lane has decoded its last pass against the old tables
        if (id_tab) {
#pragma unroll
          for (int i = 0; i < TPL; ++i)
            if (lane + 32 * i < t.y) stab[w][lane + 32 * i] = ntab[i];
        }
        if (row_tab && lane < rt.y) rstab[w][lane] = nrt;
        __syncwarp();
      }
    }
  }
  if constexpr (defer) flush_deferred<T, KB>(v, pval, pcid, pm);
}

template <typename T, int OP, int MODE, int KB, int CTAS, int LD = 0, int DF = 0, int RC = 0>
static void launch_shape(const SlabArgs& a, T* v, T* gv, cudaStream_t s) {
  const int4* slabs = a.slabs;
  const int32_t nslabs = a.nslabs;
  const int64_t want = ((int64_t)nslabs + kWarpsPerCta - 1) / kWarpsPerCta;
  const int64_t cap = (int64_t)sm_count() * CTAS;
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min(want, cap));
  k_ogsl_gather<T, OP, MODE, KB, CTAS, LD, DF, RC><<<g, kOgsThreads, 0, s>>>(
      slabs, nslabs, a.ids, a.rows, v, gv, a.codes, a.tabs, a.td, a.shift, a.rcodes, a.rtabs,
      a.rtd);
}

// One pass size with the resident CTAs the knob ogs.slab_ctas asks for (Add only;
// 0 = the shape's default).
template <typename T, int OP, int MODE, int KB>
static void launch_ctas(const SlabArgs& a, T* v, T* gv, cudaStream_t s) {
  constexpr int dflt = SlabCtas<(int)sizeof(T), KB>::value;
  // deferred stores (default on): with the 16-bit codes they took the FP64 in-place
  // gather+scatter +5 % and FP32 +14 % on 64^3 p = 7 boxes, p = 15 within +-2 %
  if constexpr (OP == SP_OP_ADD && MODE == 0) {
    if (tune(kTuneOgsSlabDefer) == 1)
      return launch_shape<T, OP, MODE, KB, dflt, 0, 1>(a, v, gv, s);
  }
  if constexpr (OP == SP_OP_ADD) {
    switch (tune(kTuneOgsSlabLoad)) {
      case 1: return launch_shape<T, OP, MODE, KB, dflt, 1>(a, v, gv, s);
      case 2: return launch_shape<T, OP, MODE, KB, dflt, 2>(a, v, gv, s);
      case 3: return launch_shape<T, OP, MODE, KB, dflt, 3>(a, v, gv, s);
      default: break;
    }
    switch (tune(kTuneOgsSlabCtas)) {
      case 1: return launch_shape<T, OP, MODE, KB, 1>(a, v, gv, s);
      case 3: return launch_shape<T, OP, MODE, KB, 3>(a, v, gv, s);
      case 4: return launch_shape<T, OP, MODE, KB, 4>(a, v, gv, s);
      default: break;
    }
  }
  // row codes (plans built with ogs.slab_row_codes): the gather's default shape
  // decodes them; every other shape reads the 32-bit row words
  if constexpr (OP == SP_OP_ADD && MODE == 1 && KB == 8) {
    if (a.rcodes) return launch_shape<T, OP, MODE, KB, dflt, 0, 0, 1>(a, v, gv, s);
  }
  launch_shape<T, OP, MODE, KB, dflt>(a, v, gv, s);
}

// Members in flight per lane and pass: 8, except 16 for the in-place
// gather+scatter of 4-byte values (knob ogs.slab_lane 0; measured on GB300: FP32
// gathers 8 per lane at 3 CTAs per SM +10 % over 16 at 2, the FP32 gather+scatter
// 16 at 2 +3 % over 8 at 3); 8 or 16 when the knob says so.  The other shape is
// compiled for Add, the op the benchmarks time; the other ops run the default.
template <typename T, int OP, int MODE>
void launch_slabs(const SlabArgs& a, T* v, T* gv, cudaStream_t s) {
  if (a.nslabs <= 0) return;
  constexpr int KB = (sizeof(T) == 4 && MODE == 0) ? 16 : 8;
  constexpr int KO = KB == 16 ? 8 : 16;
  if constexpr (OP == SP_OP_ADD) {
    const int64_t lane = tune(kTuneOgsSlabLane);
    if (lane > 0 && (lane <= 8 ? 8 : 16) == KO)
      return launch_ctas<T, OP, MODE, KO>(a, v, gv, s);
  }
  launch_ctas<T, OP, MODE, KB>(a, v, gv, s);
}

#define SP_SLAB_INST(T, OP)                                                   \
  template void launch_slabs<T, OP, 0>(const SlabArgs&, T*, T*, cudaStream_t); \
  template void launch_slabs<T, OP, 1>(const SlabArgs&, T*, T*, cudaStream_t);
#define SP_SLAB_INST_OPS(T) \
  SP_SLAB_INST(T, SP_OP_ADD) SP_SLAB_INST(T, SP_OP_MUL) SP_SLAB_INST(T, SP_OP_MAX) \
  SP_SLAB_INST(T, SP_OP_MIN)
SP_SLAB_INST_OPS(float)
SP_SLAB_INST_OPS(double)
SP_SLAB_INST_OPS(int32_t)
SP_SLAB_INST_OPS(long long)

}  // namespace sp
