// ogs gather / scatter / gather+scatter kernels and plan construction (sm_103a).
//
// Work decomposition: the rows of a CSR operator are cut into blocks of at most
// kOgsBlockNnz non-zeros.  One CTA of 256 lanes owns one block:
//   1. each lane loads up to 8 column ids of the block (coalesced) and issues the
//      8 gathers of v ahead of use, staging the values in shared memory;
//   2. one lane per row combines its values in CSR order, starting from the op's
//      identity -- the same order as the reference (ogsKernels.okl:64-67,
//      ogsOperator.cpp:382-385), hence bit-identical sums;
//   3. the row results are written back coalesced (gather: by row; scatter and
//      gather+scatter: by column slot, with the column ids still in registers).
// Every column belongs to exactly one row, so in-place gather+scatter has no
// cross-CTA hazard.
#include <algorithm>
#include <cstring>
#include <limits>
#include <type_traits>
#include <vector>

#include "sp_ogs_ops.cuh"
#include "sp_ogs_plan.h"
#include "sp_ogs_slab.h"

namespace sp {

// ------------------------------------------------------------------ kernels

// Stage the block's gathered values: s[i] = v[k + col(g0+i)*K] for i < gn.
// Lane-strided so that both the id loads and the shared stores are coalesced;
// the column ids stay in registers for a later in-place scatter.
template <typename T>
__device__ __forceinline__ void stage_values(const int32_t* __restrict__ ids, int32_t g0,
                                             int32_t gn, const T* __restrict__ v, int k, int K,
                                             T* s, int32_t (&col)[kOgsPerLane]) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int j = 0; j < kOgsPerLane; ++j) {
    const int i = tid + j * kOgsThreads;
    col[j] = (i < gn) ? __ldg(ids + g0 + i) : 0;
  }
  T val[kOgsPerLane];
#pragma unroll
  for (int j = 0; j < kOgsPerLane; ++j) {
    const int i = tid + j * kOgsThreads;
    if (i < gn) val[j] = v[k + (int64_t)col[j] * K];
  }
#pragma unroll
  for (int j = 0; j < kOgsPerLane; ++j) {
    const int i = tid + j * kOgsThreads;
    if (i < gn) s[i] = val[j];
  }
}

// Gather+scatter with the same operator for both halves (ogs::Sym).
template <typename T, int OP>
__global__ void __launch_bounds__(kOgsThreads)
k_ogs_gs_sym(const int32_t* __restrict__ blocks, const int32_t* __restrict__ rs,
             const int32_t* __restrict__ ids, T* __restrict__ v, int K) {
  __shared__ T s[kOgsBlockNnz];
  const int k = blockIdx.y;
  const int32_t r0 = __ldg(blocks + blockIdx.x), r1 = __ldg(blocks + blockIdx.x + 1);
  const int32_t g0 = __ldg(rs + r0), gn = __ldg(rs + r1) - g0;
  int32_t col[kOgsPerLane];
  stage_values<T>(ids, g0, gn, v, k, K, s, col);
  __syncthreads();
  for (int32_t row = r0 + threadIdx.x; row < r1; row += kOgsThreads) {
    const int32_t a = __ldg(rs + row) - g0, b = __ldg(rs + row + 1) - g0;
    T acc = row_combine<T, OP>(s, a, b);
    for (int32_t i = a; i < b; ++i) s[i] = acc;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kOgsPerLane; ++j) {
    const int i = threadIdx.x + j * kOgsThreads;
    if (i < gn) v[k + (int64_t)col[j] * K] = s[i];
  }
}

// Gather+scatter with different gather (gS/gI) and scatter (sS/sI) operators
// (ogs::NoTrans: N then T; ogs::Trans: T then N).  Blocks partition T rows.
template <typename T, int OP>
__global__ void __launch_bounds__(kOgsThreads)
k_ogs_gs_gen(const int32_t* __restrict__ blocks, const int32_t* __restrict__ gS,
             const int32_t* __restrict__ gI, const int32_t* __restrict__ sS,
             const int32_t* __restrict__ sI, T* __restrict__ v, int K) {
  __shared__ T s_in[kOgsBlockNnz];
  __shared__ T s_out[kOgsBlockNnz];
  const int k = blockIdx.y;
  const int32_t r0 = __ldg(blocks + blockIdx.x), r1 = __ldg(blocks + blockIdx.x + 1);
  const int32_t g0 = __ldg(gS + r0), gn = __ldg(gS + r1) - g0;
  const int32_t s0 = __ldg(sS + r0), sn = __ldg(sS + r1) - s0;
  int32_t col[kOgsPerLane];
  stage_values<T>(gI, g0, gn, v, k, K, s_in, col);
  __syncthreads();
  for (int32_t row = r0 + threadIdx.x; row < r1; row += kOgsThreads) {
    const int32_t a = __ldg(gS + row) - g0, b = __ldg(gS + row + 1) - g0;
    T acc = row_combine<T, OP>(s_in, a, b);
    const int32_t c = __ldg(sS + row) - s0, d = __ldg(sS + row + 1) - s0;
    for (int32_t i = c; i < d; ++i) s_out[i] = acc;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kOgsPerLane; ++j) {
    const int i = threadIdx.x + j * kOgsThreads;
    if (i < sn) v[k + (int64_t)__ldg(sI + s0 + i) * K] = s_out[i];
  }
}

template <typename T, int OP>
__global__ void __launch_bounds__(kOgsThreads)
k_ogs_gather(const int32_t* __restrict__ blocks, const int32_t* __restrict__ rs,
             const int32_t* __restrict__ ids, const T* __restrict__ v, T* __restrict__ gv, int K) {
  __shared__ T s[kOgsBlockNnz];
  const int k = blockIdx.y;
  const int32_t r0 = __ldg(blocks + blockIdx.x), r1 = __ldg(blocks + blockIdx.x + 1);
  const int32_t g0 = __ldg(rs + r0), gn = __ldg(rs + r1) - g0;
  int32_t col[kOgsPerLane];
  stage_values<T>(ids, g0, gn, v, k, K, s, col);
  __syncthreads();
  for (int32_t row = r0 + threadIdx.x; row < r1; row += kOgsThreads) {
    const int32_t a = __ldg(rs + row) - g0, b = __ldg(rs + row + 1) - g0;
    T acc = row_combine<T, OP>(s, a, b);
    gv[k + (int64_t)row * K] = acc;
  }
}

template <typename T>
__global__ void __launch_bounds__(kOgsThreads)
k_ogs_scatter(const int32_t* __restrict__ blocks, const int32_t* __restrict__ rs,
              const int32_t* __restrict__ ids, const T* __restrict__ gv, T* __restrict__ v, int K) {
  __shared__ T s[kOgsBlockNnz];
  const int k = blockIdx.y;
  const int32_t r0 = __ldg(blocks + blockIdx.x), r1 = __ldg(blocks + blockIdx.x + 1);
  const int32_t s0 = __ldg(rs + r0), sn = __ldg(rs + r1) - s0;
  for (int32_t row = r0 + threadIdx.x; row < r1; row += kOgsThreads) {
    const T x = gv[k + (int64_t)row * K];
    const int32_t a = __ldg(rs + row) - s0, b = __ldg(rs + row + 1) - s0;
    for (int32_t i = a; i < b; ++i) s[i] = x;
  }
  __syncthreads();
  int32_t col[kOgsPerLane];
#pragma unroll
  for (int j = 0; j < kOgsPerLane; ++j) {
    const int i = threadIdx.x + j * kOgsThreads;
    col[j] = (i < sn) ? __ldg(ids + s0 + i) : 0;
  }
#pragma unroll
  for (int j = 0; j < kOgsPerLane; ++j) {
    const int i = threadIdx.x + j * kOgsThreads;
    if (i < sn) v[k + (int64_t)col[j] * K] = s[i];
  }
}

// ------------------------------------------------------------------ warp-chunk kernels (k == 1)
//
// One warp per chunk of at most 256 non-zeros (a contiguous row range, see
// sp_ogs_order.cpp).  Each lane loads 8 column ids and issues its 8 gathers before
// using any of them; the values and the chunk's row bounds go to the warp's own
// slice of shared memory; one lane per row combines in CSR order; results go back
// coalesced.  Only __syncwarp separates the phases, so warps advance
// independently and the SM keeps many chunks' loads in flight.
//
// Rows inside a chunk are processed either in CSR order (`grouped` = 0: `rs` is the
// CSR row-start array, `ids` the CSR column ids) or grouped by size (`grouped` = 1:
// `rs` holds build_grouped's packed words and `ids` the regrouped column ids).  In
// both cases a row's members are combined in their CSR order, so the results are
// the same bits; grouping only makes the 32 rows a warp runs side by side equally
// long.  Descriptors are (r0, r1, g0, g1): rows [r0, r1), entries [g0, g1).

template <typename T>
struct WarpSmem {
  T val[kWarpsPerCta][kWarpChunkNnz];
  int32_t rs[kWarpsPerCta][kWarpChunkNnz + 8];
  uint8_t ro[kWarpsPerCta][kWarpChunkNnz];
};

// Row r of chunk d (r < nr = d.y - d.x): its members are entries [a, b) of the
// chunk and its row index is d.x + row.
struct RowRef {
  int32_t a, b, row;
};

// srs[r] (r <= nr): first entry of the r-th processed row relative to g0;
// sro[r]: that row's offset from r0 (grouped order only).
__device__ __forceinline__ void stage_rows(const int32_t* __restrict__ rs, int grouped, int4 d,
                                           int lane, int32_t* srs, uint8_t* sro) {
  const int32_t nr = d.y - d.x;
  if (grouped) {
    for (int32_t r = lane; r < nr; r += 32) {
      const int32_t w = __ldg(rs + d.x + r);
      srs[r] = w & 0xFFFF;
      sro[r] = (uint8_t)(w >> 16);
    }
    if (lane == 0) srs[nr] = d.w - d.z;
  } else {
    for (int32_t r = lane; r <= nr; r += 32) srs[r] = __ldg(rs + d.x + r) - d.z;
  }
}

__device__ __forceinline__ RowRef staged_row(const int32_t* srs, const uint8_t* sro, int grouped,
                                             int32_t r) {
  return RowRef{srs[r], srs[r + 1], grouped ? (int32_t)sro[r] : r};
}

// Row r read straight from global memory (scatter kernels, which stage no values).
__device__ __forceinline__ RowRef global_row(const int32_t* __restrict__ rs, int grouped, int4 d,
                                             int32_t r) {
  if (grouped) {
    const int32_t w = __ldg(rs + d.x + r);
    const int32_t b = (r + 1 < d.y - d.x) ? (__ldg(rs + d.x + r + 1) & 0xFFFF) : d.w - d.z;
    return RowRef{w & 0xFFFF, b, w >> 16};
  }
  return RowRef{__ldg(rs + d.x + r) - d.z, __ldg(rs + d.x + r + 1) - d.z, r};
}

// Row of the operator for walk row w: the walk is renumbered only under chunk order
// 2 (PERM = 1); otherwise no lookup is compiled in.
template <int PERM>
__device__ __forceinline__ int32_t op_row(const int32_t* __restrict__ perm, int32_t w) {
  if constexpr (PERM != 0) return __ldg(perm + w);
  return w;
}

template <typename T>
__device__ __forceinline__ void warp_stage(const int32_t* __restrict__ ids, int32_t g0, int32_t gn,
                                           const T* v, T* sv, int lane,
                                           int32_t (&col)[kOgsPerLane]) {
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u) {
    const int i = lane + 32 * u;
    col[u] = (i < gn) ? __ldg(ids + g0 + i) : 0;
  }
  T val[kOgsPerLane];
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u)
    if (lane + 32 * u < gn) val[u] = v[col[u]];
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u)
    if (lane + 32 * u < gn) sv[lane + 32 * u] = val[u];
}

template <typename T, int OP>
__global__ void __launch_bounds__(kOgsThreads, 6)
k_ogsw_gs_sym(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ rs,
              const int32_t* __restrict__ ids, T* __restrict__ v, int grouped) {
  __shared__ WarpSmem<T> sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;
  const int4 ch = __ldg(chunks + c);
  const int32_t nr = ch.y - ch.x, gn = ch.w - ch.z;
  T* sv = sm.val[w];
  int32_t* srs = sm.rs[w];
  stage_rows(rs, grouped, ch, lane, srs, sm.ro[w]);
  int32_t col[kOgsPerLane];
  warp_stage<T>(ids, ch.z, gn, v, sv, lane, col);
  __syncwarp();
  for (int32_t r = lane; r < nr; r += 32) {
    const int32_t a = srs[r], b = srs[r + 1];
    T acc = row_combine<T, OP>(sv, a, b);
    for (int32_t i = a; i < b; ++i) sv[i] = acc;
  }
  __syncwarp();
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u)
    if (lane + 32 * u < gn) v[col[u]] = sv[lane + 32 * u];
}

template <typename T, int OP, int PERM = 0>
__global__ void __launch_bounds__(kOgsThreads)
k_ogsw_gather(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ rs,
              const int32_t* __restrict__ ids, const T* __restrict__ v, T* __restrict__ gv,
              int grouped, const int32_t* __restrict__ perm) {
  __shared__ WarpSmem<T> sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;
  const int4 ch = __ldg(chunks + c);
  const int32_t nr = ch.y - ch.x, gn = ch.w - ch.z;
  T* sv = sm.val[w];
  stage_rows(rs, grouped, ch, lane, sm.rs[w], sm.ro[w]);
  int32_t col[kOgsPerLane];
  warp_stage<T>(ids, ch.z, gn, v, sv, lane, col);
  __syncwarp();
  for (int32_t r = lane; r < nr; r += 32) {
    const RowRef q = staged_row(sm.rs[w], sm.ro[w], grouped, r);
    gv[op_row<PERM>(perm, ch.x + q.row)] = row_combine<T, OP>(sv, q.a, q.b);
  }
}

template <typename T, int PERM = 0>
__global__ void __launch_bounds__(kOgsThreads)
k_ogsw_scatter(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ rs,
               const int32_t* __restrict__ ids, const T* __restrict__ gv, T* __restrict__ v,
               int grouped, const int32_t* __restrict__ perm) {
  __shared__ WarpSmem<T> sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;
  const int4 ch = __ldg(chunks + c);
  const int32_t nr = ch.y - ch.x, sn = ch.w - ch.z;
  T* sv = sm.val[w];
  int32_t col[kOgsPerLane];
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u) {
    const int i = lane + 32 * u;
    col[u] = (i < sn) ? __ldg(ids + ch.z + i) : 0;
  }
  for (int32_t r = lane; r < nr; r += 32) {
    const RowRef q = global_row(rs, grouped, ch, r);
    const T x = gv[op_row<PERM>(perm, ch.x + q.row)];
    for (int32_t i = q.a; i < q.b; ++i) sv[i] = x;
  }
  __syncwarp();
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u)
    if (lane + 32 * u < sn) v[col[u]] = sv[lane + 32 * u];
}

// Persistent, software-pipelined variants (one warp walks chunks c, c+W, c+2W, ...):
// the descriptor of chunk c+2W and the column ids of chunk c+W are loaded while
// chunk c's gathers are in flight, so each chunk costs about one dependent memory
// round trip instead of four.  Results are identical (same rows, same order).
__device__ __forceinline__ void load_cols(const int32_t* __restrict__ ids, int4 d, int lane,
                                          int32_t (&col)[kOgsPerLane]) {
  const int32_t gn = d.w - d.z;
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u) {
    const int i = lane + 32 * u;
    col[u] = (i < gn) ? __ldg(ids + d.z + i) : 0;
  }
}

// L2 prefetch of one element (a hint: no register, no scoreboard entry).
__device__ __forceinline__ void prefetch_elem_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}


// PF = 1 (kernel 5): as soon as this chunk's values have landed, the next chunk's
// values are prefetched into L2 from the column ids already in registers, so
// they stream in while this chunk is combined and written back.
// SG = 1 (grouped rows with the plan's singleton split, knob ogs.singles; the
// dispatch uses it for the in-place gather+scatter): the rows of one member -- the
// chunk's last rows, since grouped rows run largest first -- skip the staging and
// the combine loop: the lane that gathered such a row's value applies the op's
// first step to it (first(x), e.g. 0 + x) and stores it back only when its bits
// changed (-0 under Add, -Inf and NaN under Max), so the memory ends the same and
// the unchanged values are not rewritten.  (A gather through this path writes
// each single-member row from the lane that gathered it; the row word it needs then
// waits on the gather, which measured slower than the staged path.)
// sing[c] = (rows of chunk c with more than one member, their entries).
template <typename T, int OP, int MODE, int PF = 0, int PERM = 0, int SG = 0>
__global__ void __launch_bounds__(kOgsThreads, kOgsPersistentCtas)
k_ogsp_gather(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ rs,
              const int32_t* __restrict__ ids, T* v, T* __restrict__ gv, int grouped,
              const int32_t* __restrict__ perm, const int2* __restrict__ sing) {
  __shared__ WarpSmem<T> sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t W = gridDim.x * kWarpsPerCta;
  int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;
  T* sv = sm.val[w];
  int32_t* srs = sm.rs[w];
  uint8_t* sro = sm.ro[w];
  const int4 zero = make_int4(0, 0, 0, 0);
  int4 d = __ldg(chunks + c);
  int4 dn = (c + W < nchunks) ? __ldg(chunks + c + W) : zero;
  int2 sg = SG ? __ldg(sing + c) : make_int2(0, 0);
  int32_t col[kOgsPerLane];
  load_cols(ids, d, lane, col);
  while (true) {
    const int4 dnn = (c + 2 * W < nchunks) ? __ldg(chunks + c + 2 * W) : zero;
    const int2 sgn = (SG && c + W < nchunks) ? __ldg(sing + c + W) : make_int2(0, 0);
    const int32_t gn = d.w - d.z, nr = d.y - d.x;
    // rows [0, k0) of the chunk hold entries [0, s0); the rest are single members
    const int32_t k0 = SG ? sg.x : nr, s0 = SG ? sg.y : gn;
    T val[kOgsPerLane];
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u)
      if (lane + 32 * u < gn) val[u] = v[col[u]];
    if (SG && MODE == 0) {  // the single-member rows' words are not needed
      for (int32_t r = lane; r < k0; r += 32) {
        const int32_t wd = __ldg(rs + d.x + r);
        srs[r] = wd & 0xFFFF;
        sro[r] = (uint8_t)(wd >> 16);
      }
      if (lane == 0) srs[k0] = s0;
    } else {  // a gather stages every row's word; SG then stops the combine at k0
      stage_rows(rs, grouped, d, lane, srs, sro);
      if (SG && lane == 0) srs[k0] = s0;
    }
    int32_t coln[kOgsPerLane];
    load_cols(ids, dn, lane, coln);
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u) {
      const int32_t e = lane + 32 * u;
      if (e < s0) {
        sv[e] = val[u];
      } else if (SG && MODE == 0 && e < gn) {
        const T y = Op<T, OP>::first(val[u]);
        if (!same_bits(y, val[u])) v[col[u]] = y;
      }
    }
    if (PF) {
      const int32_t gnn = dn.w - dn.z;
#pragma unroll
      for (int u = 0; u < kOgsPerLane; ++u)
        if (lane + 32 * u < gnn) prefetch_elem_l2(v + coln[u]);
    }
    __syncwarp();
    if (SG && MODE == 1) {  // single-member rows: written from the gathering lane
#pragma unroll
      for (int u = 0; u < kOgsPerLane; ++u) {
        const int32_t e = lane + 32 * u;
        if (e >= s0 && e < gn)
          gv[op_row<PERM>(perm, d.x + (int32_t)sro[k0 + (e - s0)])] = Op<T, OP>::first(val[u]);
      }
    }
    for (int32_t r = lane; r < k0; r += 32) {
      const RowRef q = staged_row(srs, sro, grouped, r);
      T acc = row_combine<T, OP>(sv, q.a, q.b);
      if (MODE == 0) {
        for (int32_t i = q.a; i < q.b; ++i) sv[i] = acc;
      } else {
        gv[op_row<PERM>(perm, d.x + q.row)] = acc;
      }
    }
    __syncwarp();
    if (MODE == 0) {
#pragma unroll
      for (int u = 0; u < kOgsPerLane; ++u)
        if (lane + 32 * u < s0) v[col[u]] = sv[lane + 32 * u];
      __syncwarp();
    }
    c += W;
    if (c >= nchunks) break;
    d = dn;
    dn = dnn;
    sg = sgn;
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u) col[u] = coln[u];
  }
}

template <typename T, int PERM = 0>
__global__ void __launch_bounds__(kOgsThreads, 4)
k_ogsp_scatter(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ rs,
               const int32_t* __restrict__ ids, const T* __restrict__ gv, T* __restrict__ v,
               int grouped, const int32_t* __restrict__ perm) {
  __shared__ WarpSmem<T> sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t W = gridDim.x * kWarpsPerCta;
  int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;
  T* sv = sm.val[w];
  const int4 zero = make_int4(0, 0, 0, 0);
  int4 d = __ldg(chunks + c);
  int4 dn = (c + W < nchunks) ? __ldg(chunks + c + W) : zero;
  int32_t col[kOgsPerLane];
  load_cols(ids, d, lane, col);
  while (true) {
    const int4 dnn = (c + 2 * W < nchunks) ? __ldg(chunks + c + 2 * W) : zero;
    const int32_t sn = d.w - d.z, nr = d.y - d.x;
    int32_t coln[kOgsPerLane];
    load_cols(ids, dn, lane, coln);
    for (int32_t r = lane; r < nr; r += 32) {
      const RowRef q = global_row(rs, grouped, d, r);
      const T x = gv[op_row<PERM>(perm, d.x + q.row)];
      for (int32_t i = q.a; i < q.b; ++i) sv[i] = x;
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u)
      if (lane + 32 * u < sn) v[col[u]] = sv[lane + 32 * u];
    __syncwarp();
    c += W;
    if (c >= nchunks) break;
    d = dn;
    dn = dnn;
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u) col[u] = coln[u];
  }
}

// Asynchronously staged persistent variant (kernel 3): a chunk's gathered values
// and row words are copied global -> shared with cp.async one chunk ahead, so
// chunk c+W's gathers are in flight while chunk c is combined and written back.
// Two buffers per warp; the column ids of chunk c+2W are loaded into registers a
// further step ahead.  In gather+scatter mode chunk c+W's reads cannot see chunk
// c's writes: every column belongs to exactly one row and every row to exactly
// one chunk.
__device__ __forceinline__ void cp_async_4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
template <typename T>
__device__ __forceinline__ void cp_async_val(T* smem, const T* gmem) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte values");
  if constexpr (sizeof(T) == 8)
    cp_async_8(smem, gmem);
  else
    cp_async_4(smem, gmem);
}

template <typename T>
struct AsyncSmem {  // 48 KiB for 8-byte values
  T val[kWarpsPerCta][2][kWarpChunkNnz];
  int32_t rw[kWarpsPerCta][2][kWarpChunkNnz];  // row words as stored in `rs`
};

template <typename T>
__device__ __forceinline__ void async_issue(const int32_t* __restrict__ rs, const T* v, int4 d,
                                            const int32_t (&col)[kOgsPerLane], int lane, T* sv,
                                            int32_t* srw) {
  const int32_t gn = d.w - d.z, nr = d.y - d.x;
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u)
    if (lane + 32 * u < gn) cp_async_val<T>(sv + lane + 32 * u, v + col[u]);
  for (int32_t r = lane; r < nr; r += 32) cp_async_4(srw + r, rs + d.x + r);
}

template <typename T, int OP, int MODE>  // MODE 0: gather+scatter (Sym), 1: gather
__global__ void __launch_bounds__(kOgsThreads, 4)
k_ogsa_gather(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ rs,
              const int32_t* __restrict__ ids, T* v, T* __restrict__ gv, int grouped) {
  __shared__ AsyncSmem<T> sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t W = gridDim.x * kWarpsPerCta;
  int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;
  const int4 zero = make_int4(0, 0, 0, 0);
  int4 d = __ldg(chunks + c);
  int4 dn = (c + W < nchunks) ? __ldg(chunks + c + W) : zero;
  int32_t col[kOgsPerLane], coln[kOgsPerLane];
  load_cols(ids, d, lane, col);
  async_issue<T>(rs, v, d, col, lane, sm.val[w][0], sm.rw[w][0]);
  cp_async_commit();
  load_cols(ids, dn, lane, coln);
  int buf = 0;
  while (true) {
    const int4 dnn = (c + 2 * W < nchunks) ? __ldg(chunks + c + 2 * W) : zero;
    // chunk c+W's copies (dn is all zeros past the end: nothing is issued)
    async_issue<T>(rs, v, dn, coln, lane, sm.val[w][buf ^ 1], sm.rw[w][buf ^ 1]);
    cp_async_commit();
    int32_t colnn[kOgsPerLane];
    load_cols(ids, dnn, lane, colnn);
    cp_async_wait<1>();  // chunk c's group has landed
    __syncwarp();
    const T* sv = sm.val[w][buf];
    const int32_t* srw = sm.rw[w][buf];
    const int32_t gn = d.w - d.z, nr = d.y - d.x;
    for (int32_t r = lane; r < nr; r += 32) {
      const int32_t wa = srw[r];
      const int32_t a = grouped ? (wa & 0xFFFF) : wa - d.z;
      const int32_t b = (r + 1 < nr) ? (grouped ? (srw[r + 1] & 0xFFFF) : srw[r + 1] - d.z) : gn;
      T acc = row_combine<T, OP>(sv, a, b);
      if (MODE == 0) {
        T* svw = sm.val[w][buf];
        for (int32_t i = a; i < b; ++i) svw[i] = acc;
      } else {
        gv[d.x + (grouped ? (wa >> 16) : r)] = acc;
      }
    }
    __syncwarp();
    if (MODE == 0) {
#pragma unroll
      for (int u = 0; u < kOgsPerLane; ++u)
        if (lane + 32 * u < gn) v[col[u]] = sv[lane + 32 * u];
      __syncwarp();  // buffer `buf` is refilled by the next iteration's copies
    }
    c += W;
    if (c >= nchunks) break;
    d = dn;
    dn = dnn;
    buf ^= 1;
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u) {
      col[u] = coln[u];
      coln[u] = colnn[u];
    }
  }
  cp_async_wait<0>();
}

// Column-order gathers (kernel 4 for gathers on T chunks), pipelined and persistent
// like k_ogsp_gather: lane j of each pass loads the j-th smallest column of the
// chunk, so a warp's loads (and, in gather+scatter mode, its stores) cover
// neighbouring addresses; e2s maps each entry of the row walk to its slot, so every
// row is still combined in CSR order from the op's identity (identical bits).
template <typename T>
struct SortedSmem {
  T val[kWarpsPerCta][kWarpChunkNnz];
  int32_t rs[kWarpsPerCta][kWarpChunkNnz + 8];
  uint8_t ro[kWarpsPerCta][kWarpChunkNnz];
  uint8_t e2s[kWarpsPerCta][kWarpChunkNnz];
};

template <typename T, int OP, int MODE>  // MODE 0: gather+scatter (Sym), 1: gather
__global__ void __launch_bounds__(kOgsThreads, 4)
k_ogso_gather(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ rs,
              const int32_t* __restrict__ colS, const uint8_t* __restrict__ e2s, T* v,
              T* __restrict__ gv, int grouped) {
  __shared__ SortedSmem<T> sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t W = gridDim.x * kWarpsPerCta;
  int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;
  T* sv = sm.val[w];
  int32_t* srs = sm.rs[w];
  uint8_t* sro = sm.ro[w];
  uint8_t* se = sm.e2s[w];
  const int4 zero = make_int4(0, 0, 0, 0);
  int4 d = __ldg(chunks + c);
  int4 dn = (c + W < nchunks) ? __ldg(chunks + c + W) : zero;
  int32_t col[kOgsPerLane];
  load_cols(colS, d, lane, col);
  while (true) {
    const int4 dnn = (c + 2 * W < nchunks) ? __ldg(chunks + c + 2 * W) : zero;
    const int32_t gn = d.w - d.z, nr = d.y - d.x;
    T val[kOgsPerLane];
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u)
      if (lane + 32 * u < gn) val[u] = v[col[u]];
    stage_rows(rs, grouped, d, lane, srs, sro);
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u)
      if (lane + 32 * u < gn) se[lane + 32 * u] = __ldg(e2s + d.z + lane + 32 * u);
    int32_t coln[kOgsPerLane];
    load_cols(colS, dn, lane, coln);
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u)
      if (lane + 32 * u < gn) sv[lane + 32 * u] = val[u];
    __syncwarp();
    for (int32_t r = lane; r < nr; r += 32) {
      const RowRef q = staged_row(srs, sro, grouped, r);
      T acc = Op<T, OP>::init();
      if (q.a < q.b) {
        acc = Op<T, OP>::first(sv[se[q.a]]);
        for (int32_t i = q.a + 1; i < q.b; ++i) Op<T, OP>::apply(acc, sv[se[i]]);
      }
      if (MODE == 0) {
        for (int32_t i = q.a; i < q.b; ++i) sv[se[i]] = acc;
      } else {
        gv[d.x + q.row] = acc;
      }
    }
    __syncwarp();
    if (MODE == 0) {
#pragma unroll
      for (int u = 0; u < kOgsPerLane; ++u)
        if (lane + 32 * u < gn) v[col[u]] = sv[lane + 32 * u];
      __syncwarp();
    }
    c += W;
    if (c >= nchunks) break;
    d = dn;
    dn = dnn;
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u) col[u] = coln[u];
  }
}

// Column-order scatter (kernel 3 for scatters on T chunks): the chunk's row values
// are read as one contiguous slice of gv into shared memory, then lane j of each
// pass writes the j-th smallest column of the chunk.  Every load depends only on
// the descriptor (one dependent round trip), there is no per-row loop, and the
// stores of neighbouring lanes land on neighbouring addresses.  Copies only:
// bit-identical to every other scatter.
template <typename T, int PERM = 0>
__global__ void __launch_bounds__(kOgsThreads, kOgsScatterCtas)
k_ogss_scatter(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ colS,
               const uint8_t* __restrict__ rowOf, const T* __restrict__ gv, T* __restrict__ v,
               const int32_t* __restrict__ perm) {
  __shared__ T sres[kWarpsPerCta][kWarpChunkNnz];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;
  const int4 d = __ldg(chunks + c);
  const int32_t nr = d.y - d.x, sn = d.w - d.z;
  T* sr = sres[w];
  int32_t col[kOgsPerLane];
  int32_t ro[kOgsPerLane];
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u) {
    const int i = lane + 32 * u;
    col[u] = (i < sn) ? __ldg(colS + d.z + i) : 0;
    ro[u] = (i < sn) ? (int32_t)__ldg(rowOf + d.z + i) : 0;
  }
  for (int32_t r = lane; r < nr; r += 32) sr[r] = gv[op_row<PERM>(perm, d.x + r)];
  __syncwarp();
#pragma unroll
  for (int u = 0; u < kOgsPerLane; ++u)
    if (lane + 32 * u < sn) v[col[u]] = sr[ro[u]];
}

// Column-major scatter (kernel 5 for scatters on T): one thread per local column,
// v[i] = gv[row of i], so the stores of a warp are one contiguous run; the row
// values are read where each column's row lies (rows numbered by first
// appearance keep those reads mostly local).  Columns in no row are left alone.
template <typename T>
__global__ void __launch_bounds__(kOgsThreads)
k_ogsc_scatter(int32_t N, const int32_t* __restrict__ rowOfCol, const T* __restrict__ gv,
               T* __restrict__ v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = __ldg(rowOfCol + i);
    if (r >= 0) v[i] = gv[r];
  }
}

// The same with 16-byte accesses: each thread takes 16 / sizeof(T) consecutive
// columns (one int4 or int2 of row ids, one 16-byte store), for 16-byte-aligned v;
// the last N mod that width columns are copied one per thread by the first block.
// A column in no row keeps its value: the old vector is read only when the group
// holds such a column.
template <typename T> struct Vec16Of;
template <> struct Vec16Of<float> { using type = float4; };
template <> struct Vec16Of<double> { using type = double2; };
template <> struct Vec16Of<int32_t> { using type = int4; };
template <> struct Vec16Of<long long> { using type = longlong2; };

template <typename T>
__global__ void __launch_bounds__(kOgsThreads)
k_ogsc_scatter_vec(int64_t N, const int32_t* __restrict__ rowOfCol, const T* __restrict__ gv,
                   T* __restrict__ v) {
  constexpr int V = 16 / sizeof(T);
  using IV = typename std::conditional<V == 4, int4, int2>::type;
  using TV = typename Vec16Of<T>::type;
  const int64_t nvec = N / V;
  if (blockIdx.x == 0 && threadIdx.x < N - nvec * V) {
    const int64_t i = nvec * V + threadIdx.x;
    const int32_t r = __ldg(rowOfCol + i);
    if (r >= 0) v[i] = gv[r];
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nvec;
       i += (int64_t)gridDim.x * blockDim.x) {
    const IV rv = __ldg(reinterpret_cast<const IV*>(rowOfCol) + i);
    const int32_t* r = reinterpret_cast<const int32_t*>(&rv);
    bool any_free = false;
#pragma unroll
    for (int k = 0; k < V; ++k) any_free |= r[k] < 0;
    TV out;
    T* o = reinterpret_cast<T*>(&out);
    if (any_free) out = reinterpret_cast<const TV*>(v)[i];
#pragma unroll
    for (int k = 0; k < V; ++k)
      if (r[k] >= 0) o[k] = gv[r[k]];
    reinterpret_cast<TV*>(v)[i] = out;
  }
}

// The 16-byte column-major scatter with the pages of local columns taken in the
// main walk's visit order instead of memory order: group g (V columns) lies in the
// (g*V >> shift)-th visited page.  On a mesh whose elements sit at random places,
// the rows an element shares with its neighbours were numbered inside those
// neighbours, so in memory order each such row is fetched once per element that
// holds it, from far apart in time; in walk order the neighbours run close
// together and the second fetch usually hits L2.  Stores stay contiguous within a
// page.  Requires 16-byte-aligned v and 2^shift >= V (pages of at least 1 KiB are
// used).
template <typename T>
__global__ void __launch_bounds__(kOgsThreads)
k_ogsc_scatter_pages(int64_t ngroups, const int32_t* __restrict__ pages, int shift, int64_t N,
                     const int32_t* __restrict__ rowOfCol, const T* __restrict__ gv,
                     T* __restrict__ v) {
  constexpr int V = 16 / sizeof(T);
  using IV = typename std::conditional<V == 4, int4, int2>::type;
  using TV = typename Vec16Of<T>::type;
  const int64_t mask = ((int64_t)1 << shift) - 1;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ngroups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = g * V;
    const int64_t c = ((int64_t)__ldg(pages + (x >> shift)) << shift) + (x & mask);
    if (c + V <= N) {
      const IV rv = __ldg(reinterpret_cast<const IV*>(rowOfCol + c));
      const int32_t* r = reinterpret_cast<const int32_t*>(&rv);
      bool any_free = false;
#pragma unroll
      for (int k = 0; k < V; ++k) any_free |= r[k] < 0;
      TV out;
      T* o = reinterpret_cast<T*>(&out);
      if (any_free) out = *reinterpret_cast<const TV*>(v + c);
#pragma unroll
      for (int k = 0; k < V; ++k)
        if (r[k] >= 0) o[k] = gv[r[k]];
      *reinterpret_cast<TV*>(v + c) = out;
    } else {
      for (int64_t i = c; i < N; ++i) {
        const int32_t r = __ldg(rowOfCol + i);
        if (r >= 0) v[i] = gv[r];
      }
    }
  }
}

// Persistent column-order scatter (kernel 4 for scatters on T chunks): as kernel 3,
// with each warp walking chunks c, c+W, ... and bulk-prefetching the next chunk's
// three contiguous ranges (column ids, row offsets, gv slice) into L2 before
// working on the current one.
__device__ __forceinline__ void prefetch_range_l2(const void* base, int64_t first_byte,
                                                  int64_t end_byte, int64_t limit_byte) {
  const int64_t a = first_byte & ~(int64_t)15;
  int64_t b = (end_byte + 15) & ~(int64_t)15;
  const int64_t lim = limit_byte & ~(int64_t)15;
  b = b < lim ? b : lim;
  if (b > a)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"((const char*)base + a),
                 "r"((uint32_t)(b - a))
                 : "memory");
}

template <typename T>
__global__ void __launch_bounds__(kOgsThreads, kOgsScatterCtas)
k_ogssp_scatter(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ colS,
                const uint8_t* __restrict__ rowOf, const T* __restrict__ gv, T* __restrict__ v,
                int64_t nnz, int64_t nrows) {
  __shared__ T sres[kWarpsPerCta][kWarpChunkNnz];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t W = gridDim.x * kWarpsPerCta;
  int32_t c = blockIdx.x * kWarpsPerCta + w;
  T* sr = sres[w];
  while (c < nchunks) {
    const int4 d = __ldg(chunks + c);
    if (c + W < nchunks && lane < 3) {
      const int4 e = __ldg(chunks + c + W);
      if (lane == 0) prefetch_range_l2(colS, 4LL * e.z, 4LL * e.w, 4LL * nnz);
      if (lane == 1) prefetch_range_l2(rowOf, e.z, e.w, nnz);
      if (lane == 2)
        prefetch_range_l2(gv, (int64_t)sizeof(T) * e.x, (int64_t)sizeof(T) * e.y,
                          (int64_t)sizeof(T) * nrows);
    }
    const int32_t nr = d.y - d.x, sn = d.w - d.z;
    int32_t col[kOgsPerLane];
    int32_t ro[kOgsPerLane];
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u) {
      const int i = lane + 32 * u;
      col[u] = (i < sn) ? __ldg(colS + d.z + i) : 0;
      ro[u] = (i < sn) ? (int32_t)__ldg(rowOf + d.z + i) : 0;
    }
    for (int32_t r = lane; r < nr; r += 32) sr[r] = gv[d.x + r];
    __syncwarp();
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u)
      if (lane + 32 * u < sn) v[col[u]] = sr[ro[u]];
    __syncwarp();  // sres is refilled by the next chunk
    c += W;
  }
}

// ------------------------------------------------------------------ bulk copies
//
// TMA bulk copies global -> shared memory (cp.async.bulk, completion counted in
// bytes on an mbarrier) and bounded waits on them.

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(1) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// One bounded wait for the phase with parity `ph` to complete: true when it did.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t ph) {
  constexpr int kMaxPolls = 1 << 22;  // each poll may suspend for a while: seconds at most
  for (int i = 0; i < kMaxPolls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(ph)
        : "memory");
    if (done) return true;
  }
  return false;
}
// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) from global
// to this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

static inline unsigned persistent_grid(int32_t nchunks, int ctas_per_sm = 4) {
  const int64_t want = ((int64_t)nchunks + kWarpsPerCta - 1) / kWarpsPerCta;
  const int64_t cap = (int64_t)sm_count() * ctas_per_sm;
  return (unsigned)(want < cap ? (want < 1 ? 1 : want) : cap);
}

static inline unsigned warp_grid(int32_t nchunks) {
  return (unsigned)((nchunks + kWarpsPerCta - 1) / kWarpsPerCta);
}

// Kernel variant of an operation (knobs ogs.kernel / ogs.kernel.gather /
// ogs.kernel.scatter): 0 block kernels, 1 warp chunks, 2 pipelined warp chunks,
// 3 asynchronously staged warp chunks for the gathers and column-order warp chunks
// for the scatter, 4 column-order pipelined gathers and the persistent
// column-order scatter with L2 prefetch, 5 pipelined gathers with L2 prefetch of
// the next chunk.  Launches through the N operator take the pipelined kernels for
// the column-order variants.  The warp variants need k == 1 and a plan with chunks.
static inline int variant(TuneKey key, int K, int32_t nchunks) {
  return (K == 1 && nchunks > 0) ? (int)tune(key) : 0;
}

// The same for 4-byte values, which may take a kernel of their own (knobs
// ogs.kernel.f32 / ogs.kernel.gather.f32; -1 = as for 8-byte values).
template <typename T>
static inline int variant_for(TuneKey key, TuneKey key32, int K, int32_t nchunks) {
  if (sizeof(T) == 4 && K == 1 && nchunks > 0 && tune(key32) >= 0) return (int)tune(key32);
  return variant(key, K, nchunks);
}

// The arrays one warp-chunk launch walks: T chunks use the grouped rows when the
// plan has them; N chunks always use CSR order.
struct ChunkArgs {
  const int4* chunks;
  int32_t nchunks;
  const int32_t* rs;
  const int32_t* ids;
  int grouped;
  const int32_t* colS;  // column-order entries (T chunks only, else null)
  const uint8_t* e2s;
  const int32_t* perm;  // walk row -> row of the operator (renumbered walk only)
  int32_t* waitErr;      // the plan's count of bounded waits that gave up
  const int2* sing;      // per chunk (multi-member rows, their entries), grouped rows only
  SlabArgs slab;          // lane-row slabs of the same walk (kernel 7); slabs null if none
};
static inline ChunkArgs chunks_t(const sp_ogs_plan* p) {
  const bool g = p->row_order == 1;
  const int32_t* rs = p->d_walkRsT ? p->d_walkRsT : p->d_rowStartsT;
  const int32_t* ci = p->d_walkCiT ? p->d_walkCiT : p->d_colIdsT;
  return ChunkArgs{reinterpret_cast<const int4*>(p->d_chunksT), p->nchunksT,
                   g ? p->d_rowsGT : rs, g ? p->d_colIdsGT : ci, g ? 1 : 0,
                   p->d_colIdsST, p->d_e2sT, p->d_permT, p->d_waitErr,
                   g ? reinterpret_cast<const int2*>(p->d_singT) : nullptr,
                   SlabArgs{reinterpret_cast<const int4*>(p->d_slabsT), p->nslabsT, p->d_slabIdsT,
                            p->d_slabRowsT, p->d_slabCodesT, p->d_slabTabsT,
                            reinterpret_cast<const int2*>(p->d_slabTdT), p->slab_code_shift,
                            p->d_slabRowCodesT, p->d_slabRowTabsT,
                            reinterpret_cast<const int2*>(p->d_slabRowTdT)}};
}
// The gather+scatter walk when the plan has one (kernel 4 needs the column-order
// arrays of the main walk, so it runs as kernel 2 there).
static inline ChunkArgs chunks_gs(const sp_ogs_plan* p) {
  const int32_t* rs = p->d_rsGS ? p->d_rsGS : p->d_rowStartsT;
  const int32_t* ci = p->d_ciGS ? p->d_ciGS : p->d_colIdsT;
  return ChunkArgs{reinterpret_cast<const int4*>(p->d_chunksGS), p->nchunksGS, rs, ci,
                   p->gs_grouped, nullptr, nullptr, nullptr, p->d_waitErr,
                   p->gs_grouped ? reinterpret_cast<const int2*>(p->d_singGS) : nullptr,
                   SlabArgs{reinterpret_cast<const int4*>(p->d_slabsGS), p->nslabsGS,
                            p->d_slabIdsGS, nullptr, p->d_slabCodesGS, p->d_slabTabsGS,
                            reinterpret_cast<const int2*>(p->d_slabTdGS), p->slab_code_shift,
                            nullptr, nullptr, nullptr}};
}
static inline ChunkArgs chunks_n(const sp_ogs_plan* p) {
  return ChunkArgs{reinterpret_cast<const int4*>(p->d_chunksN), p->nchunksN, p->d_rowStartsNpad,
                   p->d_colIdsN, 0, nullptr, nullptr, nullptr, p->d_waitErr, nullptr,
                   SlabArgs{nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, 0, nullptr,
                            nullptr, nullptr}};
}

// Kernel 6: the pipelined persistent gathers of kernel 2 with the chunks' column ids
// staged in shared memory by TMA bulk copy instead of held in registers.  A chunk's
// ids are one contiguous run (<= 1 KiB); lane 0 copies the 16-byte aligned span
// around it into one of two buffers of its warp one chunk ahead, completing on an
// mbarrier, so chunk c + W's ids travel while chunk c's gathers are in flight.
// Lanes read their 8 ids from the buffer when they issue the gathers and again
// when the gather+scatter writes back, so the 16 id registers of kernel 2 are not
// needed.  Row words, the combine in CSR order and the results are those of
// kernel 2 (same bits).  Measured on GB300 it is slower than kernel 2: with 5
// CTAs per SM the register budget of 48 spills (BS6 2.9 against 5.3 TB/s on the
// permuted 64^3 p=7 box), and at kernel 2's 4 CTAs it reaches 4.6 TB/s -- the
// staging costs more than the id registers it frees; it is kept as the
// bulk-staged option, and the tuned tables do not select it.
struct __align__(128) BulkIds {
  int32_t ids[kWarpsPerCta][2][kWarpChunkNnz + 8];  // + 3 leading ids of the aligned span
  unsigned long long bar[kWarpsPerCta][2];
};

// Lane 0: copy the ids of chunk d into buffer b of warp w; returns nothing, the
// buffer holds ids[(d.z & ~3) ...] so entry i of the chunk is at (d.z & 3) + i.
__device__ __forceinline__ void stage_ids(BulkIds& bi, int w, int b, int4 d,
                                          const int32_t* __restrict__ ids) {
  const int32_t a0 = d.z & ~3, a1 = (d.w + 3) & ~3;
  const uint32_t bytes = (uint32_t)(a1 - a0) * 4u;
  mbar_expect_tx(&bi.bar[w][b], bytes);
  if (bytes) bulk_g2s(bi.ids[w][b], ids + a0, bytes, &bi.bar[w][b]);
}

template <typename T, int OP, int MODE, int PERM>
__global__ void __launch_bounds__(kOgsThreads, kOgsBulkCtas)
k_ogsb_gather(const int4* __restrict__ chunks, int32_t nchunks, const int32_t* __restrict__ rs,
              const int32_t* __restrict__ ids, T* v, T* __restrict__ gv, int grouped,
              const int32_t* __restrict__ perm, int32_t* __restrict__ werr) {
  __shared__ WarpSmem<T> sm;
  __shared__ BulkIds bi;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t W = gridDim.x * kWarpsPerCta;
  int32_t c = blockIdx.x * kWarpsPerCta + w;
  if (c >= nchunks) return;  // the whole warp leaves together
  T* sv = sm.val[w];
  int32_t* srs = sm.rs[w];
  uint8_t* sro = sm.ro[w];
  if (lane == 0) {
    mbar_init(&bi.bar[w][0]);
    mbar_init(&bi.bar[w][1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  const int4 zero = make_int4(0, 0, 0, 0);
  int4 d = __ldg(chunks + c);
  int4 dn = (c + W < nchunks) ? __ldg(chunks + c + W) : zero;
  if (lane == 0) stage_ids(bi, w, 0, d, ids);
  int b = 0;
  uint32_t ph0 = 0u, ph1 = 0u;
  while (true) {
    const bool more = c + W < nchunks;
    const int4 dnn = (c + 2 * W < nchunks) ? __ldg(chunks + c + 2 * W) : zero;
    // buffer b ^ 1 was last read in the previous iteration, which every lane has left
    if (more && lane == 0) stage_ids(bi, w, b ^ 1, dn, ids);
    if (!mbar_wait(&bi.bar[w][b], b ? ph1 : ph0)) {
      if (lane == 0) atomicAdd(werr, 1);
      if (more) mbar_wait(&bi.bar[w][b ^ 1], b ? ph0 : ph1);  // no copy may outlive the CTA
      return;
    }
    if (b) ph1 ^= 1u;
    else ph0 ^= 1u;
    const int32_t* cid = bi.ids[w][b] + (d.z & 3);
    const int32_t gn = d.w - d.z, nr = d.y - d.x;
    T val[kOgsPerLane];
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u)
      if (lane + 32 * u < gn) val[u] = v[cid[lane + 32 * u]];
    stage_rows(rs, grouped, d, lane, srs, sro);
#pragma unroll
    for (int u = 0; u < kOgsPerLane; ++u)
      if (lane + 32 * u < gn) sv[lane + 32 * u] = val[u];
    __syncwarp();
    for (int32_t r = lane; r < nr; r += 32) {
      const RowRef q = staged_row(srs, sro, grouped, r);
      T acc = row_combine<T, OP>(sv, q.a, q.b);
      if (MODE == 0) {
        for (int32_t i = q.a; i < q.b; ++i) sv[i] = acc;
      } else {
        gv[op_row<PERM>(perm, d.x + q.row)] = acc;
      }
    }
    __syncwarp();
    if (MODE == 0) {
#pragma unroll
      for (int u = 0; u < kOgsPerLane; ++u)
        if (lane + 32 * u < gn) v[cid[lane + 32 * u]] = sv[lane + 32 * u];
    }
    __syncwarp();  // buffers sv and ids[b] are refilled by the next chunks
    c += W;
    if (c >= nchunks) break;
    d = dn;
    dn = dnn;
    b ^= 1;
  }
}

template <typename T, int OP, int MODE>
static void launch_bulk_gather(const ChunkArgs& a, T* v, T* gv, bool perm, cudaStream_t s) {
  const unsigned g = persistent_grid(a.nchunks, kOgsBulkCtas);
  if (perm)
    k_ogsb_gather<T, OP, MODE, 1><<<g, kOgsThreads, 0, s>>>(a.chunks, a.nchunks, a.rs, a.ids, v,
                                                           gv, a.grouped, a.perm, a.waitErr);
  else
    k_ogsb_gather<T, OP, MODE, 0><<<g, kOgsThreads, 0, s>>>(a.chunks, a.nchunks, a.rs, a.ids, v,
                                                           gv, a.grouped, nullptr, a.waitErr);
}

// ------------------------------------------------------------------ dispatch

template <typename T, int OP, int MODE>
static void launch_chunked_gather(int kv, const ChunkArgs& a, T* v, T* gv, cudaStream_t s) {
  // a gather through a renumbered walk writes gv through perm: kernels 1, 2, 5 do
  const bool perm = MODE == 1 && a.perm;
  if (perm && (kv == 3 || kv == 4)) kv = 2;
  if (kv == 6 && !a.waitErr) kv = 2;  // a plan without chunks has no wait-error word
  if (kv == 7 && !a.slab.slabs) kv = 2;  // a plan built without slabs (ogs.slabs = 0)
  const unsigned pg = persistent_grid(a.nchunks, kOgsPersistentCtas);
  if (kv == 7) {
    launch_slabs<T, OP, MODE>(a.slab, v, gv, s);
  } else if (kv == 6) {
    launch_bulk_gather<T, OP, MODE>(a, v, gv, perm, s);
  } else if (kv == 5) {
    if (perm)
      k_ogsp_gather<T, OP, MODE, 1, 1><<<pg, kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, a.perm, nullptr);
    else
      k_ogsp_gather<T, OP, MODE, 1, 0><<<pg, kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, nullptr, nullptr);
  } else if (kv == 4 && a.e2s) {
    k_ogso_gather<T, OP, MODE><<<persistent_grid(a.nchunks), kOgsThreads, 0, s>>>(
        a.chunks, a.nchunks, a.rs, a.colS, a.e2s, v, gv, a.grouped);
  } else if (kv == 3) {
    k_ogsa_gather<T, OP, MODE><<<persistent_grid(a.nchunks), kOgsThreads, 0, s>>>(
        a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped);
  } else if (kv >= 2) {
    // the single-member path serves the in-place gather+scatter (MODE 0): there it
    // saves the staging and the unchanged stores; a gather still writes every row,
    // and measured slower with it
    const int64_t sgk = tune(kTuneOgsSingles);
    if (MODE == 0 && a.sing && a.grouped && sgk >= 1)
      k_ogsp_gather<T, OP, 0, 0, 0, 1><<<pg, kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, nullptr, a.sing);
    else if (MODE == 1 && a.sing && a.grouped && sgk == 2 && perm)
      k_ogsp_gather<T, OP, 1, 0, 1, 1><<<pg, kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, a.perm, a.sing);
    else if (MODE == 1 && a.sing && a.grouped && sgk == 2)
      k_ogsp_gather<T, OP, 1, 0, 0, 1><<<pg, kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, nullptr, a.sing);
    else if (perm)
      k_ogsp_gather<T, OP, MODE, 0, 1><<<pg, kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, a.perm, nullptr);
    else
      k_ogsp_gather<T, OP, MODE, 0, 0><<<pg, kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, nullptr, nullptr);
  } else if (MODE == 0) {
    k_ogsw_gs_sym<T, OP><<<warp_grid(a.nchunks), kOgsThreads, 0, s>>>(a.chunks, a.nchunks, a.rs,
                                                                     a.ids, v, a.grouped);
  } else if (perm) {
    k_ogsw_gather<T, OP, 1><<<warp_grid(a.nchunks), kOgsThreads, 0, s>>>(
        a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, a.perm);
  } else {
    k_ogsw_gather<T, OP, 0><<<warp_grid(a.nchunks), kOgsThreads, 0, s>>>(
        a.chunks, a.nchunks, a.rs, a.ids, v, gv, a.grouped, nullptr);
  }
}

template <typename T, int OP>
static void launch_gs(const sp_ogs_plan* p, sp_transpose trans, int K, T* v, cudaStream_t s) {
  if (p->NrowBlocksT == 0) return;
  dim3 grid(p->NrowBlocksT, K);
  const int kv = variant_for<T>(kTuneOgsKernel, kTuneOgsKernel32, K, p->nchunksT);
  if ((trans == SP_SYM || p->n_is_t) && kv > 0 && p->nchunksGS > 0) {
    launch_chunked_gather<T, OP, 0>(kv, chunks_gs(p), v, nullptr, s);  // 4 runs as 2 here
  } else if ((trans == SP_SYM || p->n_is_t) && kv > 0) {
    launch_chunked_gather<T, OP, 0>(kv, chunks_t(p), v, nullptr, s);
  } else if (trans == SP_SYM || p->n_is_t) {
    k_ogs_gs_sym<T, OP><<<grid, kOgsThreads, 0, s>>>(p->d_blocksT, p->d_rowStartsT, p->d_colIdsT,
                                                     v, K);
  } else if (trans == SP_NOTRANS) {  // gather N, scatter T
    k_ogs_gs_gen<T, OP><<<grid, kOgsThreads, 0, s>>>(p->d_blocksT, p->d_rowStartsNpad,
                                                     p->d_colIdsN, p->d_rowStartsT, p->d_colIdsT,
                                                     v, K);
  } else {  // SP_TRANS: gather T, scatter N
    k_ogs_gs_gen<T, OP><<<grid, kOgsThreads, 0, s>>>(p->d_blocksT, p->d_rowStartsT, p->d_colIdsT,
                                                     p->d_rowStartsNpad, p->d_colIdsN, v, K);
  }
}

template <typename T, int OP>
static void launch_gather(const sp_ogs_plan* p, sp_transpose trans, int K, T* gv, const T* v,
                          cudaStream_t s) {
  const bool useN = (trans == SP_NOTRANS);
  const int kv = variant_for<T>(kTuneOgsKernelGather, kTuneOgsKernelGather32, K,
                                useN ? p->nchunksN : p->nchunksT);
  if (kv > 0) {
    launch_chunked_gather<T, OP, 1>(kv, useN ? chunks_n(p) : chunks_t(p), const_cast<T*>(v), gv,
                                    s);
  } else if (useN) {
    if (p->NrowBlocksN == 0) return;
    k_ogs_gather<T, OP><<<dim3(p->NrowBlocksN, K), kOgsThreads, 0, s>>>(
        p->d_blocksN, p->d_rowStartsNpad, p->d_colIdsN, v, gv, K);
  } else {
    if (p->NrowBlocksT == 0) return;
    k_ogs_gather<T, OP><<<dim3(p->NrowBlocksT, K), kOgsThreads, 0, s>>>(
        p->d_blocksT, p->d_rowStartsT, p->d_colIdsT, v, gv, K);
  }
}

template <typename T>
static void launch_scatter(const sp_ogs_plan* p, sp_transpose trans, int K, T* v, const T* gv,
                           cudaStream_t s) {
  const bool useN = (trans == SP_TRANS);
  const int kv = variant(kTuneOgsKernelScatter, K, useN ? p->nchunksN : p->nchunksT);
  if (kv == 5 && !useN && p->d_rowOfColT) {
    constexpr int V = 16 / sizeof(T);
    const int64_t cap = (int64_t)sm_count() * 64;
    // walk-ordered pages pay when a page's stores are long runs: pages of 8 FP64
    // columns (64 bytes) at random places halve the store rate
    if (K == 1 && (reinterpret_cast<uintptr_t>(v) & 15) == 0 && p->d_pagesT &&
        tune(kTuneOgsScatterPages) == 1 && ((int64_t)sizeof(T) << p->pages_shift) >= 1024) {
      const int64_t ngroups = ((int64_t)p->npagesT << p->pages_shift) / V;
      const int64_t want = (ngroups + kOgsThreads - 1) / kOgsThreads;
      k_ogsc_scatter_pages<T>
          <<<(unsigned)std::max<int64_t>(1, std::min(want, cap)), kOgsThreads, 0, s>>>(
              ngroups, p->d_pagesT, p->pages_shift, (int64_t)p->N, p->d_rowOfColT, gv, v);
      return;
    }
    if (K == 1 && (reinterpret_cast<uintptr_t>(v) & 15) == 0) {
      const int64_t want = (p->N / V + kOgsThreads - 1) / kOgsThreads;
      k_ogsc_scatter_vec<T>
          <<<(unsigned)std::max<int64_t>(1, std::min(want, cap)), kOgsThreads, 0, s>>>(
              (int64_t)p->N, p->d_rowOfColT, gv, v);
      return;
    }
    const int64_t want = ((int64_t)p->N + kOgsThreads - 1) / kOgsThreads;
    k_ogsc_scatter<T><<<(unsigned)std::max<int64_t>(1, std::min(want, cap)), kOgsThreads, 0, s>>>(
        p->N, p->d_rowOfColT, gv, v);
    return;
  }
  // the persistent prefetching scatter reads gv slices directly: not through perm
  if (kv == 4 && !useN && p->d_colIdsST && !p->d_permT) {
    k_ogssp_scatter<T><<<persistent_grid(p->nchunksT, kOgsScatterCtas), kOgsThreads, 0, s>>>(
        reinterpret_cast<const int4*>(p->d_chunksT), p->nchunksT, p->d_colIdsST, p->d_rowOfST, gv,
        v, (int64_t)p->nnzT, (int64_t)p->NrowsT);
  } else if (kv >= 3 && !useN && p->d_colIdsST) {
    const int4* ch = reinterpret_cast<const int4*>(p->d_chunksT);
    if (p->d_permT)
      k_ogss_scatter<T, 1><<<warp_grid(p->nchunksT), kOgsThreads, 0, s>>>(
          ch, p->nchunksT, p->d_colIdsST, p->d_rowOfST, gv, v, p->d_permT);
    else
      k_ogss_scatter<T, 0><<<warp_grid(p->nchunksT), kOgsThreads, 0, s>>>(
          ch, p->nchunksT, p->d_colIdsST, p->d_rowOfST, gv, v, nullptr);
  } else if (kv > 0) {
    const ChunkArgs a = useN ? chunks_n(p) : chunks_t(p);
    if (kv >= 2 && a.perm)
      k_ogsp_scatter<T, 1><<<persistent_grid(a.nchunks), kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, gv, v, a.grouped, a.perm);
    else if (kv >= 2)
      k_ogsp_scatter<T, 0><<<persistent_grid(a.nchunks), kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, gv, v, a.grouped, nullptr);
    else if (a.perm)
      k_ogsw_scatter<T, 1><<<warp_grid(a.nchunks), kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, gv, v, a.grouped, a.perm);
    else
      k_ogsw_scatter<T, 0><<<warp_grid(a.nchunks), kOgsThreads, 0, s>>>(
          a.chunks, a.nchunks, a.rs, a.ids, gv, v, a.grouped, nullptr);
  } else if (useN) {
    if (p->NrowBlocksN == 0) return;
    k_ogs_scatter<T><<<dim3(p->NrowBlocksN, K), kOgsThreads, 0, s>>>(
        p->d_blocksN, p->d_rowStartsNpad, p->d_colIdsN, gv, v, K);
  } else {
    if (p->NrowBlocksT == 0) return;
    k_ogs_scatter<T><<<dim3(p->NrowBlocksT, K), kOgsThreads, 0, s>>>(
        p->d_blocksT, p->d_rowStartsT, p->d_colIdsT, gv, v, K);
  }
}

template <template <typename, int> class F, typename T, typename... A>
static void by_op(sp_op op, A... a) {
  switch (op) {
    case SP_OP_ADD: F<T, SP_OP_ADD>::run(a...); break;
    case SP_OP_MUL: F<T, SP_OP_MUL>::run(a...); break;
    case SP_OP_MAX: F<T, SP_OP_MAX>::run(a...); break;
    case SP_OP_MIN: F<T, SP_OP_MIN>::run(a...); break;
  }
}

template <typename T, int OP> struct GsF {
  static void run(const sp_ogs_plan* p, sp_transpose t, int K, void* v, cudaStream_t s) {
    launch_gs<T, OP>(p, t, K, static_cast<T*>(v), s);
  }
};
template <typename T, int OP> struct GatherF {
  static void run(const sp_ogs_plan* p, sp_transpose t, int K, void* gv, const void* v,
                  cudaStream_t s) {
    launch_gather<T, OP>(p, t, K, static_cast<T*>(gv), static_cast<const T*>(v), s);
  }
};

static sp_status check_common(const sp_ogs_plan* p, sp_type type, int32_t op, int32_t trans,
                              int32_t k, const char* name) {
  if (!p) return fail(SP_ERR_INVALID_ARG, "%s: null plan", name);
  if (type < SP_FLOAT || type > SP_INT64) return fail(SP_ERR_INVALID_ARG, "%s: bad type", name);
  if (op < SP_OP_ADD || op > SP_OP_MIN) return fail(SP_ERR_INVALID_ARG, "%s: bad op", name);
  if (trans < SP_SYM || trans > SP_TRANS)
    return fail(SP_ERR_INVALID_ARG, "%s: bad transpose", name);
  if (k < 1 || k > 65535) return fail(SP_ERR_INVALID_ARG, "%s: k=%d outside [1,65535]", name, k);
  return SP_SUCCESS;
}

// ------------------------------------------------------------------ plan construction

bool partition_rows(int32_t nrows, const int32_t* rs, std::vector<int32_t>& blocks) {
  const int32_t cap = (int32_t)tune(kTuneOgsBlockNnz);
  blocks.clear();
  blocks.push_back(0);
  int32_t b0 = 0;
  for (int32_t row = 0; row < nrows; ++row) {
    if (rs[row + 1] - rs[row] > cap) return false;
    if (rs[row + 1] - rs[b0] > cap || row - b0 >= cap) {
      blocks.push_back(row);
      b0 = row;
    }
  }
  if (nrows > 0) blocks.push_back(nrows);
  return true;
}

// Checks run in parallel; a failure reports the lowest offending row or entry, so
// the message does not depend on the thread schedule.
static sp_status validate_csr(int32_t N, int32_t nrows, const int32_t* rs, const int32_t* ids,
                              const char* which, int32_t& maxRow) {
  if (nrows < 0) return fail(SP_ERR_INVALID_ARG, "ogs plan: negative row count (%s)", which);
  if (!rs) return fail(SP_ERR_INVALID_ARG, "ogs plan: null rowStarts (%s)", which);
  if (rs[0] != 0) return fail(SP_ERR_CSR, "ogs plan: rowStarts[0] != 0 (%s)", which);
  int32_t bad = std::numeric_limits<int32_t>::max(), mx = maxRow;
#pragma omp parallel for schedule(static) reduction(min : bad) reduction(max : mx)
  for (int32_t r = 0; r < nrows; ++r) {
    const int32_t len = rs[r + 1] - rs[r];
    if (len < 0 || len > kOgsMaxRowSize)
      bad = std::min(bad, r);
    else
      mx = std::max(mx, len);
  }
  if (bad != std::numeric_limits<int32_t>::max()) {
    const int32_t len = rs[bad + 1] - rs[bad];
    if (len < 0)
      return fail(SP_ERR_CSR, "ogs plan: rowStarts not monotone at %d (%s)", bad, which);
    return fail(SP_ERR_SIZE,
                "Multiplicity of a global node in ogsOperator_t::setupRowBlocks is too large "
                "(row %d has %d > %d members, %s)",
                bad, len, kOgsMaxRowSize, which);
  }
  maxRow = mx;
  const int32_t nnz = rs[nrows];
  if (nnz > 0 && !ids) return fail(SP_ERR_INVALID_ARG, "ogs plan: null colIds (%s)", which);
#pragma omp parallel for schedule(static) reduction(min : bad)
  for (int32_t i = 0; i < nnz; ++i)
    if (ids[i] < 0 || ids[i] >= N) bad = std::min(bad, i);
  if (bad != std::numeric_limits<int32_t>::max())
    return fail(SP_ERR_CSR, "ogs plan: colIds[%d]=%d outside [0,%d) (%s)", bad, ids[bad], N, which);
  return SP_SUCCESS;
}

static void free_plan_device(sp_ogs_plan* p) {
  if (p->own_n_csr) {
    if (p->d_rowStartsNpad) cudaFree(p->d_rowStartsNpad);
    if (p->d_colIdsN) cudaFree(p->d_colIdsN);
  }
  if (p->own_blocks_n && p->d_blocksN) cudaFree(p->d_blocksN);
  if (p->own_chunks_n && p->d_chunksN) cudaFree(p->d_chunksN);
  if (p->d_chunksT) cudaFree(p->d_chunksT);
  p->d_chunksT = p->d_chunksN = nullptr;
  p->nchunksT = p->nchunksN = 0;
  p->own_chunks_n = false;
  if (p->d_rowsGT) cudaFree(p->d_rowsGT);
  if (p->d_colIdsGT) cudaFree(p->d_colIdsGT);
  p->d_rowsGT = p->d_colIdsGT = nullptr;
  p->row_order = 0;
  if (p->d_colIdsST) cudaFree(p->d_colIdsST);
  if (p->d_rowOfST) cudaFree(p->d_rowOfST);
  if (p->d_e2sT) cudaFree(p->d_e2sT);
  if (p->d_walkRsT) cudaFree(p->d_walkRsT);
  if (p->d_walkCiT) cudaFree(p->d_walkCiT);
  if (p->d_permT) cudaFree(p->d_permT);
  p->d_walkRsT = p->d_walkCiT = p->d_permT = nullptr;
  if (p->d_rowOfColT) cudaFree(p->d_rowOfColT);
  p->d_rowOfColT = nullptr;
  if (p->d_pagesT) cudaFree(p->d_pagesT);
  p->d_pagesT = nullptr;
  p->npagesT = 0;
  if (p->d_chunksGS) cudaFree(p->d_chunksGS);
  if (p->d_rsGS) cudaFree(p->d_rsGS);
  if (p->d_ciGS) cudaFree(p->d_ciGS);
  p->d_chunksGS = p->d_rsGS = p->d_ciGS = nullptr;
  p->nchunksGS = p->gs_grouped = 0;
  if (p->d_waitErr) cudaFree(p->d_waitErr);
  p->d_waitErr = nullptr;
  for (int32_t* q : {p->d_slabsT, p->d_slabIdsT, p->d_slabRowsT, p->d_slabsGS, p->d_slabIdsGS,
                     p->d_slabTabsT, p->d_slabTdT, p->d_slabTabsGS, p->d_slabTdGS})
    if (q) cudaFree(q);
  for (int32_t* q : {p->d_slabRowTabsT, p->d_slabRowTdT})
    if (q) cudaFree(q);
  if (p->d_slabRowCodesT) cudaFree(p->d_slabRowCodesT);
  p->d_slabRowCodesT = nullptr;
  p->d_slabRowTabsT = p->d_slabRowTdT = nullptr;
  p->slab_coded_rows = 0;
  for (uint16_t* q : {p->d_slabCodesT, p->d_slabCodesGS})
    if (q) cudaFree(q);
  p->d_slabsT = p->d_slabIdsT = p->d_slabRowsT = p->d_slabsGS = p->d_slabIdsGS = nullptr;
  p->d_slabTabsT = p->d_slabTdT = p->d_slabTabsGS = p->d_slabTdGS = nullptr;
  p->d_slabCodesT = p->d_slabCodesGS = nullptr;
  p->nslabsT = p->nslabsGS = 0;
  p->slab_code_shift = 0;
  p->slab_coded_entries = 0;
  if (p->d_singT) cudaFree(p->d_singT);
  if (p->d_singGS) cudaFree(p->d_singGS);
  p->d_singT = p->d_singGS = nullptr;
  p->d_colIdsST = nullptr;
  p->d_rowOfST = p->d_e2sT = nullptr;
  int32_t* ptrs[] = {p->d_rowStartsT, p->d_colIdsT, p->d_blocksT};
  for (int32_t* q : ptrs)
    if (q) cudaFree(q);
  p->d_rowStartsT = p->d_colIdsT = p->d_blocksT = nullptr;
  p->d_rowStartsNpad = p->d_colIdsN = p->d_blocksN = nullptr;
  p->own_n_csr = p->own_blocks_n = false;
}

template <typename E>
static sp_status upload(const std::vector<E>& h, E** d, cudaStream_t s) {
  // 16 bytes of slack past the end: kernel 6 copies the 16-byte aligned span
  // around a chunk's column ids, which may reach up to 12 bytes beyond the last id
  const size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(E) + 16;
  if (cudaMalloc(d, bytes) != cudaSuccess) {
    cudaGetLastError();
    *d = nullptr;
    return fail(SP_ERR_ALLOC, "ogs plan: cudaMalloc of %zu bytes failed", bytes);
  }
  if (!h.empty())
    SP_CUDA_TRY(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(E), cudaMemcpyHostToDevice, s));
  return SP_SUCCESS;
}

// Finishes a plan whose host CSR arrays are filled: validation, partition, upload.
// The gather+scatter walk (knob ogs.gs_order >= 0): a second chunking of T in its
// own order (pages of 2^ogs.gs_page_shift entries, balls of 2^ogs.gs_ball_shift),
// with rows grouped by size when ogs.rows is 1.  The in-place gather+scatter then
// need not share the walk that suits the gathers (measured on the permuted 64^3
// p=7 box: gathers fastest on breadth-first pages of 512 entries, gather+scatter on
// a renumbered walk of 256-entry pages in balls of 2^18 entries).
// Per chunk (r0, r1, g0, g1): the number of its rows with more than one member and
// their entries -- with rows grouped by size (largest first) those rows and
// entries come first, the single-member rows after them.
static std::vector<int32_t> singleton_split(const std::vector<int32_t>& quads,
                                            const int32_t* rs) {
  const int64_t nchunks = (int64_t)quads.size() / 4;
  std::vector<int32_t> out(2 * std::max<int64_t>(nchunks, 1), 0);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nchunks; ++c) {
    int32_t k0 = 0, s0 = 0;
    for (int32_t r = quads[4 * c]; r < quads[4 * c + 1]; ++r) {
      const int32_t n = rs[r + 1] - rs[r];
      if (n > 1) {
        ++k0;
        s0 += n;
      }
    }
    out[2 * c] = k0;
    out[2 * c + 1] = s0;
  }
  return out;
}

// Slab layout of one walk (build_slabs), uploaded; `rows_out` null for a walk that
// only serves the in-place gather+scatter.  With ogs.slab_code_shift > 0 also the
// 16-bit codes of the slabs that compress (compress_slabs) and, for a gather walk
// with ogs.slab_row_codes, those of its row words (compress_slab_rows).
static sp_status build_slab_layout(sp_ogs_plan* p, const std::vector<int32_t>& quads,
                                   const int32_t* wrs, const int32_t* wci, const int32_t* perm,
                                   bool with_rows, int32_t** desc_out, int32_t** ids_out,
                                   int32_t** rows_out, int32_t* nslabs, uint16_t** codes_out,
                                   int32_t** tabs_out, int32_t** td_out, cudaStream_t s) {
  std::vector<int32_t> desc, ids, rows;
  build_slabs(quads, wrs, wci, perm, (int)tune(kTuneOgsSlabSegShift), with_rows, desc, ids,
              rows);
  // The kernel addresses ids with 32-bit offsets; a walk whose padded slabs pass
  // 2^31 - 1 words keeps no slabs and its launches run kernel 2.
  if (ids.size() > (size_t)INT32_MAX) return SP_SUCCESS;
  sp_status st;
  if ((st = upload(desc, desc_out, s))) return st;
  if ((st = upload(ids, ids_out, s))) return st;
  if (rows_out && (st = upload(rows, rows_out, s))) return st;
  *nslabs = (int32_t)(desc.size() / 4);
  const int shift = (int)tune(kTuneOgsSlabCodeShift);
  if (shift > 0 && *nslabs > 0) {
    std::vector<uint16_t> codes;
    std::vector<int32_t> tabs, td;
    compress_slabs(desc, ids, shift, codes, tabs, td);
    if ((st = upload(codes, codes_out, s))) return st;
    if ((st = upload(tabs, tabs_out, s))) return st;
    if ((st = upload(td, td_out, s))) return st;
    p->slab_code_shift = shift;
    for (int32_t g = 0; g < *nslabs; ++g)
      if (td[2 * g + 1] > 0) {
        const int32_t w = desc[4 * g + 3];
        p->slab_coded_entries +=
            (int64_t)(((w >> 16) - 1) * (w & 255) + ((w >> 8) & 255)) * desc[4 * g + 2];
      }
    if (with_rows && tune(kTuneOgsSlabRowCodes) == 1) {
      std::vector<uint16_t> rcodes;
      std::vector<int32_t> rtabs, rtd;
      compress_slab_rows(desc, rows, shift, rcodes, rtabs, rtd);
      if ((st = upload(rcodes, &p->d_slabRowCodesT, s))) return st;
      if ((st = upload(rtabs, &p->d_slabRowTabsT, s))) return st;
      if ((st = upload(rtd, &p->d_slabRowTdT, s))) return st;
      for (int32_t g = 0; g < *nslabs; ++g)
        if (rtd[2 * g + 1] > 0) {
          const int32_t w = desc[4 * g + 3];
          p->slab_coded_rows += (int64_t)((w >> 16) - 1) * (w & 255) + ((w >> 8) & 255);
        }
      SP_CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors die with this scope
    }
  }
  SP_CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors die with this scope
  return SP_SUCCESS;
}

static sp_status build_gs_walk(sp_ogs_plan* p, cudaStream_t s) {
  const int order = (int)tune(kTuneOgsGsOrder);
  if (order < 0 || p->nchunksT == 0) return SP_SUCCESS;
  const int shift = (int)tune(kTuneOgsGsPageShift), ball = (int)tune(kTuneOgsGsBallShift);
  std::vector<int32_t> perm, walkRs, walkCi, pairs;
  const int32_t* wrs = p->rowStartsT.data();
  const int32_t* wci = p->colIdsT.data();
  if (order == 2) {
    bfs_row_sequence(p->NrowsT, wrs, wci, p->N, shift, ball, perm);
    walkRs.assign((size_t)p->NrowsT + 1, 0);
    for (int32_t k = 0; k < p->NrowsT; ++k)
      walkRs[k + 1] = walkRs[k] + (p->rowStartsT[perm[k] + 1] - p->rowStartsT[perm[k]]);
    walkCi.resize(p->nnzT);
#pragma omp parallel for schedule(static)
    for (int32_t k = 0; k < p->NrowsT; ++k)
      std::copy(p->colIdsT.begin() + p->rowStartsT[perm[k]],
                p->colIdsT.begin() + p->rowStartsT[perm[k] + 1], walkCi.begin() + walkRs[k]);
    wrs = walkRs.data();
    wci = walkCi.data();
  }
  if (!build_chunks(p->NrowsT, wrs, wci, p->N, order == 2 ? 0 : order, pairs, shift, ball))
    return SP_SUCCESS;
  std::vector<int32_t> quads(pairs.size() * 2);
  for (size_t c = 0; c < pairs.size() / 2; ++c) {
    quads[4 * c + 0] = pairs[2 * c];
    quads[4 * c + 1] = pairs[2 * c + 1];
    quads[4 * c + 2] = wrs[pairs[2 * c]];
    quads[4 * c + 3] = wrs[pairs[2 * c + 1]];
  }
  sp_status st;
  if ((st = upload(quads, &p->d_chunksGS, s))) return st;
  if (tune(kTuneOgsRows) == 1) {
    std::vector<int32_t> rowsG, colIdsG;
    build_grouped(quads, p->NrowsT, wrs, wci, rowsG, colIdsG);
    if ((st = upload(rowsG, &p->d_rsGS, s))) return st;
    if ((st = upload(colIdsG, &p->d_ciGS, s))) return st;
    p->gs_grouped = 1;
    if ((st = upload(singleton_split(quads, wrs), &p->d_singGS, s))) return st;
  } else if (order == 2) {
    if ((st = upload(walkRs, &p->d_rsGS, s))) return st;
    if ((st = upload(walkCi, &p->d_ciGS, s))) return st;
  }
  p->nchunksGS = (int32_t)(quads.size() / 4);
  if (tune(kTuneOgsSlabs) == 1 &&
      (st = build_slab_layout(p, quads, wrs, wci, nullptr, false, &p->d_slabsGS,
                              &p->d_slabIdsGS, nullptr, &p->nslabsGS, &p->d_slabCodesGS,
                              &p->d_slabTabsGS, &p->d_slabTdGS, s)))
    return st;
  SP_CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors die with this scope
  return SP_SUCCESS;
}

sp_status finalize_plan(sp_ogs_plan* p, cudaStream_t s) {
  int32_t maxRow = 0;
  sp_status st = validate_csr(p->N, p->NrowsT, p->rowStartsT.data(), p->colIdsT.data(), "T",
                              maxRow);
  if (st) return st;
  p->nnzT = p->rowStartsT[p->NrowsT];
  if (!p->n_is_t) {
    if (p->NrowsN > p->NrowsT)
      return fail(SP_ERR_CSR, "ogs plan: NrowsN %d > NrowsT %d", p->NrowsN, p->NrowsT);
    st = validate_csr(p->N, p->NrowsN, p->rowStartsN.data(), p->colIdsN.data(), "N", maxRow);
    if (st) return st;
    p->nnzN = p->rowStartsN[p->NrowsN];
    // every column at most once in T, and N's members of a row inside T's row
    std::vector<int32_t> rowOf(std::max(p->N, 1), -1);
    int32_t dup = std::numeric_limits<int32_t>::max();
    const int32_t* rsT = p->rowStartsT.data();
    const int32_t* ciT = p->colIdsT.data();
#pragma omp parallel for schedule(static) reduction(min : dup)
    for (int32_t r = 0; r < p->NrowsT; ++r)
      for (int32_t i = rsT[r]; i < rsT[r + 1]; ++i) {
        int32_t prev;
#pragma omp atomic capture
        {
          prev = rowOf[ciT[i]];
          rowOf[ciT[i]] = r;
        }
        if (prev != -1) dup = std::min(dup, ciT[i]);
      }
    if (dup != std::numeric_limits<int32_t>::max())
      return fail(SP_ERR_CSR, "ogs plan: column %d appears in two rows", dup);
    int32_t badRow = std::numeric_limits<int32_t>::max();
    const int32_t* rsN = p->rowStartsN.data();
    const int32_t* ciN = p->colIdsN.data();
#pragma omp parallel for schedule(static) reduction(min : badRow)
    for (int32_t r = 0; r < p->NrowsN; ++r)
      for (int32_t i = rsN[r]; i < rsN[r + 1]; ++i)
        if (rowOf[ciN[i]] != r) badRow = std::min(badRow, r);
    if (badRow != std::numeric_limits<int32_t>::max())
      return fail(SP_ERR_CSR, "ogs plan: an N column of row %d is not in T row %d", badRow,
                  badRow);
  } else {
    std::vector<uint8_t> seen(std::max(p->N, 1), 0);
    int32_t dup = std::numeric_limits<int32_t>::max();
    const int32_t* ciT = p->colIdsT.data();
#pragma omp parallel for schedule(static) reduction(min : dup)
    for (int32_t i = 0; i < p->nnzT; ++i) {
      uint8_t prev;
#pragma omp atomic capture
      {
        prev = seen[ciT[i]];
        seen[ciT[i]] = 1;
      }
      if (prev) dup = std::min(dup, ciT[i]);
    }
    if (dup != std::numeric_limits<int32_t>::max())
      return fail(SP_ERR_CSR, "ogs plan: column %d appears in two rows", dup);
    p->NrowsN = std::min(p->NrowsN, p->NrowsT);
    p->rowStartsN.assign(p->rowStartsT.begin(), p->rowStartsT.begin() + p->NrowsN + 1);
    p->colIdsN.assign(p->colIdsT.begin(), p->colIdsT.begin() + p->rowStartsN[p->NrowsN]);
    p->nnzN = p->rowStartsN[p->NrowsN];
  }
  p->maxRowSize = maxRow;

  // N partition: rows [0, NrowsN) of the N operator (which is T itself when
  // n_is_t, e.g. for an Unsigned handle whose flagged-only groups follow).
  std::vector<int32_t> blocksT, blocksN;
  if (!partition_rows(p->NrowsT, p->rowStartsT.data(), blocksT) ||
      !partition_rows(p->NrowsN, p->rowStartsN.data(), blocksN))
    return fail(SP_ERR_SIZE, "ogs plan: a row exceeds the block capacity %d", kOgsBlockNnz);
  p->NrowBlocksT = std::max<int32_t>(0, (int32_t)blocksT.size() - 1);
  p->NrowBlocksN = std::max<int32_t>(0, (int32_t)blocksN.size() - 1);

  SP_CUDA_TRY(cudaGetDevice(&p->device));
  if ((st = upload(p->rowStartsT, &p->d_rowStartsT, s))) return st;
  if ((st = upload(p->colIdsT, &p->d_colIdsT, s))) return st;
  if ((st = upload(blocksT, &p->d_blocksT, s))) return st;
  if (p->n_is_t) {
    p->d_rowStartsNpad = p->d_rowStartsT;
    p->d_colIdsN = p->d_colIdsT;
  } else {
    std::vector<int32_t> pad(p->rowStartsN);
    pad.resize(p->NrowsT + 1, p->nnzN);  // rows without a positive member are empty
    p->own_n_csr = true;
    if ((st = upload(pad, &p->d_rowStartsNpad, s))) return st;
    if ((st = upload(p->colIdsN, &p->d_colIdsN, s))) return st;
  }
  if (p->NrowsN == p->NrowsT && (p->n_is_t || blocksN == blocksT)) {
    p->d_blocksN = p->d_blocksT;
  } else {
    p->own_blocks_n = true;
    if ((st = upload(blocksN, &p->d_blocksN, s))) return st;
  }
  // warp chunks (only when every row fits one chunk): T in the chosen order; N,
  // whose rows hold at most one member after a unique setup, in row order.  Order 2
  // walks a copy of T whose rows are renumbered in breadth-first page order (the
  // rows of each page in turn), so chunks are full and follow the mesh whatever the
  // element numbering; perm maps a walk row back to its row of T.
  p->chunk_order = (int32_t)tune(kTuneOgsOrder);
  const int page_shift = (int)tune(kTuneOgsPageShift);
  const int ball_shift = (int)tune(kTuneOgsBallShift);
  const bool renumber = p->chunk_order == 2;
  std::vector<int32_t> walkRs, walkCi, perm, pages;
  const int32_t* wrs = p->rowStartsT.data();
  const int32_t* wci = p->colIdsT.data();
  std::vector<int32_t> chunksT, chunksN;
  bool fits = true;
  if (renumber) {
    int32_t tooBig = 0;
#pragma omp parallel for schedule(static) reduction(max : tooBig)
    for (int32_t r = 0; r < p->NrowsT; ++r)
      if (p->rowStartsT[r + 1] - p->rowStartsT[r] > kWarpChunkNnz) tooBig = 1;
    fits = !tooBig;
    if (fits) {
      bfs_row_sequence(p->NrowsT, wrs, wci, p->N, page_shift, ball_shift, perm, &pages);
      walkRs.assign((size_t)p->NrowsT + 1, 0);
      for (int32_t k = 0; k < p->NrowsT; ++k)
        walkRs[k + 1] = walkRs[k] + (p->rowStartsT[perm[k] + 1] - p->rowStartsT[perm[k]]);
      walkCi.resize(p->nnzT);
#pragma omp parallel for schedule(static)
      for (int32_t k = 0; k < p->NrowsT; ++k)
        std::copy(p->colIdsT.begin() + p->rowStartsT[perm[k]],
                  p->colIdsT.begin() + p->rowStartsT[perm[k] + 1], walkCi.begin() + walkRs[k]);
      wrs = walkRs.data();
      wci = walkCi.data();
      fits = build_chunks(p->NrowsT, wrs, wci, p->N, 0, chunksT, page_shift, ball_shift);
    }
  } else {
    fits = build_chunks(p->NrowsT, wrs, wci, p->N, p->chunk_order, chunksT, page_shift,
                        ball_shift, p->chunk_order == 1 ? &pages : nullptr);
  }
  if (fits && build_chunks(p->NrowsN, p->rowStartsN.data(), p->colIdsN.data(), p->N, 0, chunksN,
                           page_shift, 0)) {
    p->nchunksT = (int32_t)(chunksT.size() / 2);
    p->nchunksN = (int32_t)(chunksN.size() / 2);
    // descriptors (r0, r1, g0, g1): the entry range rides along with the row range
    auto quads = [](const std::vector<int32_t>& pairs, const int32_t* rs) {
      std::vector<int32_t> q(pairs.size() * 2);
      for (size_t c = 0; c < pairs.size() / 2; ++c) {
        q[4 * c + 0] = pairs[2 * c];
        q[4 * c + 1] = pairs[2 * c + 1];
        q[4 * c + 2] = rs[pairs[2 * c]];
        q[4 * c + 3] = rs[pairs[2 * c + 1]];
      }
      return q;
    };
    // N shares T's descriptors only when row AND entry ranges agree (equal row
    // ranges alone are not enough: N rows keep only the positive members)
    chunksT = quads(chunksT, wrs);
    chunksN = quads(chunksN, p->rowStartsN.data());
    const bool same = !renumber && (chunksN == chunksT);
    if ((st = upload(chunksT, &p->d_chunksT, s))) return st;
    if (same) {
      p->d_chunksN = p->d_chunksT;
    } else {
      p->own_chunks_n = true;
      if ((st = upload(chunksN, &p->d_chunksN, s))) return st;
    }
    if (renumber) {
      if ((st = upload(walkRs, &p->d_walkRsT, s))) return st;
      if ((st = upload(walkCi, &p->d_walkCiT, s))) return st;
      if ((st = upload(perm, &p->d_permT, s))) return st;
    }
    // T rows grouped by size inside each chunk (the N operator keeps CSR order)
    std::vector<int32_t> rowsG, colIdsG;
    if (tune(kTuneOgsRows) == 1 && p->nchunksT > 0) {
      build_grouped(chunksT, p->NrowsT, wrs, wci, rowsG, colIdsG);
      if ((st = upload(rowsG, &p->d_rowsGT, s))) return st;
      if ((st = upload(singleton_split(chunksT, wrs), &p->d_singT, s))) return st;
      if ((st = upload(colIdsG, &p->d_colIdsGT, s))) return st;
      p->row_order = 1;
    }
    // lane-row slabs of the main walk (kernel 7)
    if (tune(kTuneOgsSlabs) == 1 && p->nchunksT > 0 &&
        (st = build_slab_layout(p, chunksT, wrs, wci, renumber ? perm.data() : nullptr, true,
                                &p->d_slabsT, &p->d_slabIdsT, &p->d_slabRowsT, &p->nslabsT,
                                &p->d_slabCodesT, &p->d_slabTabsT, &p->d_slabTdT, s)))
      return st;
    // T chunk entries in column order: the column-order scatter and gathers
    std::vector<int32_t> colS;
    std::vector<uint8_t> rowOf, e2s;
    build_sorted(chunksT, p->NrowsT, wrs, p->row_order == 1 ? rowsG.data() : nullptr,
                 p->row_order == 1 ? colIdsG.data() : wci, colS, rowOf, e2s);
    if ((st = upload(colS, &p->d_colIdsST, s))) return st;
    if ((st = upload(rowOf, &p->d_rowOfST, s))) return st;
    if ((st = upload(e2s, &p->d_e2sT, s))) return st;
    // the row of each local column, for the column-major scatter
    std::vector<int32_t> rowOfCol(std::max(p->N, 1), -1);
#pragma omp parallel for schedule(static)
    for (int32_t r = 0; r < p->NrowsT; ++r)
      for (int32_t i = p->rowStartsT[r]; i < p->rowStartsT[r + 1]; ++i) rowOfCol[p->colIdsT[i]] = r;
    if ((st = upload(rowOfCol, &p->d_rowOfColT, s))) return st;
    // the walk-ordered scatter stores each page it is given, so it runs only when
    // the list holds every page of [0, N) (exactly once, as page_order emits them)
    const int64_t npages_all = (std::max<int64_t>(p->N, 1) + (1LL << page_shift) - 1) >> page_shift;
    if (!pages.empty() && (int64_t)pages.size() == npages_all) {
      p->npagesT = (int32_t)pages.size();
      p->pages_shift = page_shift;
      if ((st = upload(pages, &p->d_pagesT, s))) return st;
    }
    if ((st = upload(std::vector<int32_t>{0}, &p->d_waitErr, s))) return st;
    if ((st = build_gs_walk(p, s))) return st;
    SP_CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors die with this scope
  } else {
    p->nchunksT = p->nchunksN = 0;
  }
  SP_CUDA_TRY(cudaStreamSynchronize(s));
  return SP_SUCCESS;
}

}  // namespace sp

using namespace sp;

extern "C" {

int32_t sp_ogs_block_nnz(void) { return kOgsBlockNnz; }

sp_status sp_ogs_plan_create(int32_t N, int32_t NrowsT, const int32_t* h_rowStartsT,
                             const int32_t* h_colIdsT, int32_t NrowsN, const int32_t* h_rowStartsN,
                             const int32_t* h_colIdsN, sp_stream_t stream, sp_ogs_plan** out) {
  if (!out) return fail(SP_ERR_INVALID_ARG, "sp_ogs_plan_create: null out");
  *out = nullptr;
  if (N < 0 || NrowsT < 0 || !h_rowStartsT)
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_plan_create: bad sizes or null rowStartsT");
  sp_ogs_plan* p = new sp_ogs_plan();
  p->N = N;
  p->NrowsT = NrowsT;
  p->rowStartsT.assign(h_rowStartsT, h_rowStartsT + NrowsT + 1);
  const int32_t nnzT = h_rowStartsT[NrowsT];
  if (nnzT < 0) {
    delete p;
    return fail(SP_ERR_CSR, "sp_ogs_plan_create: negative nnz");
  }
  if (nnzT > 0 && !h_colIdsT) {
    delete p;
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_plan_create: null colIdsT");
  }
  p->colIdsT.assign(h_colIdsT, h_colIdsT + nnzT);
  if (h_rowStartsN) {
    if (NrowsN < 0) {
      delete p;
      return fail(SP_ERR_INVALID_ARG, "sp_ogs_plan_create: negative NrowsN");
    }
    p->n_is_t = false;
    p->NrowsN = NrowsN;
    p->rowStartsN.assign(h_rowStartsN, h_rowStartsN + NrowsN + 1);
    const int32_t nnzN = h_rowStartsN[NrowsN];
    if (nnzN < 0 || (nnzN > 0 && !h_colIdsN)) {
      delete p;
      return fail(SP_ERR_CSR, "sp_ogs_plan_create: bad N operator");
    }
    p->colIdsN.assign(h_colIdsN, h_colIdsN + nnzN);
  } else {
    p->n_is_t = true;
    p->NrowsN = (NrowsN >= 0 && NrowsN <= NrowsT) ? NrowsN : NrowsT;
  }
  sp_status st = finalize_plan(p, as_cuda(stream));
  if (st) {
    free_plan_device(p);
    delete p;
    return st;
  }
  *out = p;
  return SP_SUCCESS;
}

sp_status sp_ogs_plan_destroy(sp_ogs_plan* p) {
  if (!p) return SP_SUCCESS;
  free_plan_device(p);
  delete p;
  return SP_SUCCESS;
}

sp_status sp_ogs_plan_info(const sp_ogs_plan* p, sp_ogs_info* info) {
  if (!p || !info) return fail(SP_ERR_INVALID_ARG, "sp_ogs_plan_info: null argument");
  info->N = p->N;
  info->NrowsT = p->NrowsT;
  info->NrowsN = p->NrowsN;
  info->nnzT = p->nnzT;
  info->nnzN = p->nnzN;
  info->NrowBlocksT = p->NrowBlocksT;
  info->NrowBlocksN = p->NrowBlocksN;
  info->maxRowSize = p->maxRowSize;
  info->NgatherGlobal = p->NrowsN;
  info->NchunksT = p->nchunksT;
  info->NchunksN = p->nchunksN;
  info->chunkOrder = p->chunk_order;
  info->rowOrder = p->row_order;
  info->NchunksGS = p->nchunksGS;
  info->gsRowOrder = p->gs_grouped;
  info->NpagesT = p->npagesT;
  info->pageShift = p->pages_shift;
  info->NslabsT = p->nslabsT;
  info->NslabsGS = p->nslabsGS;
  info->slabCodeShift = p->slab_code_shift;
  info->slabCodedEntries = p->slab_coded_entries;
  info->slabCodedRows = p->slab_coded_rows;
  info->waitErrors = 0;
  if (p->d_waitErr) {
    int32_t* dev = p->d_waitErr;
    SP_CUDA_TRY(cudaMemcpy(&info->waitErrors, dev, sizeof(int32_t), cudaMemcpyDeviceToHost));
  }
  return SP_SUCCESS;
}

sp_status sp_ogs_plan_csr(const sp_ogs_plan* p, sp_transpose which, int32_t* rs, int32_t* ids) {
  if (!p) return fail(SP_ERR_INVALID_ARG, "sp_ogs_plan_csr: null plan");
  const std::vector<int32_t>& R = (which == SP_NOTRANS) ? p->rowStartsN : p->rowStartsT;
  const std::vector<int32_t>& C = (which == SP_NOTRANS) ? p->colIdsN : p->colIdsT;
  if (rs) std::memcpy(rs, R.data(), R.size() * sizeof(int32_t));
  if (ids && !C.empty()) std::memcpy(ids, C.data(), C.size() * sizeof(int32_t));
  return SP_SUCCESS;
}

sp_status sp_ogs_gather_scatter(const sp_ogs_plan* p, sp_type type, sp_op op, sp_transpose trans,
                                int32_t k, void* v, sp_stream_t stream) {
  sp_status st = check_common(p, type, op, trans, k, "sp_ogs_gather_scatter");
  if (st) return st;
  if (p->nnzT > 0 && !v) return fail(SP_ERR_INVALID_ARG, "sp_ogs_gather_scatter: null vector");
  if (p->NrowBlocksT == 0) return SP_SUCCESS;
  cudaStream_t s = as_cuda(stream);
  switch (type) {
    case SP_FLOAT: by_op<GsF, float>(op, p, trans, (int)k, v, s); break;
    case SP_DOUBLE: by_op<GsF, double>(op, p, trans, (int)k, v, s); break;
    case SP_INT32: by_op<GsF, int32_t>(op, p, trans, (int)k, v, s); break;
    case SP_INT64: by_op<GsF, long long>(op, p, trans, (int)k, v, s); break;
  }
  return check_launch("sp_ogs_gather_scatter");
}

sp_status sp_ogs_gather(const sp_ogs_plan* p, sp_type type, sp_op op, sp_transpose trans,
                        int32_t k, void* gv, const void* v, sp_stream_t stream) {
  sp_status st = check_common(p, type, op, trans, k, "sp_ogs_gather");
  if (st) return st;
  const int32_t nb = (trans == SP_NOTRANS) ? p->NrowBlocksN : p->NrowBlocksT;
  if (nb == 0) return SP_SUCCESS;
  if (!v || !gv) return fail(SP_ERR_INVALID_ARG, "sp_ogs_gather: null vector");
  cudaStream_t s = as_cuda(stream);
  switch (type) {
    case SP_FLOAT: by_op<GatherF, float>(op, p, trans, (int)k, gv, v, s); break;
    case SP_DOUBLE: by_op<GatherF, double>(op, p, trans, (int)k, gv, v, s); break;
    case SP_INT32: by_op<GatherF, int32_t>(op, p, trans, (int)k, gv, v, s); break;
    case SP_INT64: by_op<GatherF, long long>(op, p, trans, (int)k, gv, v, s); break;
  }
  return check_launch("sp_ogs_gather");
}

sp_status sp_ogs_scatter(const sp_ogs_plan* p, sp_type type, sp_transpose trans, int32_t k,
                         void* v, const void* gv, sp_stream_t stream) {
  sp_status st = check_common(p, type, SP_OP_ADD, trans, k, "sp_ogs_scatter");
  if (st) return st;
  const int32_t nb = (trans == SP_TRANS) ? p->NrowBlocksN : p->NrowBlocksT;
  if (nb == 0) return SP_SUCCESS;
  if (!v || !gv) return fail(SP_ERR_INVALID_ARG, "sp_ogs_scatter: null vector");
  cudaStream_t s = as_cuda(stream);
  switch (type) {
    case SP_FLOAT: launch_scatter<float>(p, trans, k, (float*)v, (const float*)gv, s); break;
    case SP_DOUBLE: launch_scatter<double>(p, trans, k, (double*)v, (const double*)gv, s); break;
    case SP_INT32: launch_scatter<int32_t>(p, trans, k, (int32_t*)v, (const int32_t*)gv, s); break;
    case SP_INT64:
      launch_scatter<long long>(p, trans, k, (long long*)v, (const long long*)gv, s);
      break;
  }
  return check_launch("sp_ogs_scatter");
}

}  // extern "C"
