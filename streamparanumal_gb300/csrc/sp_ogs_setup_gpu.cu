// Gather-scatter setup on the device.  The same grouping, unique-owner choice, row
// numbering and CSR as the host setup (sp_ogs_setup.cpp, after ogsBase_t::Setup,
// libs/ogs/ogsSetup.cpp:87-290 and EnumerateGatherGroups/SortByRow :492-579), from
// global ids that are already in device memory:
//   1. (|id|, local index) pairs of the non-zero ids are radix-sorted by |id|; the
//      sort is stable, so each group's members come out in ascending local index;
//   2. group heads -> scan -> group numbers and offsets;
//   3. unique: group n (ascending |id|) takes draw n of the reference's LCG stream
//      (random.cpp:47-172, seed 0), reached by jumping the affine recurrence ahead
//      n steps instead of stepping through it;
//   4. rows: the first member of every group is flagged in local-index space, and
//      two exclusive scans rank the groups with and without a positive member by
//      first appearance;
//   5. row starts by an exclusive scan of the group sizes in row order; every
//      sorted pair then lands at its CSR slot; the N operator keeps the positive
//      members of the first NrowsP rows.
// The CSR comes back to the host once and the plan is finished as any other.
// CUB (CCCL, part of the CUDA toolkit) does the radix sort and scans of this
// once-per-mesh setup; no BS kernel uses it.
#include <cub/cub.cuh>

#include <vector>

#include "sp_ogs_plan.h"

namespace sp {
namespace {

constexpr int kSetupThreads = 256;

__device__ __forceinline__ unsigned long long uabs(long long v) {
  return v < 0 ? 0ULL - (unsigned long long)v : (unsigned long long)v;
}

unsigned setup_grid(int64_t n) {
  const int64_t want = (n + kSetupThreads - 1) / kSetupThreads;
  const int64_t cap = (int64_t)sm_count() * 32;
  return (unsigned)(want < 1 ? 1 : (want < cap ? want : cap));
}

// stats[0] = max |id|, stats[1] = number of non-zero ids
__global__ void k_id_stats(int32_t N, const long long* __restrict__ ids,
                           unsigned long long* __restrict__ stats) {
  unsigned long long mx = 0, cnt = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const long long v = ids[i];
    if (v != 0) {
      mx = max(mx, uabs(v));
      ++cnt;
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(stats, mx);
    atomicAdd(stats + 1, cnt);
  }
}

// ignored entries (id 0) get the largest key and sort behind every group
__global__ void k_keys(int32_t N, const long long* __restrict__ ids,
                       unsigned long long* __restrict__ keys, int32_t* __restrict__ vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const long long v = ids[i];
    keys[i] = v != 0 ? uabs(v) : ~0ULL;
    vals[i] = (int32_t)i;
  }
}

__global__ void k_heads(int32_t nids, const unsigned long long* __restrict__ keys,
                        int32_t* __restrict__ head) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nids;
       j += (int64_t)gridDim.x * blockDim.x)
    head[j] = (j == 0 || keys[j] != keys[j - 1]) ? 1 : 0;
}

// gscan = inclusive scan of the heads: entry j is in group gscan[j] - 1
__global__ void k_offsets(int32_t nids, const int32_t* __restrict__ gscan, int32_t* __restrict__ off) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nids;
       j += (int64_t)gridDim.x * blockDim.x) {
    if (j == 0 || gscan[j] != gscan[j - 1]) off[gscan[j] - 1] = (int32_t)j;
    if (j == nids - 1) off[gscan[j]] = nids;
  }
}

// State of the LCG x_{k+1} = A x_k + C after n steps from x_0 = A (~0 ^ seed) + C,
// seed 0: the affine map is raised to the n-th power by squaring.
__device__ __forceinline__ unsigned long long lcg_state(unsigned long long n) {
  const unsigned long long A = 6364136223846793005ULL, C = 1ULL;
  const unsigned long long x0 = A * ~0ULL + C;
  unsigned long long ra = 1, rc = 0;  // accumulated map x -> ra x + rc
  unsigned long long pa = A, pc = C;  // map raised to the current power of two
  while (n) {
    if (n & 1) {
      rc = pa * rc + pc;
      ra = pa * ra;
    }
    pc = pa * pc + pc;
    pa = pa * pa;
    n >>= 1;
  }
  return ra * x0 + rc;
}

// unique: every member flagged negative, member draw % size made positive (none
// when the draw is INT_MIN, whose absolute value stays negative -- as on the host)
__global__ void k_unique(int32_t ngroups, const int32_t* __restrict__ off,
                         const int32_t* __restrict__ vals,
                         const unsigned long long* __restrict__ keys, long long* __restrict__ ids) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < ngroups;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = off[n], b = off[n + 1];
    const int32_t v = (int32_t)(uint32_t)lcg_state((unsigned long long)n);
    const int32_t draw = v < 0 ? (int32_t)(0u - (uint32_t)v) : v;
    const int32_t m = draw % (b - a);
    const long long key = (long long)keys[a];
    for (int32_t j = a; j < b; ++j) ids[vals[j]] = -key;
    if (m >= 0) ids[vals[a + m]] = key;
  }
}

// positive[n], and the first (smallest) member of each group flagged in local
// index space by class; npos[0] counts the groups with a positive member
__global__ void k_group_flags(int32_t ngroups, const int32_t* __restrict__ off,
                              const int32_t* __restrict__ vals, const long long* __restrict__ ids,
                              uint8_t* __restrict__ positive, int32_t* __restrict__ fpos,
                              int32_t* __restrict__ fneg, int32_t* __restrict__ npos) {
  int32_t cnt = 0;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < ngroups;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = off[n], b = off[n + 1];
    bool pos = false;
    for (int32_t j = a; j < b && !pos; ++j) pos = ids[vals[j]] > 0;
    positive[n] = pos ? 1 : 0;
    (pos ? fpos : fneg)[vals[a]] = 1;
    cnt += pos ? 1 : 0;
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(npos, cnt);
}

__global__ void k_rows(int32_t ngroups, const int32_t* __restrict__ off,
                       const int32_t* __restrict__ vals, const uint8_t* __restrict__ positive,
                       const int32_t* __restrict__ rpos, const int32_t* __restrict__ rneg,
                       int32_t NrowsP, int32_t* __restrict__ rowOf, int32_t* __restrict__ sizeByRow) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < ngroups;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t first = vals[off[n]];
    const int32_t r = positive[n] ? rpos[first] : NrowsP + rneg[first];
    rowOf[n] = r;
    sizeByRow[r] = off[n + 1] - off[n];
  }
}

__global__ void k_fill_t(int32_t nids, const int32_t* __restrict__ gscan,
                         const int32_t* __restrict__ off, const int32_t* __restrict__ rowOf,
                         const int32_t* __restrict__ rsT, const int32_t* __restrict__ vals,
                         int32_t* __restrict__ ciT) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nids;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t n = gscan[j] - 1;
    ciT[rsT[rowOf[n]] + ((int32_t)j - off[n])] = vals[j];
  }
}

__global__ void k_count_n(int32_t NrowsP, const int32_t* __restrict__ rsT,
                          const int32_t* __restrict__ ciT, const long long* __restrict__ ids,
                          int32_t* __restrict__ cntN) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < NrowsP;
       r += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = 0;
    for (int32_t i = rsT[r]; i < rsT[r + 1]; ++i) c += ids[ciT[i]] > 0 ? 1 : 0;
    cntN[r] = c;
  }
}

__global__ void k_fill_n(int32_t NrowsP, const int32_t* __restrict__ rsT,
                         const int32_t* __restrict__ ciT, const long long* __restrict__ ids,
                         const int32_t* __restrict__ rsN, int32_t* __restrict__ ciN) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < NrowsP;
       r += (int64_t)gridDim.x * blockDim.x) {
    int32_t nn = rsN[r];
    for (int32_t i = rsT[r]; i < rsT[r + 1]; ++i)
      if (ids[ciT[i]] > 0) ciN[nn++] = ciT[i];
  }
}

// Box-mesh global ids on the device (the lattice rule of sp_mesh_box_hex_ids): node
// (i, j, k) of lexicographic element (ex, ey, ez) lies on lattice point
// (ex p + i, ey p + j, ez p + k); its id is 1 + the smallest local index over the
// (up to 8) element nodes on that point, each element stored at its slot.
__device__ __forceinline__ int axis_options(int32_t ec, int32_t lc, int32_t ne, int32_t p,
                                            int32_t (&oe)[2], int32_t (&ol)[2]) {
  if (lc == 0 && ec > 0) {
    oe[0] = ec - 1; ol[0] = p; oe[1] = ec; ol[1] = 0;
    return 2;
  }
  if (lc == p && ec < ne - 1) {
    oe[0] = ec; ol[0] = p; oe[1] = ec + 1; ol[1] = 0;
    return 2;
  }
  oe[0] = ec; ol[0] = lc;
  return 1;
}

__global__ void k_box_ids(int32_t nx, int32_t ny, int32_t nz, int32_t p,
                          const int32_t* __restrict__ slot, long long* __restrict__ ids) {
  const int32_t Nq = p + 1;
  const int64_t Np = (int64_t)Nq * Nq * Nq;
  const int64_t total = (int64_t)nx * ny * nz * Np;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / Np;
    const int32_t n = (int32_t)(t - e * Np);
    const int32_t i = n % Nq, j = (n / Nq) % Nq, k = n / (Nq * Nq);
    const int32_t ex = (int32_t)(e % nx), ey = (int32_t)((e / nx) % ny);
    const int32_t ez = (int32_t)(e / ((int64_t)nx * ny));
    int32_t xe[2], xl[2], ye[2], yl[2], ze[2], zl[2];
    const int nxo = axis_options(ex, i, nx, p, xe, xl);
    const int nyo = axis_options(ey, j, ny, p, ye, yl);
    const int nzo = axis_options(ez, k, nz, p, ze, zl);
    long long best = 0x7fffffffffffffffLL;
    for (int c = 0; c < nzo; ++c)
      for (int b = 0; b < nyo; ++b)
        for (int a = 0; a < nxo; ++a) {
          const int64_t e2 = xe[a] + (int64_t)ye[b] * nx + (int64_t)ze[c] * nx * ny;
          const long long l = (long long)slot[e2] * Np + xl[a] + yl[b] * Nq + zl[c] * Nq * Nq;
          best = l < best ? l : best;
        }
    ids[(int64_t)slot[e] * Np + n] = 1 + best;
  }
}

// Device scratch freed on every exit path.
struct Scratch {
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename E>
  cudaError_t get(E** p, size_t n) {
    *p = nullptr;
    const cudaError_t e = cudaMalloc((void**)p, (n > 0 ? n : 1) * sizeof(E));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

}  // namespace
}  // namespace sp

using namespace sp;

#define SETUP_TRY(expr)                                                                  \
  do {                                                                                   \
    const cudaError_t e_ = (expr);                                                       \
    if (e_ != cudaSuccess) {                                                             \
      cudaGetLastError();                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? SP_ERR_ALLOC : SP_ERR_CUDA,          \
                  "%s: %s (%s)", __func__, cudaGetErrorString(e_), #expr);               \
    }                                                                                    \
  } while (0)

#define SETUP_LAUNCH(kernel, n, ...)                                                     \
  do {                                                                                   \
    kernel<<<setup_grid(n), kSetupThreads, 0, s>>>(__VA_ARGS__);                         \
    count_launch(1);                                                                     \
    SETUP_TRY(cudaGetLastError());                                                       \
  } while (0)

extern "C" {

sp_status sp_ogs_setup_device(int32_t N, int64_t* d_ids, sp_kind kind, int32_t unique,
                              sp_stream_t stream, sp_ogs_plan** out) {
  if (!out) return fail(SP_ERR_INVALID_ARG, "sp_ogs_setup_device: null out");
  *out = nullptr;
  if (N < 0 || N == 2147483647 || (N > 0 && !d_ids))
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_setup_device: bad ids");
  if (kind < SP_KIND_UNSIGNED || kind > SP_KIND_HALO)
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_setup_device: bad kind");
  if ((kind == SP_KIND_UNSIGNED && unique) || (kind == SP_KIND_HALO && unique))
    return fail(SP_ERR_INVALID_ARG, "Invalid ogs setup requested");
  cudaStream_t s = as_cuda(stream);
  long long* ids = reinterpret_cast<long long*>(d_ids);
  Scratch S;

  // ---- 1. key statistics and the sort
  unsigned long long* stats;
  SETUP_TRY(S.get(&stats, 2));
  SETUP_TRY(cudaMemsetAsync(stats, 0, 2 * sizeof(unsigned long long), s));
  if (N > 0) SETUP_LAUNCH(k_id_stats, N, N, ids, stats);
  unsigned long long h_stats[2] = {0, 0};
  SETUP_TRY(cudaMemcpyAsync(h_stats, stats, sizeof(h_stats), cudaMemcpyDeviceToHost, s));
  SETUP_TRY(cudaStreamSynchronize(s));
  const int32_t nids = (int32_t)h_stats[1];
  int end_bit = 1;  // bits of maxAbs + 1, so no real key has every sorted bit set
  while (end_bit < 64 && (h_stats[0] + 1) >> end_bit) ++end_bit;

  std::vector<int32_t> rsT(1, 0), ciT, rsN(1, 0), ciN;
  int32_t ngroups = 0, NrowsP = 0;
  if (nids > 0) {
    unsigned long long *keys, *keys_s;
    int32_t *vals, *vals_s;
    SETUP_TRY(S.get(&keys, N));
    SETUP_TRY(S.get(&keys_s, N));
    SETUP_TRY(S.get(&vals, N));
    SETUP_TRY(S.get(&vals_s, N));
    SETUP_LAUNCH(k_keys, N, N, ids, keys, vals);
    size_t sort_bytes = 0, scan_bytes = 0, scan2_bytes = 0;
    SETUP_TRY(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, keys, keys_s, vals, vals_s, N,
                                              0, end_bit, s));
    SETUP_TRY(cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, vals, vals_s, nids, s));
    SETUP_TRY(cub::DeviceScan::ExclusiveSum(nullptr, scan2_bytes, vals, vals_s, N + 1, s));
    void* temp;
    const size_t temp_bytes = std::max(sort_bytes, std::max(scan_bytes, scan2_bytes));
    SETUP_TRY(S.get((char**)&temp, temp_bytes));
    size_t tb = temp_bytes;
    SETUP_TRY(cub::DeviceRadixSort::SortPairs(temp, tb, keys, keys_s, vals, vals_s, N, 0, end_bit,
                                              s));

    // ---- 2. groups
    int32_t *head, *gscan;
    SETUP_TRY(S.get(&head, nids));
    SETUP_TRY(S.get(&gscan, nids));
    SETUP_LAUNCH(k_heads, nids, nids, keys_s, head);
    tb = temp_bytes;
    SETUP_TRY(cub::DeviceScan::InclusiveSum(temp, tb, head, gscan, nids, s));
    SETUP_TRY(cudaMemcpyAsync(&ngroups, gscan + nids - 1, sizeof(int32_t), cudaMemcpyDeviceToHost,
                              s));
    SETUP_TRY(cudaStreamSynchronize(s));
    int32_t* off;
    SETUP_TRY(S.get(&off, (size_t)ngroups + 1));
    SETUP_LAUNCH(k_offsets, nids, nids, gscan, off);

    // ---- 3. unique owners
    if (unique) SETUP_LAUNCH(k_unique, ngroups, ngroups, off, vals_s, keys_s, ids);

    // ---- 4. row numbers: positive groups by first appearance, then the others
    uint8_t* positive;
    int32_t *fpos, *fneg, *rpos, *rneg, *npos;
    SETUP_TRY(S.get(&positive, ngroups));
    SETUP_TRY(S.get(&fpos, (size_t)N + 1));
    SETUP_TRY(S.get(&fneg, (size_t)N + 1));
    SETUP_TRY(S.get(&rpos, (size_t)N + 1));
    SETUP_TRY(S.get(&rneg, (size_t)N + 1));
    SETUP_TRY(S.get(&npos, 1));
    SETUP_TRY(cudaMemsetAsync(fpos, 0, ((size_t)N + 1) * sizeof(int32_t), s));
    SETUP_TRY(cudaMemsetAsync(fneg, 0, ((size_t)N + 1) * sizeof(int32_t), s));
    SETUP_TRY(cudaMemsetAsync(npos, 0, sizeof(int32_t), s));
    SETUP_LAUNCH(k_group_flags, ngroups, ngroups, off, vals_s, ids, positive, fpos, fneg, npos);
    tb = temp_bytes;
    SETUP_TRY(cub::DeviceScan::ExclusiveSum(temp, tb, fpos, rpos, N + 1, s));
    tb = temp_bytes;
    SETUP_TRY(cub::DeviceScan::ExclusiveSum(temp, tb, fneg, rneg, N + 1, s));
    SETUP_TRY(cudaMemcpyAsync(&NrowsP, npos, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    SETUP_TRY(cudaStreamSynchronize(s));
    int32_t *rowOf, *sizeByRow, *d_rsT, *d_ciT;
    SETUP_TRY(S.get(&rowOf, ngroups));
    SETUP_TRY(S.get(&sizeByRow, (size_t)ngroups + 1));
    SETUP_TRY(S.get(&d_rsT, (size_t)ngroups + 1));
    SETUP_TRY(S.get(&d_ciT, nids));
    SETUP_TRY(cudaMemsetAsync(sizeByRow + ngroups, 0, sizeof(int32_t), s));
    SETUP_LAUNCH(k_rows, ngroups, ngroups, off, vals_s, positive, rpos, rneg, NrowsP, rowOf,
                 sizeByRow);

    // ---- 5. CSR of T, then of N
    tb = temp_bytes;
    SETUP_TRY(cub::DeviceScan::ExclusiveSum(temp, tb, sizeByRow, d_rsT, ngroups + 1, s));
    SETUP_LAUNCH(k_fill_t, nids, nids, gscan, off, rowOf, d_rsT, vals_s, d_ciT);
    rsT.resize((size_t)ngroups + 1);
    ciT.resize(nids);
    SETUP_TRY(cudaMemcpyAsync(rsT.data(), d_rsT, rsT.size() * sizeof(int32_t),
                              cudaMemcpyDeviceToHost, s));
    SETUP_TRY(cudaMemcpyAsync(ciT.data(), d_ciT, ciT.size() * sizeof(int32_t),
                              cudaMemcpyDeviceToHost, s));
    if (kind != SP_KIND_UNSIGNED && NrowsP > 0) {
      int32_t *cntN, *d_rsN, *d_ciN;
      SETUP_TRY(S.get(&cntN, (size_t)NrowsP + 1));
      SETUP_TRY(S.get(&d_rsN, (size_t)NrowsP + 1));
      SETUP_TRY(cudaMemsetAsync(cntN + NrowsP, 0, sizeof(int32_t), s));
      SETUP_LAUNCH(k_count_n, NrowsP, NrowsP, d_rsT, d_ciT, ids, cntN);
      tb = temp_bytes;
      SETUP_TRY(cub::DeviceScan::ExclusiveSum(temp, tb, cntN, d_rsN, NrowsP + 1, s));
      rsN.resize((size_t)NrowsP + 1);
      SETUP_TRY(cudaMemcpyAsync(rsN.data(), d_rsN, rsN.size() * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, s));
      SETUP_TRY(cudaStreamSynchronize(s));
      SETUP_TRY(S.get(&d_ciN, rsN[NrowsP]));
      SETUP_LAUNCH(k_fill_n, NrowsP, NrowsP, d_rsT, d_ciT, ids, d_rsN, d_ciN);
      ciN.resize(rsN[NrowsP]);
      if (!ciN.empty())
        SETUP_TRY(cudaMemcpyAsync(ciN.data(), d_ciN, ciN.size() * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, s));
    } else {
      rsN.assign((size_t)NrowsP + 1, 0);
    }
    SETUP_TRY(cudaStreamSynchronize(s));
  }
  if (kind == SP_KIND_UNSIGNED)  // N shares T's CSR over its first NrowsP rows
    return sp_ogs_plan_create(N, ngroups, rsT.data(), ciT.data(), NrowsP, nullptr, nullptr,
                              stream, out);
  return sp_ogs_plan_create(N, ngroups, rsT.data(), ciT.data(), NrowsP, rsN.data(), ciN.data(),
                            stream, out);
}

sp_status sp_mesh_box_hex_ids_device(int32_t nx, int32_t ny, int32_t nz, int32_t p,
                                     uint64_t perm_seed, int64_t* d_ids, sp_stream_t stream) {
  if (nx < 1 || ny < 1 || nz < 1 || p < 1 || !d_ids)
    return fail(SP_ERR_INVALID_ARG, "sp_mesh_box_hex_ids_device: bad arguments");
  const int64_t Nq = p + 1, E = (int64_t)nx * ny * nz;
  if (E * Nq * Nq * Nq > 2147483647LL)
    return fail(SP_ERR_SIZE, "sp_mesh_box_hex_ids_device: %lld local nodes exceed int32",
                (long long)(E * Nq * Nq * Nq));
  cudaStream_t s = as_cuda(stream);
  const std::vector<int32_t> h_slot = box_slots(E, perm_seed);
  Scratch S;
  int32_t* slot;
#undef SETUP_TRY
#define SETUP_TRY(expr)                                                                  \
  do {                                                                                   \
    const cudaError_t e_ = (expr);                                                       \
    if (e_ != cudaSuccess) {                                                             \
      cudaGetLastError();                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? SP_ERR_ALLOC : SP_ERR_CUDA,          \
                  "%s: %s (%s)", __func__, cudaGetErrorString(e_), #expr);               \
    }                                                                                    \
  } while (0)
  SETUP_TRY(S.get(&slot, E));
  SETUP_TRY(cudaMemcpyAsync(slot, h_slot.data(), E * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  SETUP_LAUNCH(k_box_ids, E * Nq * Nq * Nq, nx, ny, nz, p, slot,
               reinterpret_cast<long long*>(d_ids));
  SETUP_TRY(cudaStreamSynchronize(s));  // the slot table is freed on return
  return SP_SUCCESS;
}

}  // extern "C"
