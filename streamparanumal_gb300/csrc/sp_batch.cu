// Batched instances in one persistent launch.
//
// A batch holds independent instances; instance i owns CG vectors x, r, p, Ap of
// length n_i with a scalar alpha_i, and a node field q_i with its own gather-scatter
// plan.  One launch of k_batch performs, for every instance,
//     x += alpha p;  r -= alpha Ap;  rdotr = r.r      (as sp_cg_update_f64 / _f32)
//     q <- GatherScatter(q, Add, Sym)                 (as sp_ogs_gather_scatter)
// over a flat task list: CG tiles of kBatchTile entries, then groups of 8 warp chunks
// of a plan.  CTAs take tasks round-robin.  Each CG tile writes its partial r.r
// (FP64; FP32 storage accumulates compensated FP32 partials first); the last tile
// of an instance to finish (per-instance ticket) adds the partials in tile order, so
// r.r is deterministic.  x, r and q are bit-identical to the one-instance entry
// points of the same storage type.
#include <algorithm>
#include <vector>

#include "sp_compensated.cuh"
#include "sp_ogs_plan.h"

namespace sp {

constexpr int kBatchThreads = 256;
constexpr int kBatchTile = 8192;  // CG entries per task (32 per lane)
constexpr int kBatchCtasPerSm = 4;  // register budget 64 per lane; the grid is 4 CTAs per SM

template <typename T>
struct BatchInst {
  T* x;
  T* r;
  const T* p;
  const T* Ap;
  double* rdotr;
  T* q;
  const int32_t* rs;
  const int32_t* ids;
  const int4* chunks;
  int64_t n;
  double alpha;
  int32_t nchunks;
  int32_t ntiles;
  int64_t partial_off;  // first tile partial of this instance
  int32_t grouped;      // rs / ids hold the plan's rows grouped by size
};

struct BatchTask {
  int32_t inst;
  int32_t kind;   // 0: CG tile, 1: gather-scatter chunk group
  int64_t first;  // CG: first entry; GS: first chunk
};

__device__ __forceinline__ double bwarp_sum(double v) {
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) v += __shfl_down_sync(0xffffffffu, v, h);
  return v;
}

// One CG tile: the updates of entries [e0, e1) and this lane's share of r.r.  Each
// lane takes its entries kCgUnroll at a time, all loads issued before the updates.
constexpr int kCgUnroll = 2;

__device__ __forceinline__ double cg_tile(const BatchInst<double>& I, int64_t e0, int64_t e1,
                                          int tid) {
  double acc = 0.0;
  for (int64_t base = e0 + tid; base < e1; base += (int64_t)kBatchThreads * kCgUnroll) {
    double xp[kCgUnroll], xa[kCgUnroll], xx[kCgUnroll], xr[kCgUnroll];
#pragma unroll
    for (int u = 0; u < kCgUnroll; ++u) {
      const int64_t i = base + (int64_t)u * kBatchThreads;
      if (i < e1) {
        xp[u] = I.p[i];
        xa[u] = I.Ap[i];
        xx[u] = I.x[i];
        xr[u] = I.r[i];
      }
    }
#pragma unroll
    for (int u = 0; u < kCgUnroll; ++u) {
      const int64_t i = base + (int64_t)u * kBatchThreads;
      if (i < e1) {
        const double xn = fma(I.alpha, xp[u], xx[u]);
        const double rn = fma(-I.alpha, xa[u], xr[u]);
        I.x[i] = xn;
        I.r[i] = rn;
        acc = fma(rn, rn, acc);
      }
    }
  }
  return acc;
}
__device__ __forceinline__ double cg_tile(const BatchInst<float>& I, int64_t e0, int64_t e1,
                                          int tid) {
  const float a = (float)I.alpha;
  float sum = 0.f, comp = 0.f;
  for (int64_t base = e0 + tid; base < e1; base += (int64_t)kBatchThreads * kCgUnroll) {
    float xp[kCgUnroll], xa[kCgUnroll], xx[kCgUnroll], xr[kCgUnroll];
#pragma unroll
    for (int u = 0; u < kCgUnroll; ++u) {
      const int64_t i = base + (int64_t)u * kBatchThreads;
      if (i < e1) {
        xp[u] = I.p[i];
        xa[u] = I.Ap[i];
        xx[u] = I.x[i];
        xr[u] = I.r[i];
      }
    }
#pragma unroll
    for (int u = 0; u < kCgUnroll; ++u) {
      const int64_t i = base + (int64_t)u * kBatchThreads;
      if (i < e1) {
        const float xn = fmaf(a, xp[u], xx[u]);
        const float rn = fmaf(-a, xa[u], xr[u]);
        I.x[i] = xn;
        I.r[i] = rn;
        dot2_step(rn, rn, sum, comp);
      }
    }
  }
  return (double)sum + (double)comp;
}

// 0 + v0 == v0 except -0 -> +0: the first member is taken by an integer select
__device__ __forceinline__ double first_plus(double v) {
  const long long b = __double_as_longlong(v);
  return __longlong_as_double(b == (long long)0x8000000000000000ULL ? 0LL : b);
}
__device__ __forceinline__ float first_plus(float v) {
  const int b = __float_as_int(v);
  return __int_as_float(b == (int)0x80000000u ? 0 : b);
}

template <typename T>
__global__ void __launch_bounds__(kBatchThreads, kBatchCtasPerSm)
k_batch(const BatchInst<T>* __restrict__ inst, const BatchTask* __restrict__ tasks, int64_t ntasks,
        double* __restrict__ partial, unsigned int* __restrict__ tickets) {
  __shared__ double s_red[kBatchThreads / 32];
  __shared__ bool s_last;
  __shared__ T s_val[kWarpsPerCta][kWarpChunkNnz];
  __shared__ int32_t s_rs[kWarpsPerCta][kWarpChunkNnz + 8];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int64_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const BatchTask task = tasks[t];
    const BatchInst<T>& I = inst[task.inst];
    if (task.kind == 0) {
      // ---- CG tile: entries [first, first + kBatchTile) of instance I
      const int64_t e0 = task.first;
      const int64_t e1 = min(e0 + (int64_t)kBatchTile, I.n);
      double acc = bwarp_sum(cg_tile(I, e0, e1, tid));
      if (lane == 0) s_red[w] = acc;
      __syncthreads();
      if (tid == 0) {
        double b = 0.0;
        for (int k = 0; k < kBatchThreads / 32; ++k) b += s_red[k];
        const int64_t tile = (e0 / kBatchTile);
        partial[I.partial_off + tile] = b;
        __threadfence();
        const unsigned tk = atomicAdd(tickets + task.inst, 1u);
        s_last = (tk == (unsigned)I.ntiles - 1u);
      }
      __syncthreads();
      if (s_last && w == 0) {
        __threadfence();
        double v = 0.0;
        for (int k = lane; k < I.ntiles; k += 32) v += __ldcg(partial + I.partial_off + k);
        v = bwarp_sum(v);
        if (lane == 0) {
          I.rdotr[0] = v;
          tickets[task.inst] = 0u;
        }
      }
      __syncthreads();
    } else {
      // ---- gather+scatter (Add, Sym): warp w takes chunk first + w
      const int64_t c = task.first + w;
      if (c < I.nchunks) {
        const int4 d = I.chunks[c];
        const int32_t gn = d.w - d.z, nr = d.y - d.x;
        T* sv = s_val[w];
        int32_t* srs = s_rs[w];
        if (I.grouped) {  // packed words: first entry - g0 | row offset << 16
          for (int32_t r = lane; r < nr; r += 32) srs[r] = I.rs[d.x + r] & 0xFFFF;
          if (lane == 0) srs[nr] = gn;
        } else {
          for (int32_t r = lane; r <= nr; r += 32) srs[r] = I.rs[d.x + r] - d.z;
        }
        int32_t col[kOgsPerLane];
        T val[kOgsPerLane];
#pragma unroll
        for (int u = 0; u < kOgsPerLane; ++u)
          col[u] = (lane + 32 * u < gn) ? I.ids[d.z + lane + 32 * u] : 0;
#pragma unroll
        for (int u = 0; u < kOgsPerLane; ++u)
          if (lane + 32 * u < gn) val[u] = I.q[col[u]];
#pragma unroll
        for (int u = 0; u < kOgsPerLane; ++u)
          if (lane + 32 * u < gn) sv[lane + 32 * u] = val[u];
        __syncwarp();
        for (int32_t r = lane; r < nr; r += 32) {
          const int32_t a = srs[r], b = srs[r + 1];
          T acc = T(0);
          if (a < b) acc = first_plus(sv[a]);
          for (int32_t i = a + 1; i < b; ++i) acc = acc + sv[i];
          for (int32_t i = a; i < b; ++i) sv[i] = acc;
        }
        __syncwarp();
#pragma unroll
        for (int u = 0; u < kOgsPerLane; ++u)
          if (lane + 32 * u < gn) I.q[col[u]] = sv[lane + 32 * u];
      }
      __syncwarp();
    }
  }
}

}  // namespace sp

struct sp_batch {
  int32_t ninst = 0;
  int64_t ntasks = 0;
  bool f32 = false;
  void* d_inst = nullptr;  // BatchInst<double> or BatchInst<float>
  sp::BatchTask* d_tasks = nullptr;
  double* d_partial = nullptr;
  unsigned int* d_tickets = nullptr;
  unsigned grid = 0;
};

using namespace sp;

namespace sp {

template <typename T>
static sp_status batch_create(const char* name, int32_t ninst, const sp_ogs_plan* const* plans,
                              const int64_t* n, T* const* x, T* const* r, const T* const* p,
                              const T* const* Ap, double* const* rdotr, T* const* q,
                              const double* alpha, sp_stream_t stream, sp_batch** out) {
  if (!out) return fail(SP_ERR_INVALID_ARG, "%s: null out", name);
  *out = nullptr;
  if (ninst < 1 || !plans || !n || !x || !r || !p || !Ap || !rdotr || !q || !alpha)
    return fail(SP_ERR_INVALID_ARG, "%s: null argument or empty batch", name);
  std::vector<BatchInst<T>> inst(ninst);
  std::vector<BatchTask> tasks;
  int64_t npartial = 0;
  for (int32_t i = 0; i < ninst; ++i) {
    const sp_ogs_plan* P = plans[i];
    if (!P) return fail(SP_ERR_INVALID_ARG, "%s: null plan %d", name, i);
    if (P->nchunksT == 0)
      return fail(SP_ERR_UNSUPPORTED, "%s: plan %d has rows beyond %d entries", name, i,
                  kWarpChunkNnz);
    if (n[i] < 0) return fail(SP_ERR_INVALID_ARG, "%s: negative n[%d]", name, i);
    if (!rdotr[i] || (n[i] > 0 && (!x[i] || !r[i] || !p[i] || !Ap[i])) ||
        (P->nnzT > 0 && !q[i]))
      return fail(SP_ERR_INVALID_ARG, "%s: null vector in instance %d", name, i);
    BatchInst<T>& I = inst[i];
    I.x = x[i];
    I.r = r[i];
    I.p = p[i];
    I.Ap = Ap[i];
    I.rdotr = rdotr[i];
    I.q = q[i];
    // the rows the plan's T chunks walk: grouped by size, renumbered, or as in T
    I.grouped = P->row_order == 1 ? 1 : 0;
    I.rs = I.grouped ? P->d_rowsGT : (P->d_walkRsT ? P->d_walkRsT : P->d_rowStartsT);
    I.ids = I.grouped ? P->d_colIdsGT : (P->d_walkCiT ? P->d_walkCiT : P->d_colIdsT);
    I.chunks = reinterpret_cast<const int4*>(P->d_chunksT);
    I.n = n[i];
    I.alpha = alpha[i];
    I.nchunks = P->nchunksT;
    I.ntiles = (int32_t)std::max<int64_t>(1, (n[i] + kBatchTile - 1) / kBatchTile);
    I.partial_off = npartial;
    npartial += I.ntiles;
    for (int32_t t = 0; t < I.ntiles; ++t) tasks.push_back({i, 0, (int64_t)t * kBatchTile});
  }
  for (int32_t i = 0; i < ninst; ++i)
    for (int32_t c = 0; c < inst[i].nchunks; c += kWarpsPerCta) tasks.push_back({i, 1, c});
  sp_batch* b = new sp_batch();
  b->ninst = ninst;
  b->ntasks = (int64_t)tasks.size();
  b->f32 = sizeof(T) == 4;
  cudaStream_t s = as_cuda(stream);
  cudaError_t e = cudaMalloc(&b->d_inst, sizeof(BatchInst<T>) * ninst);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_tasks, sizeof(BatchTask) * tasks.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->d_partial, sizeof(double) * npartial);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_tickets, sizeof(unsigned) * ninst);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_inst, inst.data(), sizeof(BatchInst<T>) * ninst,
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_tasks, tasks.data(), sizeof(BatchTask) * tasks.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_tickets, 0, sizeof(unsigned) * ninst, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    sp_batch_destroy(b);
    cudaGetLastError();
    return fail(SP_ERR_ALLOC, "%s: %s", name, cudaGetErrorString(e));
  }
  const int64_t cap = (int64_t)sm_count() * kBatchCtasPerSm;
  b->grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cap, b->ntasks));
  *out = b;
  return SP_SUCCESS;
}

}  // namespace sp

extern "C" {

sp_status sp_batch_create(int32_t ninst, const sp_ogs_plan* const* plans, const int64_t* n,
                          double* const* x, double* const* r, const double* const* p,
                          const double* const* Ap, double* const* rdotr, double* const* q,
                          const double* alpha, sp_stream_t stream, sp_batch** out) {
  return batch_create<double>("sp_batch_create", ninst, plans, n, x, r, p, Ap, rdotr, q, alpha,
                              stream, out);
}

sp_status sp_batch_create_f32(int32_t ninst, const sp_ogs_plan* const* plans, const int64_t* n,
                              float* const* x, float* const* r, const float* const* p,
                              const float* const* Ap, double* const* rdotr, float* const* q,
                              const double* alpha, sp_stream_t stream, sp_batch** out) {
  return batch_create<float>("sp_batch_create_f32", ninst, plans, n, x, r, p, Ap, rdotr, q, alpha,
                             stream, out);
}

sp_status sp_batch_run(const sp_batch* b, sp_stream_t stream) {
  if (!b) return fail(SP_ERR_INVALID_ARG, "sp_batch_run: null batch");
  if (b->f32)
    k_batch<float><<<b->grid, kBatchThreads, 0, as_cuda(stream)>>>(
        static_cast<const BatchInst<float>*>(b->d_inst), b->d_tasks, b->ntasks, b->d_partial,
        b->d_tickets);
  else
    k_batch<double><<<b->grid, kBatchThreads, 0, as_cuda(stream)>>>(
        static_cast<const BatchInst<double>*>(b->d_inst), b->d_tasks, b->ntasks, b->d_partial,
        b->d_tickets);
  return check_launch("sp_batch_run");
}

sp_status sp_batch_destroy(sp_batch* b) {
  if (!b) return SP_SUCCESS;
  if (b->d_inst) cudaFree(b->d_inst);
  if (b->d_tasks) cudaFree(b->d_tasks);
  if (b->d_partial) cudaFree(b->d_partial);
  if (b->d_tickets) cudaFree(b->d_tickets);
  delete b;
  return SP_SUCCESS;
}

}  // extern "C"
