// BS0-BS5 streaming kernels for sm_103a.
//
// All FP64 arithmetic is written with explicit fma()/add so the rounding is fixed
// by the source, not by the compiler's contraction choices.  The choices follow
// the reference's CUDA mode, which compiles OKL with --fmad=true
// (libs/core/platformProperties.cpp:76):
//   bs2:  alpha*x + beta*y   -> fma(alpha, x, beta*y)
//   bs3:  acc += a*a         -> fma(a, a, acc)
//   bs4:  acc += a*b         -> fma(a, b, acc)
//   bs5:  r + alpha*Ap       -> fma(alpha, Ap, r);  acc += r*r -> fma(r, r, acc)
#include <cstdint>
#include <initializer_list>
#include <map>
#include <mutex>
#include <utility>

#include "sp_internal.h"
#include "sp_compensated.cuh"
#include "sp_sumsq.cuh"

namespace sp {

// ------------------------------------------------------------------ helpers

template <typename T> struct Vec16;
template <> struct Vec16<double> { using type = double2; static constexpr int W = 2; };
template <> struct Vec16<float>  { using type = float4;  static constexpr int W = 4; };

__device__ __forceinline__ double2 vload(const double2* p) { return __ldcs(p); }
__device__ __forceinline__ float4  vload(const float4* p)  { return __ldcs(p); }
__device__ __forceinline__ void vstore(double2* p, double2 v) { __stcs(p, v); }
__device__ __forceinline__ void vstore(float4* p, float4 v)   { __stcs(p, v); }

static inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Grid for a "U vectors of 16 bytes per thread" streaming kernel.
static inline unsigned stream_grid(int64_t nvec, int threads, int U) {
  int64_t per = (int64_t)threads * U;
  int64_t g = (nvec + per - 1) / per;
  if (g < 1) g = 1;
  return (unsigned)g;
}

// ------------------------------------------------------------------ BS0

__global__ void k_bs0(int n, const double* __restrict__ a, double* __restrict__ b) {
  (void)a;
  // one block, one thread: the store happens only when n == 0 (bs0.okl:33-35)
  if ((int)threadIdx.x == n && (int)blockIdx.x == n) b[0] = 0.0;
}

// ------------------------------------------------------------------ BS1 copy

constexpr int kStreamThreads = 256;

template <typename T, int U>
__global__ void __launch_bounds__(kStreamThreads)
k_copy_vec(const typename Vec16<T>::type* __restrict__ a, typename Vec16<T>::type* __restrict__ b,
           int64_t nvec, const T* __restrict__ as, T* __restrict__ bs, int64_t n) {
  using V = typename Vec16<T>::type;
  const int64_t base = (int64_t)blockIdx.x * (kStreamThreads * U) + threadIdx.x;
  V v[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = base + (int64_t)u * kStreamThreads;
    if (i < nvec) v[u] = vload(a + i);
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = base + (int64_t)u * kStreamThreads;
    if (i < nvec) vstore(b + i, v[u]);
  }
  // scalar tail (fewer than one vector)
  if (blockIdx.x == 0) {
    const int64_t t = nvec * Vec16<T>::W + threadIdx.x;
    if (t < n) bs[t] = as[t];
  }
}

template <typename T>
__global__ void __launch_bounds__(kStreamThreads)
k_copy_scalar(const T* __restrict__ a, T* __restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

template <typename T>
static sp_status launch_copy(int64_t n, const T* a, T* b, cudaStream_t s, const char* name) {
  if (n < 0) return fail(SP_ERR_INVALID_ARG, "%s: negative length %lld", name, (long long)n);
  if (n == 0) return SP_SUCCESS;
  if (!a || !b) return fail(SP_ERR_INVALID_ARG, "%s: null pointer", name);
  constexpr int W = Vec16<T>::W;
  if (aligned16(a) && aligned16(b)) {
    constexpr int U = 4;
    const int64_t nvec = n / W;
    k_copy_vec<T, U><<<stream_grid(nvec, kStreamThreads, U), kStreamThreads, 0, s>>>(
        reinterpret_cast<const typename Vec16<T>::type*>(a),
        reinterpret_cast<typename Vec16<T>::type*>(b), nvec, a, b, n);
  } else {
    k_copy_scalar<T><<<stream_grid(n, kStreamThreads, 4), kStreamThreads, 0, s>>>(a, b, n);
  }
  return check_launch(name);
}

// ------------------------------------------------------------------ BS2 axpy

__device__ __forceinline__ double axpby(double al, double x, double be, double y) {
  return fma(al, x, be * y);
}
__device__ __forceinline__ float axpby(float al, float x, float be, float y) {
  return fmaf(al, x, be * y);
}
__device__ __forceinline__ double2 axpby(double al, double2 x, double be, double2 y) {
  return make_double2(axpby(al, x.x, be, y.x), axpby(al, x.y, be, y.y));
}
__device__ __forceinline__ float4 axpby(float al, float4 x, float be, float4 y) {
  return make_float4(axpby(al, x.x, be, y.x), axpby(al, x.y, be, y.y), axpby(al, x.z, be, y.z),
                     axpby(al, x.w, be, y.w));
}

template <typename T, int U>
__global__ void __launch_bounds__(kStreamThreads)
k_axpy_vec(int64_t nvec, T alpha, const typename Vec16<T>::type* __restrict__ x, T beta,
           typename Vec16<T>::type* __restrict__ y, const T* __restrict__ xs, T* __restrict__ ys,
           int64_t n) {
  using V = typename Vec16<T>::type;
  const int64_t base = (int64_t)blockIdx.x * (kStreamThreads * U) + threadIdx.x;
  V vx[U], vy[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = base + (int64_t)u * kStreamThreads;
    if (i < nvec) { vx[u] = vload(x + i); vy[u] = vload(y + i); }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = base + (int64_t)u * kStreamThreads;
    if (i < nvec) vstore(y + i, axpby(alpha, vx[u], beta, vy[u]));
  }
  if (blockIdx.x == 0) {
    const int64_t t = nvec * Vec16<T>::W + threadIdx.x;
    if (t < n) ys[t] = axpby(alpha, xs[t], beta, ys[t]);
  }
}

template <typename T>
__global__ void __launch_bounds__(kStreamThreads)
k_axpy_scalar(int64_t n, T alpha, const T* __restrict__ x, T beta, T* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = axpby(alpha, x[i], beta, y[i]);
}

template <typename T>
static sp_status launch_axpy(int64_t n, T alpha, const T* x, T beta, T* y, cudaStream_t s,
                             const char* name) {
  if (n < 0) return fail(SP_ERR_INVALID_ARG, "%s: negative length %lld", name, (long long)n);
  if (n == 0) return SP_SUCCESS;
  if (!x || !y) return fail(SP_ERR_INVALID_ARG, "%s: null pointer", name);
  constexpr int W = Vec16<T>::W;
  if (aligned16(x) && aligned16(y)) {
    constexpr int U = 4;
    const int64_t nvec = n / W;
    k_axpy_vec<T, U><<<stream_grid(nvec, kStreamThreads, U), kStreamThreads, 0, s>>>(
        nvec, alpha, reinterpret_cast<const typename Vec16<T>::type*>(x), beta,
        reinterpret_cast<typename Vec16<T>::type*>(y), x, y, n);
  } else {
    k_axpy_scalar<T><<<stream_grid(n, kStreamThreads, 4), kStreamThreads, 0, s>>>(n, alpha, x,
                                                                                   beta, y);
  }
  return check_launch(name);
}

// ------------------------------------------------------------------ order-exact reductions
//
// The halving tree of the reference's reduction kernels (bs3.okl:43-63 and the
// identical trees of bs4/bs5): level h adds s[t+h] into s[t] for t < h, for
// h = BS/2 ... 2, and the result is s[0] + s[1].  Levels h >= 64 run through
// shared memory; h = 32 ... 1 run in warp 0 with shuffles, which performs the
// same additions on the same operands.
template <int BS>
__device__ __forceinline__ double tree_reduce(double v, double* s) {
  const int t = threadIdx.x;
  s[t] = v;
  __syncthreads();
#pragma unroll
  for (int h = BS / 2; h >= 64; h >>= 1) {
    if (t < h) s[t] = s[t] + s[t + h];
    __syncthreads();
  }
  double r = 0.0;
  if (t < 32) {
    r = s[t] + s[t + 32];
    r = r + __shfl_down_sync(0xffffffffu, r, 16);
    r = r + __shfl_down_sync(0xffffffffu, r, 8);
    r = r + __shfl_down_sync(0xffffffffu, r, 4);
    r = r + __shfl_down_sync(0xffffffffu, r, 2);
    r = r + __shfl_down_sync(0xffffffffu, r, 1);
  }
  return r;  // valid in thread 0
}

// Lane t of logical block b visits t + b*BS + j*BS*nblocks for j = 0, 1, ...
// (bs3.okl:36-41).  For a fixed j the block's lanes read one contiguous chunk of
// BS values, so each CTA streams through its chunks j = 0, 1, 2, ...  Two things
// keep enough bytes in flight with only nblocks*BS lanes:
//   * U chunks' loads are issued ahead of the in-order accumulation;
//   * with pd > 0, lanes of warp 0 issue cp.async.bulk.prefetch.L2 for the chunks
//     pd ahead, so the lanes' loads hit L2 (fire-and-forget: nothing waits on it).

// Bulk L2 prefetch of `bytes` (multiple of 16) from a 16-byte aligned address.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Prefetch chunk j (BS doubles at base + j*stride) of x, clipped to n.
template <int BS>
__device__ __forceinline__ void prefetch_chunk(const double* x, int64_t base, int64_t stride,
                                               int64_t j, int64_t n) {
  const int64_t start = base + j * stride;
  if (start >= n) return;
  const int64_t cnt = (n - start < BS) ? (n - start) : BS;
  const uint32_t bytes = (uint32_t)(cnt * 8) & ~15u;
  if (bytes) prefetch_l2(x + start, bytes);
}

// ROLL = true keeps U loads in flight at all times: each value is replaced by the
// load of the same lane slot of the next group as soon as it has been read, and
// the in-order accumulation then waits on the older loads only.  ROLL = false
// loads a group, consumes it, loads the next.  Both add in the same order.
template <int BS, int U, bool ROLL>
__global__ void __launch_bounds__(BS)
k_bs3_1(int nblocks, int64_t n, const double* __restrict__ a, double* __restrict__ partial,
        int pd) {
  __shared__ double s[BS];
  const int t = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * BS;
  const int64_t stride = (int64_t)BS * nblocks;
  const bool pf = pd > 0 && ((reinterpret_cast<uintptr_t>(a) & 15u) == 0);
  if (pf && t < pd) prefetch_chunk<BS>(a, base, stride, t, n);
  int64_t id = base + t, j = 0;
  double acc = 0.0;
  if (ROLL) {
    if (id + (U - 1) * stride < n) {
      double v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = __ldcs(a + id + u * stride);
      id += U * stride;
      j += U;
      for (; id + (U - 1) * stride < n; id += U * stride, j += U) {
        if (pf && t < U) prefetch_chunk<BS>(a, base, stride, j + pd + t, n);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const double x = v[u];
          v[u] = __ldcs(a + id + u * stride);
          acc = fma(x, x, acc);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) acc = fma(v[u], v[u], acc);
    }
  } else {
    for (; id + (U - 1) * stride < n; id += U * stride, j += U) {
      if (pf && t < U) prefetch_chunk<BS>(a, base, stride, j + pd + t, n);
      double v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = __ldcs(a + id + u * stride);
#pragma unroll
      for (int u = 0; u < U; ++u) acc = fma(v[u], v[u], acc);
    }
  }
  for (; id < n; id += stride) {
    const double v = __ldcs(a + id);
    acc = fma(v, v, acc);
  }
  const double r = tree_reduce<BS>(acc, s);
  if (t == 0) partial[blockIdx.x] = r;
}

template <int BS, int U, bool ROLL>
__global__ void __launch_bounds__(BS)
k_bs4_1(int nblocks, int64_t n, const double* __restrict__ a, const double* __restrict__ b,
        double* __restrict__ partial, int pd) {
  __shared__ double s[BS];
  const int t = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * BS;
  const int64_t stride = (int64_t)BS * nblocks;
  const bool pf = pd > 0 && (((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) &
                              15u) == 0);
  if (pf && t < pd) prefetch_chunk<BS>(a, base, stride, t, n);
  if (pf && t >= 32 && t < 32 + pd) prefetch_chunk<BS>(b, base, stride, t - 32, n);
  int64_t id = base + t, j = 0;
  double acc = 0.0;
  if (ROLL) {
    if (id + (U - 1) * stride < n) {
      double va[U], vb[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        va[u] = __ldcs(a + id + u * stride);
        vb[u] = __ldcs(b + id + u * stride);
      }
      id += U * stride;
      j += U;
      for (; id + (U - 1) * stride < n; id += U * stride, j += U) {
        if (pf && t < U) prefetch_chunk<BS>(a, base, stride, j + pd + t, n);
        if (pf && t >= 32 && t < 32 + U) prefetch_chunk<BS>(b, base, stride, j + pd + t - 32, n);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const double x = va[u], y = vb[u];
          va[u] = __ldcs(a + id + u * stride);
          vb[u] = __ldcs(b + id + u * stride);
          acc = fma(x, y, acc);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) acc = fma(va[u], vb[u], acc);
    }
  } else {
    for (; id + (U - 1) * stride < n; id += U * stride, j += U) {
      if (pf && t < U) prefetch_chunk<BS>(a, base, stride, j + pd + t, n);
      if (pf && t >= 32 && t < 32 + U) prefetch_chunk<BS>(b, base, stride, j + pd + t - 32, n);
      double va[U], vb[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        va[u] = __ldcs(a + id + u * stride);
        vb[u] = __ldcs(b + id + u * stride);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) acc = fma(va[u], vb[u], acc);
    }
  }
  for (; id < n; id += stride) acc = fma(__ldcs(a + id), __ldcs(b + id), acc);
  const double r = tree_reduce<BS>(acc, s);
  if (t == 0) partial[blockIdx.x] = r;
}

template <int BS, int U, bool ROLL>
__global__ void __launch_bounds__(BS)
k_bs5_1(int nblocks, int64_t n, const double* __restrict__ Ap, double alpha, double* __restrict__ r,
        double* __restrict__ partial, int pd) {
  __shared__ double s[BS];
  const int t = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * BS;
  const int64_t stride = (int64_t)BS * nblocks;
  const bool pf = pd > 0 && (((reinterpret_cast<uintptr_t>(Ap) | reinterpret_cast<uintptr_t>(r)) &
                              15u) == 0);
  if (pf && t < pd) prefetch_chunk<BS>(r, base, stride, t, n);
  if (pf && t >= 32 && t < 32 + pd) prefetch_chunk<BS>(Ap, base, stride, t - 32, n);
  int64_t id = base + t, j = 0;
  double acc = 0.0;
  if (ROLL) {
    if (id + (U - 1) * stride < n) {
      double vr[U], va[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        vr[u] = __ldcs(r + id + u * stride);
        va[u] = __ldcs(Ap + id + u * stride);
      }
      int64_t prev = id;
      id += U * stride;
      j += U;
      for (; id + (U - 1) * stride < n; prev = id, id += U * stride, j += U) {
        if (pf && t < U) prefetch_chunk<BS>(r, base, stride, j + pd + t, n);
        if (pf && t >= 32 && t < 32 + U) prefetch_chunk<BS>(Ap, base, stride, j + pd + t - 32, n);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const double rr = fma(alpha, va[u], vr[u]);
          vr[u] = __ldcs(r + id + u * stride);
          va[u] = __ldcs(Ap + id + u * stride);
          __stcs(r + prev + u * stride, rr);
          acc = fma(rr, rr, acc);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const double rr = fma(alpha, va[u], vr[u]);
        __stcs(r + prev + u * stride, rr);
        acc = fma(rr, rr, acc);
      }
    }
  } else {
    for (; id + (U - 1) * stride < n; id += U * stride, j += U) {
      if (pf && t < U) prefetch_chunk<BS>(r, base, stride, j + pd + t, n);
      if (pf && t >= 32 && t < 32 + U) prefetch_chunk<BS>(Ap, base, stride, j + pd + t - 32, n);
      double vr[U], va[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        vr[u] = __ldcs(r + id + u * stride);
        va[u] = __ldcs(Ap + id + u * stride);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const double rr = fma(alpha, va[u], vr[u]);
        __stcs(r + id + u * stride, rr);
        acc = fma(rr, rr, acc);
      }
    }
  }
  for (; id < n; id += stride) {
    const double rr = fma(alpha, __ldcs(Ap + id), __ldcs(r + id));
    __stcs(r + id, rr);
    acc = fma(rr, rr, acc);
  }
  const double res = tree_reduce<BS>(acc, s);
  if (t == 0) partial[blockIdx.x] = res;
}

// Stage 2 (bs3.okl:66-102): lane t holds 0.0 + partial[t] (t < nblocks, each lane
// sees at most one entry because the stride BS*nblocks >= nblocks), then the tree.
template <int BS>
__global__ void __launch_bounds__(BS)
k_finish(int nblocks, const double* __restrict__ partial, double* __restrict__ out) {
  __shared__ double s[BS];
  const int t = threadIdx.x;
  double v = 0.0;
  if (t < nblocks) v = 0.0 + partial[t];
  const double r = tree_reduce<BS>(v, s);
  if (t == 0) out[0] = r;
}

// Launch helpers of the stage-1 kernels: U per block size, ROLL from the tuning knob.
template <bool R>
static void launch_bs3_impl(int bs, int nb, int64_t n, const double* a, double* part, int pd,
                            cudaStream_t s) {
  if (bs == 256) k_bs3_1<256, 16, R><<<nb, 256, 0, s>>>(nb, n, a, part, pd);
  else if (bs == 512) k_bs3_1<512, 8, R><<<nb, 512, 0, s>>>(nb, n, a, part, pd);
  else k_bs3_1<1024, 4, R><<<nb, 1024, 0, s>>>(nb, n, a, part, pd);
}
template <bool R>
static void launch_bs4_impl(int bs, int nb, int64_t n, const double* a, const double* b,
                            double* part, int pd, cudaStream_t s) {
  if (bs == 256) k_bs4_1<256, 8, R><<<nb, 256, 0, s>>>(nb, n, a, b, part, pd);
  else if (bs == 512) k_bs4_1<512, 4, R><<<nb, 512, 0, s>>>(nb, n, a, b, part, pd);
  else k_bs4_1<1024, 4, R><<<nb, 1024, 0, s>>>(nb, n, a, b, part, pd);
}
template <bool R>
static void launch_bs5_impl(int bs, int nb, int64_t n, const double* Ap, double alpha, double* r,
                            double* part, int pd, cudaStream_t s) {
  if (bs == 256) k_bs5_1<256, 8, R><<<nb, 256, 0, s>>>(nb, n, Ap, alpha, r, part, pd);
  else if (bs == 512) k_bs5_1<512, 4, R><<<nb, 512, 0, s>>>(nb, n, Ap, alpha, r, part, pd);
  else k_bs5_1<1024, 4, R><<<nb, 1024, 0, s>>>(nb, n, Ap, alpha, r, part, pd);
}
// Prefetch distance: the knob when set (>= 0), else the per-kernel default measured
// on GB300 with the rolling pipeline (BS3 0, BS4 16, BS5 0 chunks).
static int prefetch_for(int dflt) {
  const int64_t v = tune(kTuneReducePrefetch);
  return v >= 0 ? (int)v : dflt;
}
static void launch_bs3(int bs, int nb, int64_t n, const double* a, double* part, cudaStream_t s) {
  const int pd = prefetch_for(0);
  if (tune(kTuneReduceRolling)) launch_bs3_impl<true>(bs, nb, n, a, part, pd, s);
  else launch_bs3_impl<false>(bs, nb, n, a, part, pd, s);
}
static void launch_bs4(int bs, int nb, int64_t n, const double* a, const double* b, double* part,
                       cudaStream_t s) {
  const int pd = prefetch_for(16);
  if (tune(kTuneReduceRolling)) launch_bs4_impl<true>(bs, nb, n, a, b, part, pd, s);
  else launch_bs4_impl<false>(bs, nb, n, a, b, part, pd, s);
}
static void launch_bs5(int bs, int nb, int64_t n, const double* Ap, double alpha, double* r,
                       double* part, cudaStream_t s) {
  const int pd = prefetch_for(0);
  if (tune(kTuneReduceRolling)) launch_bs5_impl<true>(bs, nb, n, Ap, alpha, r, part, pd, s);
  else launch_bs5_impl<false>(bs, nb, n, Ap, alpha, r, part, pd, s);
}

static sp_status check_exact_args(int32_t bs, int32_t nblocks, int64_t n, const char* name) {
  if (bs != 256 && bs != 512 && bs != 1024)
    return fail(SP_ERR_INVALID_ARG, "%s: block_size %d not in {256,512,1024}", name, bs);
  if (nblocks < 1 || nblocks > bs)
    return fail(SP_ERR_INVALID_ARG, "%s: nblocks %d outside [1, %d]", name, nblocks, bs);
  if (n < 0) return fail(SP_ERR_INVALID_ARG, "%s: negative length", name);
  return SP_SUCCESS;
}

// ------------------------------------------------------------------ single-launch reductions
//
// Fixed grid of G blocks; lane accumulation over a grid-stride loop, block tree,
// per-block partial to scratch, and the last block to arrive (ticket counter)
// reduces the G partials in a fixed order and resets the counter to zero.

constexpr int kRedThreads = 256;

struct RedScratch {
  unsigned int* ticket;
  double* partial;  // kRedPartialBytes per block (two doubles, or an AccBits)
};

__host__ __device__ inline RedScratch red_scratch(void* p) {
  char* c = static_cast<char*>(p);
  return RedScratch{reinterpret_cast<unsigned int*>(c),
                    reinterpret_cast<double*>(c + kRedPartialOff)};
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) v += __shfl_down_sync(0xffffffffu, v, h);
  return v;
}

// Sum of `v` over the block (result valid in thread 0), fixed order.
__device__ __forceinline__ double block_sum(double v, double* s) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) s[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? s[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Writes the block's value, and lets the last block finish into out[0].
__device__ __forceinline__ void finish_ticket(double block_val, RedScratch sc, double* out,
                                              double* s) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    sc.partial[blockIdx.x] = block_val;
    __threadfence();
    const unsigned t = atomicAdd(sc.ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) v += __ldcg(sc.partial + i);
  const double r = block_sum(v, s);
  if (threadIdx.x == 0) {
    out[0] = r;
    *sc.ticket = 0u;  // leave the scratch zeroed for the next call
  }
}

template <int U>
__global__ void __launch_bounds__(kRedThreads)
k_dot_f64_fast(int64_t nvec, const double2* __restrict__ a, const double2* __restrict__ b,
               const double* __restrict__ as, const double* __restrict__ bs, int64_t n,
               void* scratch, double* out) {
  __shared__ double s[32];
  const RedScratch sc = red_scratch(scratch);
  double acc0 = 0.0, acc1 = 0.0;
  const int64_t step = (int64_t)gridDim.x * kRedThreads * U;
  for (int64_t base = (int64_t)blockIdx.x * kRedThreads * U + threadIdx.x; base < nvec;
       base += step) {
    double2 va[U], vb[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * kRedThreads;
      if (i < nvec) {
        va[u] = __ldcs(a + i);
        vb[u] = (b == a) ? va[u] : __ldcs(b + i);
      } else {
        va[u] = make_double2(0.0, 0.0);
        vb[u] = va[u];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      acc0 = fma(va[u].x, vb[u].x, acc0);
      acc1 = fma(va[u].y, vb[u].y, acc1);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) acc0 = fma(as[n - 1], bs[n - 1], acc0);
  const double bv = block_sum(acc0 + acc1, s);
  finish_ticket(bv, sc, out, s);
}

// FP32-storage dot: compensated FP32 partials (two Dot2 chains) over a rolling load
// pipeline (the next U vectors of both inputs load while the current ones are
// added); FP64 across lanes and blocks.
template <int U>
__global__ void __launch_bounds__(kRedThreads)
k_dot_f32_fast(int64_t nvec, const float4* __restrict__ a, const float4* __restrict__ b,
               const float* __restrict__ as, const float* __restrict__ bs, int64_t n,
               void* scratch, double* out) {
  __shared__ double s[32];
  const RedScratch sc = red_scratch(scratch);
  // two independent compensated sums (lanes .x/.y and .z/.w) halve the FADD chain
  float sum = 0.f, comp = 0.f, sum1 = 0.f, comp1 = 0.f;
  const int64_t step = (int64_t)gridDim.x * kRedThreads * U;
  int64_t base = (int64_t)blockIdx.x * kRedThreads * U + threadIdx.x;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 ca[U], cb[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = base + (int64_t)u * kRedThreads;
    ca[u] = (i < nvec) ? __ldcs(a + i) : z;
    cb[u] = (i < nvec) ? __ldcs(b + i) : z;
  }
  for (; base < nvec; base += step) {
    float4 na[U], nb[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + step + (int64_t)u * kRedThreads;
      na[u] = (i < nvec) ? __ldcs(a + i) : z;
      nb[u] = (i < nvec) ? __ldcs(b + i) : z;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      dot2_step(ca[u].x, cb[u].x, sum, comp);
      dot2_step(ca[u].z, cb[u].z, sum1, comp1);
      dot2_step(ca[u].y, cb[u].y, sum, comp);
      dot2_step(ca[u].w, cb[u].w, sum1, comp1);
      ca[u] = na[u];
      cb[u] = nb[u];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int64_t t = nvec * 4; t < n; ++t) dot2_step(as[t], bs[t], sum, comp);
  }
  const double bv = block_sum(((double)sum + (double)comp) + ((double)sum1 + (double)comp1), s);
  finish_ticket(bv, sc, out, s);
}

// ------------------------------------------------------------------ BS3 norm on the integer pipe
//
// sum a*a with the per-element work on the integer pipe (sp_sumsq.cuh): a fixed
// grid of kNormCtas CTAs per SM, U 16-byte loads per lane issued before use, one
// fixed-point accumulator per lane, double-double across lanes and blocks in a
// fixed order (deterministic for a given n and device), the last block to arrive
// adds the block partials.  The result is within a few ulps of the exactly
// rounded sum for every input.  With nzero > 1 the last block also writes
// out[1 .. nzero) = 0, so that the reference's stage 2 (bs3_2 over nzero
// partials, an exact sum of zeros) returns out[0] unchanged.


// A block's (or a lane's) integer-pipe accumulator in 32 bytes of scratch or
// shared memory: the four words, the window top, and the FP64 side sum.
struct AccBits {
  uint32_t a0, a1, a2, a3, e20, pad;
  double f;
};
static_assert(sizeof(AccBits) == kRedPartialBytes, "one scratch slot per block");

__device__ __forceinline__ void store_acc(AccBits* d, const sumsq::Acc& a) {
  d->a0 = a.a0;
  d->a1 = a.a1;
  d->a2 = a.a2;
  d->a3 = a.a3;
  d->e20 = a.e20;
  d->f = a.f;
}
// From shared memory (plain loads).
__device__ __forceinline__ sumsq::Acc load_acc_shared(const AccBits* d) {
  sumsq::Acc a;
  a.a0 = d->a0;
  a.a1 = d->a1;
  a.a2 = d->a2;
  a.a3 = d->a3;
  a.e20 = d->e20;
  a.f = d->f;
  return a;
}
// From the global scratch written by other blocks (loads that bypass L1; these
// are global-space loads and must never be given a shared-memory address).
__device__ __forceinline__ sumsq::Acc load_acc_global(const AccBits* d) {
  sumsq::Acc a;
  a.a0 = __ldcg(&d->a0);
  a.a1 = __ldcg(&d->a1);
  a.a2 = __ldcg(&d->a2);
  a.a3 = __ldcg(&d->a3);
  a.e20 = __ldcg(&d->e20);
  a.f = __ldcg(&d->f);
  return a;
}

// The lanes' accumulators of a warp summed into lane 0: aligned to the warp's
// largest window top, then 128-bit adds down a shuffle tree; side sums in FP64.
__device__ __forceinline__ void warp_merge(sumsq::Acc& acc) {
  sumsq::align_to(acc, __reduce_max_sync(0xffffffffu, acc.e20));
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const uint32_t b0 = __shfl_down_sync(0xffffffffu, acc.a0, h);
    const uint32_t b1 = __shfl_down_sync(0xffffffffu, acc.a1, h);
    const uint32_t b2 = __shfl_down_sync(0xffffffffu, acc.a2, h);
    const uint32_t b3 = __shfl_down_sync(0xffffffffu, acc.a3, h);
    sumsq::add128(acc, b0, b1, b2, b3);
  }
  if (__any_sync(0xffffffffu, acc.f != 0.0)) {
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) acc.f += __shfl_down_sync(0xffffffffu, acc.f, h);
  }
}

// The block's sum as one accumulator (valid in thread 0): warps merge in
// integers, thread 0 merges the warps' sums in warp order.
__device__ __forceinline__ sumsq::Acc block_merge(sumsq::Acc acc, AccBits* sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  warp_merge(acc);
  if (lane == 0) store_acc(sm + w, acc);
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) sumsq::merge(acc, load_acc_shared(sm + i));
  __syncthreads();
  return acc;
}

// Bits the block partials drop when the last block sums them: the grid's total
// then fits 128 bits for up to 2^41 elements.
constexpr int kGridShift = 8;

// Writes the block's accumulator (from thread 0), and lets the last block to arrive
// sum the block partials in integers -- lane t takes blocks t, t + 256, ..., then
// the warps and the block as above -- and round the total once into out[0];
// out[1 .. nzero) = 0.
__device__ __forceinline__ void finish_ticket_acc(const sumsq::Acc& bacc, RedScratch sc,
                                                  double* out, AccBits* sm, int nzero) {
  __shared__ bool last;
  AccBits* part = reinterpret_cast<AccBits*>(sc.partial);
  if (threadIdx.x == 0) {
    store_acc(part + blockIdx.x, bacc);
    __threadfence();
    const unsigned t = atomicAdd(sc.ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  sumsq::Acc a;
  sumsq::init(a);
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    sumsq::Acc b = load_acc_global(part + i);
    sumsq::shift_down(b, kGridShift);
    sumsq::merge(a, b);
  }
  a = block_merge(a, sm);
  if (threadIdx.x == 0) {
    const sumsq::DD r = sumsq::value(a, kGridShift);
    out[0] = r.hi + r.lo;
    *sc.ticket = 0u;  // leave the scratch zeroed for the next call
  }
  for (int i = 1 + threadIdx.x; i < nzero; i += blockDim.x) out[i] = 0.0;
}

template <int U, int CTAS, bool ROLL>
__global__ void __launch_bounds__(kRedThreads, CTAS)
k_norm2_int(int64_t nvec, const double2* __restrict__ a, const double* __restrict__ as, int64_t n,
            void* scratch, double* out, int nzero) {
  __shared__ AccBits s[kRedThreads / 32];
  const RedScratch sc = red_scratch(scratch);
  sumsq::Acc acc;
  sumsq::init(acc);
  const int64_t step = (int64_t)gridDim.x * kRedThreads * U;
  int64_t base = (int64_t)blockIdx.x * kRedThreads * U + threadIdx.x;
  if (ROLL) {
    double2 cur[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * kRedThreads;
      cur[u] = (i < nvec) ? __ldcs(a + i) : make_double2(0.0, 0.0);
    }
    for (; base < nvec; base += step) {
      double2 nxt[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = base + step + (int64_t)u * kRedThreads;
        nxt[u] = (i < nvec) ? __ldcs(a + i) : make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        sumsq::add(acc, cur[u].x);
        sumsq::add(acc, cur[u].y);
        cur[u] = nxt[u];
      }
    }
  } else {
    for (; base < nvec; base += step) {
      double2 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = base + (int64_t)u * kRedThreads;
        v[u] = (i < nvec) ? __ldcs(a + i) : make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        sumsq::add(acc, v[u].x);
        sumsq::add(acc, v[u].y);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) sumsq::add(acc, as[n - 1]);
  finish_ticket_acc(block_merge(acc, s), sc, out, s, nzero);
}

// Resident CTAs per SM (knob reduce.norm_ctas: 4 or 6; the kernel fits 6 x 256
// lanes in the register file) and the persistent grid of that many per SM.
static unsigned norm_grid(int64_t nvec, int U, int ctas) {
  int64_t per = (int64_t)kRedThreads * U;
  int64_t g = (nvec + per - 1) / per;
  int64_t cap = (int64_t)ctas * sm_count();
  if (cap > kMaxRedBlocks) cap = kMaxRedBlocks;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

static void launch_norm2_int(int64_t n, const double* a, void* scratch, double* out, int nzero,
                             cudaStream_t s) {
  constexpr int U = 4;
  const int64_t nvec = n / 2;
  const auto* a2 = reinterpret_cast<const double2*>(a);
  const int ctas = tune(kTuneNormCtas) == 6 ? 6 : 4;
  const unsigned g = norm_grid(nvec, U, ctas);
  if (ctas == 6 && tune(kTuneNormRoll))  // two vectors per lane ahead fit 6 CTAs per SM
    k_norm2_int<2, 6, true><<<norm_grid(nvec, 2, 6), kRedThreads, 0, s>>>(nvec, a2, a, n, scratch,
                                                                           out, nzero);
  else if (ctas == 6)
    k_norm2_int<U, 6, false><<<g, kRedThreads, 0, s>>>(nvec, a2, a, n, scratch, out, nzero);
  else if (tune(kTuneNormRoll))
    k_norm2_int<U, 4, true><<<g, kRedThreads, 0, s>>>(nvec, a2, a, n, scratch, out, nzero);
  else
    k_norm2_int<U, 4, false><<<g, kRedThreads, 0, s>>>(nvec, a2, a, n, scratch, out, nzero);
}

// FP32-storage norm: compensated FP32 partials (Dot2 steps, two independent
// chains) over a rolling load pipeline -- the next U vectors of a lane are in
// flight while the current ones are summed -- on a grid of the CTAs the SMs hold
// at once; FP64 across lanes and blocks.
template <int U>
__global__ void __launch_bounds__(kRedThreads, 4)
k_norm2_f32(int64_t nvec, const float4* __restrict__ a, const float* __restrict__ as, int64_t n,
            void* scratch, double* out) {
  __shared__ double s[32];
  const RedScratch sc = red_scratch(scratch);
  float sum = 0.f, comp = 0.f, sum1 = 0.f, comp1 = 0.f;
  const int64_t step = (int64_t)gridDim.x * kRedThreads * U;
  int64_t base = (int64_t)blockIdx.x * kRedThreads * U + threadIdx.x;
  float4 cur[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = base + (int64_t)u * kRedThreads;
    cur[u] = (i < nvec) ? __ldcs(a + i) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (; base < nvec; base += step) {
    float4 nxt[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + step + (int64_t)u * kRedThreads;
      nxt[u] = (i < nvec) ? __ldcs(a + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      dot2_step(cur[u].x, cur[u].x, sum, comp);
      dot2_step(cur[u].z, cur[u].z, sum1, comp1);
      dot2_step(cur[u].y, cur[u].y, sum, comp);
      dot2_step(cur[u].w, cur[u].w, sum1, comp1);
      cur[u] = nxt[u];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int64_t t = nvec * 4; t < n; ++t) dot2_step(as[t], as[t], sum, comp);
  }
  const double bv = block_sum(((double)sum + (double)comp) + ((double)sum1 + (double)comp1), s);
  finish_ticket(bv, sc, out, s);
}

// FULL: x += alpha p ; r -= alpha Ap ; out = sum r*r     (FP64 storage)
// !FULL (the reference's BS5 update): r += alpha Ap ; out = sum r*r
// The updates are FP64 fma (bit-exact); sum r*r takes the integer-pipe
// accumulator of the norm (one DFMA per entry fewer, within a few ulps of the
// exactly rounded sum of the stored r).
template <int U, bool FULL = true>
__global__ void __launch_bounds__(kRedThreads)
k_cg_f64(int64_t nvec, double alpha, const double2* __restrict__ p, const double2* __restrict__ Ap,
         double2* __restrict__ x, double2* __restrict__ r, const double* __restrict__ ps,
         const double* __restrict__ Aps, double* __restrict__ xs, double* __restrict__ rs,
         int64_t n, void* scratch, double* out, int nzero) {
  __shared__ AccBits s[kRedThreads / 32];
  const RedScratch sc = red_scratch(scratch);
  sumsq::Acc acc;
  sumsq::init(acc);
  const int64_t step = (int64_t)gridDim.x * kRedThreads * U;
  for (int64_t base = (int64_t)blockIdx.x * kRedThreads * U + threadIdx.x; base < nvec;
       base += step) {
    double2 vp[U], va[U], vx[U], vr[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * kRedThreads;
      if (i < nvec) {
        if (FULL) {
          vp[u] = __ldcs(p + i);
          vx[u] = __ldcs(x + i);
        }
        va[u] = __ldcs(Ap + i);
        vr[u] = __ldcs(r + i);
      }
    }
    const double ar = FULL ? -alpha : alpha;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * kRedThreads;
      if (i < nvec) {
        double2 nr;
        if (FULL) {
          double2 nx;
          nx.x = fma(alpha, vp[u].x, vx[u].x);
          nx.y = fma(alpha, vp[u].y, vx[u].y);
          __stcs(x + i, nx);
        }
        nr.x = fma(ar, va[u].x, vr[u].x);
        nr.y = fma(ar, va[u].y, vr[u].y);
        __stcs(r + i, nr);
        sumsq::add(acc, nr.x);
        sumsq::add(acc, nr.y);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) {
    const int64_t t = n - 1;
    if (FULL) xs[t] = fma(alpha, ps[t], xs[t]);
    const double nr = fma(FULL ? -alpha : alpha, Aps[t], rs[t]);
    rs[t] = nr;
    sumsq::add(acc, nr);
  }
  finish_ticket_acc(block_merge(acc, s), sc, out, s, nzero);
}

// FP32 storage: x, r, p, Ap in FP32; update in FP32 with alpha rounded to FP32;
// r.r with compensated FP32 lanes and an FP64 cross-block finish.  FULL as k_cg_f64.
template <int U, bool FULL = true>
__global__ void __launch_bounds__(kRedThreads)
k_cg_f32(int64_t nvec, float alpha, const float4* __restrict__ p, const float4* __restrict__ Ap,
         float4* __restrict__ x, float4* __restrict__ r, const float* __restrict__ ps,
         const float* __restrict__ Aps, float* __restrict__ xs, float* __restrict__ rs, int64_t n,
         void* scratch, double* out) {
  __shared__ double s[32];
  const RedScratch sc = red_scratch(scratch);
  float sum = 0.f, comp = 0.f, sum1 = 0.f, comp1 = 0.f;
  const int64_t step = (int64_t)gridDim.x * kRedThreads * U;
  for (int64_t base = (int64_t)blockIdx.x * kRedThreads * U + threadIdx.x; base < nvec;
       base += step) {
    float4 vp[U], va[U], vx[U], vr[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * kRedThreads;
      if (i < nvec) {
        if (FULL) {
          vp[u] = __ldcs(p + i);
          vx[u] = __ldcs(x + i);
        }
        va[u] = __ldcs(Ap + i);
        vr[u] = __ldcs(r + i);
      }
    }
    const float ar = FULL ? -alpha : alpha;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + (int64_t)u * kRedThreads;
      if (i < nvec) {
        float4 nr;
        if (FULL) {
          float4 nx;
          nx.x = fmaf(alpha, vp[u].x, vx[u].x);
          nx.y = fmaf(alpha, vp[u].y, vx[u].y);
          nx.z = fmaf(alpha, vp[u].z, vx[u].z);
          nx.w = fmaf(alpha, vp[u].w, vx[u].w);
          __stcs(x + i, nx);
        }
        nr.x = fmaf(ar, va[u].x, vr[u].x);
        nr.y = fmaf(ar, va[u].y, vr[u].y);
        nr.z = fmaf(ar, va[u].z, vr[u].z);
        nr.w = fmaf(ar, va[u].w, vr[u].w);
        __stcs(r + i, nr);
        dot2_step(nr.x, nr.x, sum, comp);
        dot2_step(nr.z, nr.z, sum1, comp1);
        dot2_step(nr.y, nr.y, sum, comp);
        dot2_step(nr.w, nr.w, sum1, comp1);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int64_t t = nvec * 4; t < n; ++t) {
      if (FULL) xs[t] = fmaf(alpha, ps[t], xs[t]);
      const float nr = fmaf(FULL ? -alpha : alpha, Aps[t], rs[t]);
      rs[t] = nr;
      dot2_step(nr, nr, sum, comp);
    }
  }
  const double bv = block_sum(((double)sum + (double)comp) + ((double)sum1 + (double)comp1), s);
  finish_ticket(bv, sc, out, s);
}

// CTAs of `kernel` (kRedThreads lanes each) that one SM holds at once, per device.
static int resident_ctas(const void* kernel) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find({kernel, dev});
  if (it != cache.end()) return it->second;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kRedThreads, 0) != cudaSuccess ||
      nb < 1) {
    cudaGetLastError();
    nb = 1;
  }
  cache[{kernel, dev}] = nb;
  return nb;
}

// Persistent grid of the single-launch reductions: as many CTAs as the SMs hold at
// once (no CTA waits for a second wave while the others stream), at most one CTA
// per U*kRedThreads vectors, at most kMaxRedBlocks.
static unsigned red_grid(const void* kernel, int64_t nvec, int U) {
  int64_t per = (int64_t)kRedThreads * U;
  int64_t g = (nvec + per - 1) / per;
  int64_t cap = (int64_t)resident_ctas(kernel) * sm_count();
  if (cap > kMaxRedBlocks) cap = kMaxRedBlocks;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

static sp_status check_red_args(int64_t n, const void* scratch, const void* out,
                                std::initializer_list<const void*> vecs, const char* name) {
  if (n < 0) return fail(SP_ERR_INVALID_ARG, "%s: negative length", name);
  if (!scratch || !out) return fail(SP_ERR_INVALID_ARG, "%s: null scratch/out", name);
  if (reinterpret_cast<uintptr_t>(scratch) & 255u)
    return fail(SP_ERR_INVALID_ARG, "%s: scratch must be 256-byte aligned", name);
  for (const void* v : vecs) {
    if (n > 0 && !v) return fail(SP_ERR_INVALID_ARG, "%s: null vector", name);
    if (n > 0 && !aligned16(v))
      return fail(SP_ERR_INVALID_ARG, "%s: vectors must be 16-byte aligned", name);
  }
  return SP_SUCCESS;
}

}  // namespace sp

using namespace sp;

extern "C" {

sp_status sp_bs0(int32_t n, const double* a, double* b, sp_stream_t stream) {
  if (!b && n == 0) return fail(SP_ERR_INVALID_ARG, "sp_bs0: null output with n == 0");
  k_bs0<<<1, 1, 0, as_cuda(stream)>>>(n, a, b);
  return check_launch("sp_bs0");
}

sp_status sp_bs1_copy_f64(int64_t n, const double* a, double* b, sp_stream_t stream) {
  return launch_copy<double>(n, a, b, as_cuda(stream), "sp_bs1_copy_f64");
}
sp_status sp_bs1_copy_f32(int64_t n, const float* a, float* b, sp_stream_t stream) {
  return launch_copy<float>(n, a, b, as_cuda(stream), "sp_bs1_copy_f32");
}

sp_status sp_bs2_axpy_f64(int64_t n, double alpha, const double* x, double beta, double* y,
                          sp_stream_t stream) {
  return launch_axpy<double>(n, alpha, x, beta, y, as_cuda(stream), "sp_bs2_axpy_f64");
}
sp_status sp_bs2_axpy_f32(int64_t n, float alpha, const float* x, float beta, float* y,
                          sp_stream_t stream) {
  return launch_axpy<float>(n, alpha, x, beta, y, as_cuda(stream), "sp_bs2_axpy_f32");
}

sp_status sp_bs3_1_f64(int32_t bs, int32_t nblocks, int64_t n, const double* a, double* partial,
                       sp_stream_t stream) {
  sp_status st = check_exact_args(bs, nblocks, n, "sp_bs3_1_f64");
  if (st) return st;
  if (!partial || (n > 0 && !a)) return fail(SP_ERR_INVALID_ARG, "sp_bs3_1_f64: null pointer");
  cudaStream_t s = as_cuda(stream);
  launch_bs3(bs, nblocks, n, a, partial, s);
  return check_launch("sp_bs3_1_f64");
}

sp_status sp_bs4_1_f64(int32_t bs, int32_t nblocks, int64_t n, const double* a, const double* b,
                       double* partial, sp_stream_t stream) {
  sp_status st = check_exact_args(bs, nblocks, n, "sp_bs4_1_f64");
  if (st) return st;
  if (!partial || (n > 0 && (!a || !b)))
    return fail(SP_ERR_INVALID_ARG, "sp_bs4_1_f64: null pointer");
  cudaStream_t s = as_cuda(stream);
  launch_bs4(bs, nblocks, n, a, b, partial, s);
  return check_launch("sp_bs4_1_f64");
}

sp_status sp_bs5_1_f64(int32_t bs, int32_t nblocks, int64_t n, const double* Ap, double alpha,
                       double* r, double* partial, sp_stream_t stream) {
  sp_status st = check_exact_args(bs, nblocks, n, "sp_bs5_1_f64");
  if (st) return st;
  if (!partial || (n > 0 && (!Ap || !r)))
    return fail(SP_ERR_INVALID_ARG, "sp_bs5_1_f64: null pointer");
  cudaStream_t s = as_cuda(stream);
  launch_bs5(bs, nblocks, n, Ap, alpha, r, partial, s);
  return check_launch("sp_bs5_1_f64");
}

sp_status sp_reduce_finish_f64(int32_t bs, int32_t nblocks, const double* partial, double* out,
                               sp_stream_t stream) {
  sp_status st = check_exact_args(bs, nblocks, 0, "sp_reduce_finish_f64");
  if (st) return st;
  if (!partial || !out) return fail(SP_ERR_INVALID_ARG, "sp_reduce_finish_f64: null pointer");
  cudaStream_t s = as_cuda(stream);
  if (bs == 256) k_finish<256><<<1, 256, 0, s>>>(nblocks, partial, out);
  else if (bs == 512) k_finish<512><<<1, 512, 0, s>>>(nblocks, partial, out);
  else k_finish<1024><<<1, 1024, 0, s>>>(nblocks, partial, out);
  return check_launch("sp_reduce_finish_f64");
}

size_t sp_reduce_scratch_bytes(void) { return kRedScratchSize; }

sp_status sp_dot_f64(int64_t n, const double* a, const double* b, double* out, void* scratch,
                     sp_stream_t stream) {
  sp_status st = check_red_args(n, scratch, out, {a, b}, "sp_dot_f64");
  if (st) return st;
  constexpr int U = 4;
  const int64_t nvec = n / 2;
  k_dot_f64_fast<U><<<red_grid((const void*)k_dot_f64_fast<U>, nvec, U), kRedThreads, 0,
                      as_cuda(stream)>>>(
      nvec, reinterpret_cast<const double2*>(a), reinterpret_cast<const double2*>(b), a, b, n,
      scratch, out);
  return check_launch("sp_dot_f64");
}

sp_status sp_norm2_f64(int64_t n, const double* a, double* out, void* scratch,
                       sp_stream_t stream) {
  sp_status st = check_red_args(n, scratch, out, {a}, "sp_norm2_f64");
  if (st) return st;
  launch_norm2_int(n, a, scratch, out, 1, as_cuda(stream));
  return check_launch("sp_norm2_f64");
}

sp_status sp_bs3_1_fast_f64(int32_t bs, int32_t nblocks, int64_t n, const double* a,
                            double* partial, void* scratch, sp_stream_t stream) {
  sp_status st = check_exact_args(bs, nblocks, n, "sp_bs3_1_fast_f64");
  if (st) return st;
  if ((st = check_red_args(n, scratch, partial, {a}, "sp_bs3_1_fast_f64"))) return st;
  launch_norm2_int(n, a, scratch, partial, nblocks, as_cuda(stream));
  return check_launch("sp_bs3_1_fast_f64");
}

sp_status sp_dot_f32(int64_t n, const float* a, const float* b, double* out, void* scratch,
                     sp_stream_t stream) {
  sp_status st = check_red_args(n, scratch, out, {a, b}, "sp_dot_f32");
  if (st) return st;
  constexpr int U = 2;
  const int64_t nvec = n / 4;
  k_dot_f32_fast<U><<<red_grid((const void*)k_dot_f32_fast<U>, nvec, U), kRedThreads, 0,
                      as_cuda(stream)>>>(
      nvec, reinterpret_cast<const float4*>(a), reinterpret_cast<const float4*>(b), a, b, n,
      scratch, out);
  return check_launch("sp_dot_f32");
}

sp_status sp_norm2_f32(int64_t n, const float* a, double* out, void* scratch,
                       sp_stream_t stream) {
  sp_status st = check_red_args(n, scratch, out, {a}, "sp_norm2_f32");
  if (st) return st;
  constexpr int U = 4;
  const int64_t nvec = n / 4;
  k_norm2_f32<U><<<red_grid((const void*)k_norm2_f32<U>, nvec, U), kRedThreads, 0,
                   as_cuda(stream)>>>(nvec, reinterpret_cast<const float4*>(a), a, n, scratch,
                                      out);
  return check_launch("sp_norm2_f32");
}

sp_status sp_cg_update_f64(int64_t n, double alpha, const double* p, const double* Ap, double* x,
                           double* r, double* rdotr, void* scratch, sp_stream_t stream) {
  sp_status st = check_red_args(n, scratch, rdotr, {p, Ap, x, r}, "sp_cg_update_f64");
  if (st) return st;
  constexpr int U = 2;
  const int64_t nvec = n / 2;
  k_cg_f64<U><<<red_grid((const void*)k_cg_f64<U>, nvec, U), kRedThreads, 0,
                as_cuda(stream)>>>(
      nvec, alpha, reinterpret_cast<const double2*>(p), reinterpret_cast<const double2*>(Ap),
      reinterpret_cast<double2*>(x), reinterpret_cast<double2*>(r), p, Ap, x, r, n, scratch,
      rdotr, 1);
  return check_launch("sp_cg_update_f64");
}

sp_status sp_cg_update_f32(int64_t n, double alpha, const float* p, const float* Ap, float* x,
                           float* r, double* rdotr, void* scratch, sp_stream_t stream) {
  sp_status st = check_red_args(n, scratch, rdotr, {p, Ap, x, r}, "sp_cg_update_f32");
  if (st) return st;
  constexpr int U = 2;
  const int64_t nvec = n / 4;
  k_cg_f32<U><<<red_grid((const void*)k_cg_f32<U>, nvec, U), kRedThreads, 0,
                as_cuda(stream)>>>(
      nvec, (float)alpha, reinterpret_cast<const float4*>(p), reinterpret_cast<const float4*>(Ap),
      reinterpret_cast<float4*>(x), reinterpret_cast<float4*>(r), p, Ap, x, r, n, scratch, rdotr);
  return check_launch("sp_cg_update_f32");
}

sp_status sp_cg_update_ref_f64(int64_t n, double alpha, const double* Ap, double* r,
                               double* rdotr, void* scratch, sp_stream_t stream) {
  sp_status st = check_red_args(n, scratch, rdotr, {Ap, r}, "sp_cg_update_ref_f64");
  if (st) return st;
  constexpr int U = 2;
  const int64_t nvec = n / 2;
  k_cg_f64<U, false><<<red_grid((const void*)k_cg_f64<U, false>, nvec, U), kRedThreads, 0,
                       as_cuda(stream)>>>(
      nvec, alpha, nullptr, reinterpret_cast<const double2*>(Ap), nullptr,
      reinterpret_cast<double2*>(r), nullptr, Ap, nullptr, r, n, scratch, rdotr, 1);
  return check_launch("sp_cg_update_ref_f64");
}

sp_status sp_bs5_1_fast_f64(int32_t bs, int32_t nblocks, int64_t n, const double* Ap,
                            double alpha, double* r, double* partial, void* scratch,
                            sp_stream_t stream) {
  sp_status st = check_exact_args(bs, nblocks, n, "sp_bs5_1_fast_f64");
  if (st) return st;
  if ((st = check_red_args(n, scratch, partial, {Ap, r}, "sp_bs5_1_fast_f64"))) return st;
  constexpr int U = 2;
  const int64_t nvec = n / 2;
  k_cg_f64<U, false><<<red_grid((const void*)k_cg_f64<U, false>, nvec, U), kRedThreads, 0,
                       as_cuda(stream)>>>(
      nvec, alpha, nullptr, reinterpret_cast<const double2*>(Ap), nullptr,
      reinterpret_cast<double2*>(r), nullptr, Ap, nullptr, r, n, scratch, partial, nblocks);
  return check_launch("sp_bs5_1_fast_f64");
}

sp_status sp_cg_update_ref_f32(int64_t n, double alpha, const float* Ap, float* r,
                               double* rdotr, void* scratch, sp_stream_t stream) {
  sp_status st = check_red_args(n, scratch, rdotr, {Ap, r}, "sp_cg_update_ref_f32");
  if (st) return st;
  constexpr int U = 2;
  const int64_t nvec = n / 4;
  k_cg_f32<U, false><<<red_grid((const void*)k_cg_f32<U, false>, nvec, U), kRedThreads, 0,
                       as_cuda(stream)>>>(
      nvec, (float)alpha, nullptr, reinterpret_cast<const float4*>(Ap), nullptr,
      reinterpret_cast<float4*>(r), nullptr, Ap, nullptr, r, n, scratch, rdotr);
  return check_launch("sp_cg_update_ref_f32");
}

// ------------------------------------------------------------------ BS0 graph form

}  // extern "C"

static thread_local int64_t g_capture_start = 0;

struct sp_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int32_t nlaunches = 0;
};

extern "C" {

sp_status sp_bs0_graph_create(int32_t nlaunches, int32_t n, const double* a, double* b,
                              sp_stream_t stream, sp_graph** out) {
  if (!out || nlaunches < 1) return fail(SP_ERR_INVALID_ARG, "sp_bs0_graph_create: bad args");
  if (!b && n == 0) return fail(SP_ERR_INVALID_ARG, "sp_bs0_graph_create: null output");
  *out = nullptr;
  cudaStream_t cap = nullptr;
  SP_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  sp_graph* g = new sp_graph();
  g->nlaunches = nlaunches;
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    for (int i = 0; i < nlaunches; ++i) k_bs0<<<1, 1, 0, cap>>>(n, a, b);
    e = cudaStreamEndCapture(cap, &g->graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e == cudaSuccess) e = cudaGraphUpload(g->exec, as_cuda(stream));
  cudaStreamDestroy(cap);
  if (e != cudaSuccess) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return fail(SP_ERR_CUDA, "sp_bs0_graph_create: %s", cudaGetErrorString(e));
  }
  *out = g;
  return SP_SUCCESS;
}

sp_status sp_graph_begin(sp_stream_t stream) {
  if (!stream) return fail(SP_ERR_INVALID_ARG, "sp_graph_begin: capture needs a created stream");
  SP_CUDA_TRY(cudaStreamBeginCapture(as_cuda(stream), cudaStreamCaptureModeThreadLocal));
  g_capture_start = sp_launch_count();
  return SP_SUCCESS;
}

sp_status sp_graph_end(sp_stream_t stream, sp_graph** out) {
  if (!stream || !out) return fail(SP_ERR_INVALID_ARG, "sp_graph_end: null argument");
  *out = nullptr;
  sp_graph* g = new sp_graph();
  cudaError_t e = cudaStreamEndCapture(as_cuda(stream), &g->graph);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e == cudaSuccess) e = cudaGraphUpload(g->exec, as_cuda(stream));
  if (e != cudaSuccess) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    cudaGetLastError();
    return fail(SP_ERR_CUDA, "sp_graph_end: %s", cudaGetErrorString(e));
  }
  g->nlaunches = (int32_t)(sp_launch_count() - g_capture_start);
  // launches recorded into the graph ran nothing yet: count them when it is replayed
  count_launch(-(int64_t)g->nlaunches);
  *out = g;
  return SP_SUCCESS;
}

sp_status sp_graph_launch(const sp_graph* g, sp_stream_t stream) {
  if (!g || !g->exec) return fail(SP_ERR_INVALID_ARG, "sp_graph_launch: null graph");
  SP_CUDA_TRY(cudaGraphLaunch(g->exec, as_cuda(stream)));
  count_launch(g->nlaunches);
  return SP_SUCCESS;
}

sp_status sp_graph_destroy(sp_graph* g) {
  if (!g) return SP_SUCCESS;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return SP_SUCCESS;
}

}  // extern "C"

// ------------------------------------------------------------------ allocation-free BS4 dot
//
// For callers that cannot allocate device memory themselves -- e.g. a solver whose
// device memory all belongs to another allocator or a fixed pool, or code that must
// not pay cudaMalloc's device-wide synchronisation inside its loop -- and so cannot
// provide the partial-sum buffer that sp_bs4_1_f64 needs.  The partial sums live
// in a static device array of the library instead: every GPU that loads the
// library holds these kNoAllocMaxBlocks doubles (8 KiB) until the process exits.

namespace sp {

constexpr int kNoAllocMaxBlocks = 1024;
static __device__ __align__(256) double g_noalloc_partial[kNoAllocMaxBlocks];

// Device address of g_noalloc_partial, looked up once per device (with that device
// current) on the first call there.
constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static double* g_noalloc_addr[kNoAllocMaxDevices] = {};

static sp_status noalloc_partials(double** out) {
  int dev = 0;
  SP_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(SP_ERR_UNSUPPORTED, "sp_bs4_dot_f64_noalloc: device %d beyond %d", dev,
                kNoAllocMaxDevices);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
    if (e != cudaSuccess || !p)
      return fail(SP_ERR_CUDA, "sp_bs4_dot_f64_noalloc: cudaGetSymbolAddress failed: %s",
                  cudaGetErrorString(e));
    g_noalloc_addr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_addr[dev];
  return SP_SUCCESS;
}

}  // namespace sp

extern "C" {

sp_status sp_bs4_dot_f64_noalloc(int32_t bs, int32_t nblocks, int64_t n, const double* a,
                                 const double* b, double* out, sp_stream_t stream) {
  if (nblocks > kNoAllocMaxBlocks)
    return fail(SP_ERR_SIZE,
                "sp_bs4_dot_f64_noalloc: nblocks %d exceeds the static partial-sum capacity %d",
                nblocks, kNoAllocMaxBlocks);
  sp_status st = check_exact_args(bs, nblocks, n, "sp_bs4_dot_f64_noalloc");
  if (st) return st;
  if (!out || (n > 0 && (!a || !b)))
    return fail(SP_ERR_INVALID_ARG, "sp_bs4_dot_f64_noalloc: null pointer");
  double* partial = nullptr;
  if ((st = noalloc_partials(&partial))) return st;
  // stage 1 writes partial[0, nblocks) in full before stage 2 reads it, so nothing
  // in the shared array has to start at zero
  cudaStream_t s = as_cuda(stream);
  launch_bs4(bs, nblocks, n, a, b, partial, s);
  if ((st = check_launch("sp_bs4_dot_f64_noalloc"))) return st;
  if (bs == 256) k_finish<256><<<1, 256, 0, s>>>(nblocks, partial, out);
  else if (bs == 512) k_finish<512><<<1, 512, 0, s>>>(nblocks, partial, out);
  else k_finish<1024><<<1, 1024, 0, s>>>(nblocks, partial, out);
  return check_launch("sp_bs4_dot_f64_noalloc");
}

}  // extern "C"
