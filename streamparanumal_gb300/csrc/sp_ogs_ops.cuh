// Element operations of the ogs kernels, shared by the translation units that
// gather (sp_ogs.cu: block, chunk and staged kernels; sp_ogs_slab.cu: lane-row
// slabs), so every kernel combines with the same identities and rules.
#pragma once

#include <cstdint>

#include "../../include/sp_capi.h"

namespace sp {

// ------------------------------------------------------------------ ops
// Identities and update rules of libs/ogs/ogsUtils.cpp:62-103 (device) and
// libs/ogs/ogsOperator.cpp:37-56 (host): Max/Min start from -+numeric max and
// keep the current value unless the new one compares strictly greater/less.
template <typename T> struct Lim;
template <> struct Lim<float>  { static __device__ float big()  { return 3.402823466e+38f; } };
template <> struct Lim<double> { static __device__ double big() { return 1.7976931348623157e+308; } };
template <> struct Lim<int32_t> { static __device__ int32_t big() { return 2147483647; } };
template <> struct Lim<long long> { static __device__ long long big() { return 9223372036854775807LL; } };

template <typename T> __device__ __forceinline__ T wrap_add(T a, T b) { return a + b; }
template <typename T> __device__ __forceinline__ T wrap_mul(T a, T b) { return a * b; }
template <> __device__ __forceinline__ int32_t wrap_add(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a + (uint32_t)b);
}
template <> __device__ __forceinline__ int32_t wrap_mul(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a * (uint32_t)b);
}
template <> __device__ __forceinline__ long long wrap_add(long long a, long long b) {
  return (long long)((unsigned long long)a + (unsigned long long)b);
}
template <> __device__ __forceinline__ long long wrap_mul(long long a, long long b) {
  return (long long)((unsigned long long)a * (unsigned long long)b);
}

// first(v) is apply(init(), v) computed without floating-point arithmetic where
// that is exact: identity + v == v for every v except -0 (which becomes +0), and
// 1 * v == v.  On GB300 the FP64 pipe is narrow, and this removes one FP64 add per
// row -- every add of a multiplicity-1 row -- without changing a single bit.
__device__ __forceinline__ double plus_zero(double v) {
  const long long b = __double_as_longlong(v);
  return __longlong_as_double(b == (long long)0x8000000000000000ULL ? 0LL : b);
}
__device__ __forceinline__ float plus_zero(float v) {
  const int b = __float_as_int(v);
  return __int_as_float(b == (int)0x80000000u ? 0 : b);
}
__device__ __forceinline__ int32_t plus_zero(int32_t v) { return v; }
__device__ __forceinline__ long long plus_zero(long long v) { return v; }

template <typename T, int OP> struct Op;
template <typename T> struct Op<T, SP_OP_ADD> {
  static __device__ __forceinline__ T init() { return T(0); }
  static __device__ __forceinline__ T first(T v) { return plus_zero(v); }
  static __device__ __forceinline__ void apply(T& a, T b) { a = wrap_add(a, b); }
};
template <typename T> struct Op<T, SP_OP_MUL> {
  static __device__ __forceinline__ T init() { return T(1); }
  static __device__ __forceinline__ T first(T v) { return v; }
  static __device__ __forceinline__ void apply(T& a, T b) { a = wrap_mul(a, b); }
};
template <typename T> struct Op<T, SP_OP_MAX> {
  static __device__ __forceinline__ T init() { return -Lim<T>::big(); }
  static __device__ __forceinline__ T first(T v) {
    T a = init();
    apply(a, v);
    return a;
  }
  static __device__ __forceinline__ void apply(T& a, T b) { a = (b > a) ? b : a; }
};
template <typename T> struct Op<T, SP_OP_MIN> {
  static __device__ __forceinline__ T init() { return Lim<T>::big(); }
  static __device__ __forceinline__ T first(T v) {
    T a = init();
    apply(a, v);
    return a;
  }
  static __device__ __forceinline__ void apply(T& a, T b) { a = (b < a) ? b : a; }
};

// Combines s[a, b) in order from the op's identity.
template <typename T, int OP>
__device__ __forceinline__ T row_combine(const T* s, int32_t a, int32_t b) {
  if (a >= b) return Op<T, OP>::init();
  T acc = Op<T, OP>::first(s[a]);
  for (int32_t i = a + 1; i < b; ++i) Op<T, OP>::apply(acc, s[i]);
  return acc;
}


// Bit equality (x = first(x) for most values: then a gather+scatter need not store).
__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}
__device__ __forceinline__ bool same_bits(float a, float b) {
  return __float_as_int(a) == __float_as_int(b);
}
__device__ __forceinline__ bool same_bits(int32_t a, int32_t b) { return a == b; }
__device__ __forceinline__ bool same_bits(long long a, long long b) { return a == b; }

}  // namespace sp
