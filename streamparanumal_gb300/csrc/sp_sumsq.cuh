// Sum of squares of FP64 values on the integer pipe (the BS3 norm's fast form).
//
// GB300 issues 2 FP64 FMA lanes per SM per clock, so a norm that spends one DFMA
// per 8-byte element is capped near 5 TB/s, well under HBM.  Here the per-element
// work is integer arithmetic:
//
//   * an element a = m * 2^(E-1075) (m the 53-bit significand, E the biased
//     exponent) enters a per-thread fixed-point accumulator when E lies in a
//     window of kWin binades below the thread's largest exponent Emax so far;
//   * its square is formed from the top 31 and the low 22 bits of m with one
//     32x32->64 multiply-add and one high-half multiply: T ~ m^2 / 2^44 with a
//     relative error below 2^-59 (the dropped low-part square and two floors);
//   * T, shifted right by 2 (Emax - E), is added into a 128-bit accumulator in
//     which T at shift 0 occupies bits [32, 96) -- the 32 bits below keep what the
//     shift moves out, so nothing inside the window is truncated;
//   * a larger exponent moves the window up (the accumulator is shifted down);
//     elements more than kWin binades below Emax, subnormals, Inf and NaN are
//     added to an FP64 side sum with fma() -- FP64 semantics for the special
//     values, negligible weight for the rest;
//   * lanes, warps and blocks are combined as integers (aligned to the larger
//     window top, then 128-bit adds) in a fixed order, and the total becomes a
//     double once, at the end -- on GB300 a dependent FP64 operation costs a
//     whole warp slot of a 2-lane pipe, so a double-double tree over lanes or
//     blocks would cost microseconds per launch.
//
// The result is the sum of squares to about 2^-59 relative (each term's error
// is below that, and all terms are non-negative), i.e. it is within a few units
// in the last place of the exactly rounded value, for any input.  The
// reference's order-exact chain (bs3.okl:36-41) differs from the exact value by
// its own rounding; the two agree to well within 1e-14 relative.
//
// Everything here is plain C++ on the host as well, so the arithmetic is
// checked on the CPU against an exact sum.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define SP_SQ_HD __host__ __device__ __forceinline__
#else
#define SP_SQ_HD inline
#endif

namespace sp {
namespace sumsq {

constexpr uint32_t kWin = 15;            // binades below Emax kept on the integer path
constexpr uint32_t kExpMask = 0x7FF00000u;
// Initial window top: exponent 16, so E = 0 (zero, subnormal) always falls
// outside the window and never takes the implicit leading bit.
constexpr uint32_t kE20Init = 16u << 20;

struct Acc {
  uint32_t a0, a1, a2, a3;  // 128-bit fixed point; unit = 2^(2*Emax - 2138)
  uint32_t e20;             // Emax << 20 (the exponent field of the high word)
  double f;                 // FP64 sum of the squares outside the window
};

SP_SQ_HD void init(Acc& s) {
  s.a0 = s.a1 = s.a2 = s.a3 = 0u;
  s.e20 = kE20Init;
  s.f = 0.0;
}

// (hi:lo) << sh, high word; sh < 32
SP_SQ_HD uint32_t funnel_l(uint32_t lo, uint32_t hi, uint32_t sh) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(lo, hi, sh);
#else
  return (uint32_t)((((uint64_t)hi << 32) | lo) << sh >> 32);
#endif
}
// (hi:lo) >> sh, low word; sh < 32
SP_SQ_HD uint32_t funnel_r(uint32_t lo, uint32_t hi, uint32_t sh) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_r(lo, hi, sh);
#else
  return (uint32_t)((((uint64_t)hi << 32) | lo) >> sh);
#endif
}
SP_SQ_HD uint32_t mulhi(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// acc += (w2:w1:w0), carry into a3
SP_SQ_HD void add96(Acc& s, uint32_t w0, uint32_t w1, uint32_t w2) {
#if defined(__CUDA_ARCH__)
  asm("add.cc.u32 %0, %0, %4;\n\t"
      "addc.cc.u32 %1, %1, %5;\n\t"
      "addc.cc.u32 %2, %2, %6;\n\t"
      "addc.u32 %3, %3, 0;"
      : "+r"(s.a0), "+r"(s.a1), "+r"(s.a2), "+r"(s.a3)
      : "r"(w0), "r"(w1), "r"(w2));
#else
  uint64_t t = (uint64_t)s.a0 + w0;
  s.a0 = (uint32_t)t;
  t = (uint64_t)s.a1 + w1 + (t >> 32);
  s.a1 = (uint32_t)t;
  t = (uint64_t)s.a2 + w2 + (t >> 32);
  s.a2 = (uint32_t)t;
  s.a3 += (uint32_t)(t >> 32);
#endif
}

// acc += (b3:b2:b1:b0)
SP_SQ_HD void add128(Acc& s, uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3) {
#if defined(__CUDA_ARCH__)
  asm("add.cc.u32 %0, %0, %4;\n\t"
      "addc.cc.u32 %1, %1, %5;\n\t"
      "addc.cc.u32 %2, %2, %6;\n\t"
      "addc.u32 %3, %3, %7;"
      : "+r"(s.a0), "+r"(s.a1), "+r"(s.a2), "+r"(s.a3)
      : "r"(b0), "r"(b1), "r"(b2), "r"(b3));
#else
  uint64_t t = (uint64_t)s.a0 + b0;
  s.a0 = (uint32_t)t;
  t = (uint64_t)s.a1 + b1 + (t >> 32);
  s.a1 = (uint32_t)t;
  t = (uint64_t)s.a2 + b2 + (t >> 32);
  s.a2 = (uint32_t)t;
  s.a3 += b3 + (uint32_t)(t >> 32);
#endif
}

// Adds the square of the element with words (hi, lo), whose exponent lies s2/2
// binades below Emax (s2 = 2 (Emax - E) <= 2 kWin < 32).
SP_SQ_HD void add_window(Acc& s, uint32_t lo, uint32_t hi, uint32_t s2) {
  // bits 52..22 of the significand (implicit bit at 30) and bits 21..0 (left-aligned)
  const uint32_t m31 = (funnel_l(lo, hi, 10) & 0x3FFFFFFFu) | 0x40000000u;
  const uint32_t ml = lo << 10;
  // m^2 / 2^44 = m31^2 + m31 ml22 2^-21 + ml22^2 2^-44; the middle term is
  // floor((2 m31)(ml22 2^10) / 2^32), the last one (< 1) is dropped
  const uint64_t T = (uint64_t)m31 * m31 + mulhi(m31 << 1, ml);
  const uint32_t tl = (uint32_t)T, th = (uint32_t)(T >> 32);
  add96(s, funnel_r(0u, tl, s2), funnel_r(tl, th, s2), th >> s2);
}

// Shifts the accumulator right by sh bits (moving the window up by sh/2 binades).
SP_SQ_HD void shift_down(Acc& s, uint32_t sh) {
  uint64_t H = ((uint64_t)s.a3 << 32) | s.a2, L = ((uint64_t)s.a1 << 32) | s.a0;
  if (sh >= 128u) {
    H = L = 0u;
  } else if (sh >= 64u) {
    L = (sh == 64u) ? H : (H >> (sh - 64u));
    H = 0u;
  } else if (sh > 0u) {
    L = (L >> sh) | (H << (64u - sh));
    H >>= sh;
  }
  s.a3 = (uint32_t)(H >> 32);
  s.a2 = (uint32_t)H;
  s.a1 = (uint32_t)(L >> 32);
  s.a0 = (uint32_t)L;
}

// Moves the window top up to e20 >= s.e20 (the accumulator is shifted down; bits
// below its last place, under 2^-94 of the new unit's square scale, are dropped).
SP_SQ_HD void align_to(Acc& s, uint32_t e20) {
  shift_down(s, (e20 - s.e20) >> 19);
  s.e20 = e20;
}

SP_SQ_HD void add_outside(Acc& s, double a, uint32_t lo, uint32_t hi, uint32_t ef) {
  if (ef == kExpMask) {  // Inf or NaN: the FP64 result (Inf, or NaN)
    s.f = fma(a, a, s.f);
  } else if (ef > s.e20) {  // a new largest exponent: move the window up
    shift_down(s, (ef - s.e20) >> 19);
    s.e20 = ef;
    add_window(s, lo, hi, 0u);
  } else if (((hi << 1) | lo) != 0u) {  // more than kWin binades below Emax
    s.f = fma(a, a, s.f);
  }
}

SP_SQ_HD void add(Acc& s, double a) {
  uint64_t b;
#if defined(__CUDA_ARCH__)
  b = (uint64_t)__double_as_longlong(a);
#else
  std::memcpy(&b, &a, 8);
#endif
  const uint32_t lo = (uint32_t)b, hi = (uint32_t)(b >> 32);
  const uint32_t t = s.e20 - (hi & kExpMask);  // (Emax - E) << 20, wraps when E > Emax
  if (t <= (kWin << 20)) add_window(s, lo, hi, t >> 19);
  else if (((hi << 1) | lo) != 0u) add_outside(s, a, lo, hi, hi & kExpMask);  // +-0 adds nothing
}

// a += b: both aligned to the larger window top, then added as integers; the
// side sums are added in FP64.
SP_SQ_HD void merge(Acc& a, Acc b) {
  const uint32_t e = a.e20 > b.e20 ? a.e20 : b.e20;
  align_to(a, e);
  align_to(b, e);
  add128(a, b.a0, b.a1, b.a2, b.a3);
  a.f += b.f;
}

// ---------------------------------------------------------------- double-double
struct DD {
  double hi, lo;
};

// a + b for double-doubles (Knuth TwoSum on the high parts, then renormalise);
// a non-finite high part carries the FP64 result alone.
SP_SQ_HD DD dd_add(DD a, DD b) {
  const double s = a.hi + b.hi;
  if (!(fabs(s) <= 1.79769313486231570815e+308)) return DD{s, 0.0};
  const double bb = s - a.hi;
  const double e = (a.hi - (s - bb)) + (b.hi - bb) + a.lo + b.lo;
  const double h = s + e;
  return DD{h, e - (h - s)};
}

// The accumulator's value (plus the side sum) as a double-double: the four 32-bit
// words are exact doubles, added in double-double (any 128-bit value).  `extra`
// bits were shifted out of the words after accumulation (their unit is then
// 2^extra times the accumulator's).
SP_SQ_HD DD value(const Acc& s, int extra = 0) {
  DD v{0.0, 0.0};
  if (s.a0 | s.a1 | s.a2 | s.a3) {
    v = dd_add(DD{(double)s.a3 * 0x1p96, 0.0}, DD{(double)s.a2 * 0x1p64, 0.0});
    v = dd_add(v, DD{(double)s.a1 * 0x1p32, 0.0});
    v = dd_add(v, DD{(double)s.a0, 0.0});
    // unit of the accumulator: 2^(2 Emax - 2138), Emax >= 16
    const int k = 2 * (int)(s.e20 >> 20) - 2138 + extra;
    v = DD{ldexp(v.hi, k), ldexp(v.lo, k)};
  }
  return dd_add(v, DD{s.f, 0.0});
}

}  // namespace sumsq
}  // namespace sp
