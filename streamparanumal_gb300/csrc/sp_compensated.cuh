// Compensated FP32 accumulation shared by the FP32-storage reductions.
#pragma once

namespace sp {

// Error-free transformation a + b = s + e (Knuth TwoSum), FP32.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Compensated FP32 accumulation of a product (Ogita-Rump-Oishi Dot2 step).
__device__ __forceinline__ void dot2_step(float a, float b, float& s, float& c) {
  const float p = a * b;
  const float pe = fmaf(a, b, -p);
  float t, e;
  two_sum(s, p, t, e);
  s = t;
  c += e + pe;
}

}  // namespace sp
