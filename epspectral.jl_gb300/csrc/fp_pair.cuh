// fp_pair.cuh -- FP64 values carried as float pairs on the tensor-core path, for kernels that must
// form a cancelling difference exactly but otherwise run on the FP32 units.
#pragma once
#include <cuda_runtime.h>

namespace epsp {

// x = hi + lo with hi = float(x) (to ~2^-48 relative).
__device__ __forceinline__ float2 split_df(double x) {
  const float h = float(x);
  return make_float2(h, float(x - double(h)));
}

// s + e = a + b exactly (Knuth's two-sum; additions only, so no contraction into FMA applies).
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}

// (x - e) - Re Σ(x) with Re Σ(x) = lo + t (hi - lo), x, e and the Re Σ nodes as float pairs (lo, hi
// carry theirs in .x/.y): the cancelling part x - e - lo is formed exactly (two two-sums on the
// high words, the low words added after), the interpolation step t (hi - lo) in FP32.
__device__ __forceinline__ float re_z(float2 x, float2 e, float4 lo, float4 hi, float t) {
  float e1, e2;
  const float s1 = two_sum(x.x, -e.x, e1);
  const float s2 = two_sum(s1, -lo.x, e2);
  const float r = s2 + (e1 + e2 + ((x.y - e.y) - lo.y));
  const float d = (hi.x - lo.x) + (hi.y - lo.y);
  return r - t * d;
}

// Im(1/(c + i d)) by Smith's algorithm in FP32.
__device__ __forceinline__ float imag_inv_f(float c, float d) {
  if (fabsf(d) <= fabsf(c)) {
    const float r = d / c;
    return -r * (1.f / (c + d * r));
  }
  const float r = c / d;
  return -(1.f / (d + c * r));
}

}  // namespace epsp
