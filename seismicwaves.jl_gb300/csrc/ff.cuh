// Double-FP32 ("compensated") arithmetic shared by the compensated forward
// steps of the acoustic and variable-density paths: a value is the
// unevaluated sum hi + lo of two FP32 numbers.  Error-free transformations:
// Knuth's TwoSum, Dekker's Fast2Sum and the FMA form of Dekker's TwoProduct
// (a*b - fl(a*b) = fma(a, b, -fl(a*b))), combined as in the double-double
// arithmetic of Dekker (1971) and of the QD library of Hida, Li and Bailey;
// about 48 bits of significand.  Every operation uses the round-to-nearest
// intrinsics so that no compiler contraction changes the roundings.
#pragma once

namespace swgb {

struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
// The QD library's "sloppy" addition: one TwoSum of the high parts, the low
// parts added in FP32, one Fast2Sum; its error is a few units of 2^-46
// relative to |a| + |b|, far below the FP32 roundings this arithmetic removes.
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  return fast_two_sum(p, e);
}
__device__ __forceinline__ float ff_round(ff a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ double ff_to_d(ff a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ ff d_to_ff(double v) {
  const float hi = (float)v;
  return ff{hi, (float)(v - (double)hi)};
}

}  // namespace swgb
