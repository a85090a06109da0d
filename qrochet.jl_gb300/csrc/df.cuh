// Double-float (FP32 pair) arithmetic shared by the Jacobi polish and the double-float GEMM.
// A value x is held as hi + lo (two FP32 numbers, ~48 significant bits).  The error-free
// transformations are the published ones: Knuth's TwoSum, Dekker's FastTwoSum and the FMA form of
// TwoProd (as in Hida, Li & Bailey's double-double library), so every operation runs on the FP32
// pipes, which are ~70x faster than the FP64 pipes on this part.
//
// The transformations are exact only if every rounding happens where it is written: the plain
// additions and the product whose error an FMA recovers use the __fadd_rn / __fsub_rn /
// __fmul_rn intrinsics, which the compiler never contracts into a fused multiply-add.
#pragma once
#include <cuda_runtime.h>

namespace qr {

struct dfl {
  float h, l;
};

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  const dfl s = df_two_sum(a.h, b.h);
  return df_fast_two_sum(s.h, __fadd_rn(__fadd_rn(s.l, a.l), b.l));
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dfl df_from(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}

// x + f for a double-float x and an FP32 f (TwoSum on the high parts)
__device__ __forceinline__ dfl df_add_f(dfl x, float f) {
  const dfl s = df_two_sum(x.h, f);
  return df_fast_two_sum(s.h, __fadd_rn(s.l, x.l));
}

// Compensated (Dot2-style) accumulation of sum x y for double-float x, y.  The accumulator keeps
// a running FP32 value s and a correction lo: the hi x hi product is split exactly (p + e, FMA
// TwoProd), p enters s through Knuth's TwoSum, and e, the TwoSum error and the hi x lo cross
// products go into lo.  Error ~2^-48 of sum |x||y| (Ogita, Rump & Oishi, 2005).
struct DotAcc {
  float s, lo;
};
__device__ __forceinline__ void dot2_step(DotAcc& acc, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float e = fmaf(xh, yh, -p);
  const float t = __fadd_rn(acc.s, p);
  const float bv = __fsub_rn(t, acc.s);
  const float err = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, bv)), __fsub_rn(p, bv));
  acc.s = t;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(err, e));
  acc.lo = fmaf(xh, yl, acc.lo);
  acc.lo = fmaf(xl, yh, acc.lo);
}
__device__ __forceinline__ dfl dot_final(DotAcc a) { return df_fast_two_sum(a.s, a.lo); }

}  // namespace qr
