// Double-float ("df64") arithmetic on the FP32 pipe: a value is an
// unevaluated sum hi + lo of two floats (about 48 significant bits). On
// GB300 the FP32 pipe retires 64 times more operations per clock than the
// FP64 pipe, so one-SM dense work (projected eigenproblems, factorisations)
// runs several times faster in df64 than in FP64 at about 1e-14 relative
// accuracy. Shared by k_dense.cu and k_heig_large.cu.
#pragma once
#include <cuda_runtime.h>

namespace ncgm {
namespace {

struct dfl {
  float hi, lo;
};
struct dfc {
  dfl re, im;
};
// The operations of the error-free transformations use the _rn intrinsics,
// which the compiler never contracts into FMAs (a contracted p + e in the
// product, for instance, loses the low part: 1e-9 instead of 1e-13).
__device__ __forceinline__ dfl dfAdd(dfl a, dfl b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float v = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  const float h = __fadd_rn(s, e);
  return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ dfl dfNeg(dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfl dfMul(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float h = __fadd_rn(p, e);
  return {h, __fsub_rn(e, __fsub_rn(h, p))};
}
__device__ __forceinline__ dfl dfFrom(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(__dsub_rn(x, (double)h))};
}
__device__ __forceinline__ double dfTo(dfl a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfl dfSub(dfl a, dfl b) { return dfAdd(a, dfNeg(b)); }
// a / b: the FP32 quotient of the leading parts, then one correction from
// the double-float residual a - b q1 (long division in base 2^24); about
// 44 correct bits
__device__ __forceinline__ dfl dfDiv(dfl a, dfl b) {
  const float r = __frcp_rn(b.hi);
  const float q1 = __fmul_rn(a.hi, r);
  // p = b q1 exactly as a double-float, then the residual
  const float ph = __fmul_rn(b.hi, q1);
  float pl = fmaf(b.hi, q1, -ph);
  pl = fmaf(b.lo, q1, pl);
  const dfl rem = dfAdd(a, dfNeg(dfl{ph, pl}));
  const float q2 = __fmul_rn(rem.hi, r);
  const float h = __fadd_rn(q1, q2);
  return {h, __fsub_rn(q2, __fsub_rn(h, q1))};
}
// sqrt(a) for a >= 0: the FP32 root of the leading part, one Newton
// correction in double-float
__device__ __forceinline__ dfl dfSqrt(dfl a) {
  if (a.hi <= 0.f) return {0.f, 0.f};
  const float s = sqrtf(a.hi);
  const float sh = __fmul_rn(s, s);
  float sl = fmaf(s, s, -sh);
  const dfl rem = dfAdd(a, dfNeg(dfl{sh, sl}));
  const float c = __fmul_rn(rem.hi, __frcp_rn(2.f * s));
  const float h = __fadd_rn(s, c);
  return {h, __fsub_rn(c, __fsub_rn(h, s))};
}
__device__ __forceinline__ dfc dfcFrom(double2 v) {
  return {dfFrom(v.x), dfFrom(v.y)};
}
__device__ __forceinline__ double2 dfcTo(dfc a) {
  return make_double2(dfTo(a.re), dfTo(a.im));
}
// a * conj(b)
__device__ __forceinline__ dfc dfcMulConj(dfc a, dfc b) {
  return {dfAdd(dfMul(a.re, b.re), dfMul(a.im, b.im)),
          dfSub(dfMul(a.im, b.re), dfMul(a.re, b.im))};
}
// conj(a) * b
__device__ __forceinline__ dfc dfcConjMul(dfc a, dfc b) {
  return {dfAdd(dfMul(a.re, b.re), dfMul(a.im, b.im)),
          dfSub(dfMul(a.re, b.im), dfMul(a.im, b.re))};
}
__device__ __forceinline__ dfc dfcMul(dfc a, dfc b) {
  return {dfSub(dfMul(a.re, b.re), dfMul(a.im, b.im)),
          dfAdd(dfMul(a.re, b.im), dfMul(a.im, b.re))};
}
__device__ __forceinline__ dfc dfcAdd(dfc a, dfc b) {
  return {dfAdd(a.re, b.re), dfAdd(a.im, b.im)};
}
__device__ __forceinline__ dfc dfcSub(dfc a, dfc b) {
  return {dfSub(a.re, b.re), dfSub(a.im, b.im)};
}

} // namespace
} // namespace ncgm
