// Arithmetic on (hi, lo) float pairs ("double-float") for the reduced-FP64 step forms: error-free
// products (TwoProduct with an FMA, Dekker / Ogita-Rump-Oishi) and sums (TwoSum, Knuth), exact up to
// ~2^-47 of the operands' magnitude, and the LLG right-hand side on pairs.  Explicit _rn intrinsics
// keep the compiler from contracting or reassociating the compensation steps.
#pragma once

#include "mgx_internal.cuh"

namespace mgx {

__device__ __forceinline__ float2 split_double(double x) {
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - (double)hi);
  return make_float2(hi, lo);
}

// value h + l
struct dfp {
  float h, l;
};

__device__ __forceinline__ dfp dfp_of(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ dfp dfp_neg(dfp a) { return {-a.h, -a.l}; }

// a * b: exact product of the high parts plus the cross terms (|l| ~ 2^-23 |h|, not renormalised)
__device__ __forceinline__ dfp dfp_mul(dfp a, dfp b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  return {p, e};
}

// a + b, renormalised so that |l| <= ulp(h) / 2
__device__ __forceinline__ dfp dfp_add(dfp a, dfp b) {
  const float s = __fadd_rn(a.h, b.h);
  const float bp = __fsub_rn(s, a.h);
  const float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bp)), __fsub_rn(b.h, bp));
  const float t = __fadd_rn(__fadd_rn(a.l, b.l), err);
  const float r = __fadd_rn(s, t);
  const float rp = __fsub_rn(r, s);
  return {r, __fadd_rn(__fsub_rn(s, __fsub_rn(r, rp)), __fsub_rn(t, rp))};
}

__device__ __forceinline__ double dfp_double(dfp a) { return (double)a.h + (double)a.l; }

// f = pre [e x B + alpha e x (e x B)] (magex/llg.py:21-28) on pairs
__device__ __forceinline__ void dfp_rhs(const dfp e[3], const dfp B[3], dfp a, dfp pre, bool precession, dfp f[3]) {
  dfp c[3], d[3];
  c[0] = dfp_add(dfp_mul(e[1], B[2]), dfp_neg(dfp_mul(e[2], B[1])));
  c[1] = dfp_add(dfp_mul(e[2], B[0]), dfp_neg(dfp_mul(e[0], B[2])));
  c[2] = dfp_add(dfp_mul(e[0], B[1]), dfp_neg(dfp_mul(e[1], B[0])));
  d[0] = dfp_add(dfp_mul(e[1], c[2]), dfp_neg(dfp_mul(e[2], c[1])));
  d[1] = dfp_add(dfp_mul(e[2], c[0]), dfp_neg(dfp_mul(e[0], c[2])));
  d[2] = dfp_add(dfp_mul(e[0], c[1]), dfp_neg(dfp_mul(e[1], c[0])));
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const dfp ad = dfp_mul(a, d[k]);
    f[k] = dfp_mul(pre, precession ? dfp_add(c[k], ad) : dfp_add(ad, {0.f, 0.f}));
  }
}

}  // namespace mgx
