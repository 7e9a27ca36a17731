// sipg_df.cuh -- compensated ("double-float") arithmetic on the FP32 pipes.
//
// A value is an unevaluated sum hi + lo of two floats.  Products of a float
// input with a table coefficient (itself split into hi + lo) are formed with
// the error-free transformation p + e = fl(a*x) + fma(a, x, -fl(a*x))
// (Dekker 1971, via FMA), and sums with Knuth's TwoSum, so a sum of many
// terms carries the rounding error of its large terms exactly in `lo`.  The
// relative error of a result is then about eps_32^2 times the size of the
// terms, instead of eps_32: sums with heavy cancellation -- the SIPG operator
// applied to a smooth vector loses about log10(condition number) digits --
// keep ~13 correct digits while running at FP32 throughput, which on GB300 is
// ~50x the FP64 rate.  Every operation is an explicit __f*_rn intrinsic so
// that no contraction or reassociation can break the transformations.
#pragma once

#include <cuda_runtime.h>

namespace sipg {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_zero() { return df{0.f, 0.f}; }

// s + e = a + b exactly (Knuth TwoSum, 6 flops)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// acc + (ah + al) * x, x a float
__device__ __forceinline__ df df_mac(df acc, float ah, float al, float x) {
  const float p = __fmul_rn(ah, x);
  const float e = __fmaf_rn(ah, x, -p);  // exact: ah*x = p + e
  float s, err;
  two_sum(acc.hi, p, s, err);
  return df{s, __fadd_rn(acc.lo, __fadd_rn(err, __fmaf_rn(al, x, e)))};
}

// acc + c * x with c = (ch, cl) a coefficient and x = (xh, xl) a df value
__device__ __forceinline__ df df_mac2(df acc, float ch, float cl, df x) {
  const float p = __fmul_rn(ch, x.hi);
  const float e = __fmaf_rn(ch, x.hi, -p);
  float s, err;
  two_sum(acc.hi, p, s, err);
  const float small = __fmaf_rn(ch, x.lo, __fmaf_rn(cl, x.hi, e));
  return df{s, __fadd_rn(acc.lo, __fadd_rn(err, small))};
}

// A table coefficient as three floats, c = h + m + l (about 72 bits): with
// two, the coefficients of the operator itself would be off by 2^-48
// relative -- a fixed perturbation whose effect on smooth vectors does not
// average out and which a CG therefore cannot iterate past.
struct cf {
  float h, m, l;
};

// acc + c * x, c a three-float coefficient, x a df value; the terms below
// 2^-48 |c x| that remain are rounding, not a perturbation of c
__device__ __forceinline__ df df_macc(df acc, cf c, df x) {
  const float p = __fmul_rn(c.h, x.hi);
  const float e = __fmaf_rn(c.h, x.hi, -p);
  float s, err;
  two_sum(acc.hi, p, s, err);
  // the small terms gathered on their own, then added to acc.lo once: folding
  // acc.lo into the FMA chain first saves an operation but rounds each small
  // term at the running sum's scale, four times per call -- in this
  // operator's cancelling sums enough noise to take the mixed solve at 512^2,
  // p = 6 from 560 to 1398 inner iterations (measured)
  float t = __fmul_rn(c.l, x.hi);
  t = __fmaf_rn(c.m, x.lo, t);
  t = __fmaf_rn(c.m, x.hi, t);
  t = __fmaf_rn(c.h, x.lo, t);
  return df{s, __fadd_rn(acc.lo, __fadd_rn(err, __fadd_rn(e, t)))};
}

__device__ __forceinline__ df df_mulc(cf c, df x) { return df_macc(df{0.f, 0.f}, c, x); }

__device__ __forceinline__ df df_add(df a, df b) {
  float s, err;
  two_sum(a.hi, b.hi, s, err);
  return df{s, __fadd_rn(__fadd_rn(a.lo, b.lo), err)};
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }

// c * x with c = (ch, cl), x a df value
__device__ __forceinline__ df df_mul(float ch, float cl, df x) { return df_mac2(df_zero(), ch, cl, x); }

// exact a - b of two floats
__device__ __forceinline__ df df_sub_ff(float a, float b) {
  float s, e;
  two_sum(a, -b, s, e);
  return df{s, e};
}

__device__ __forceinline__ float df_round(df a) { return __fadd_rn(a.hi, a.lo); }

// a float, exactly, into the df sum: acc + x
__device__ __forceinline__ df df_add_f(df acc, float x) {
  float s, err;
  two_sum(acc.hi, x, s, err);
  return df{s, __fadd_rn(acc.lo, err)};
}

}  // namespace sipg
