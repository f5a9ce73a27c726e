// Double-float ("df64") arithmetic on the FP32 pipe: a value is an
// unevaluated sum hi + lo of two floats (about 48 significant bits).
//
// GB300 runs FP32 FMA ~60x faster than FP64 FMA (73 vs 1.2 TFLOP/s measured),
// so the FP64-accuracy products of the eigenpair refinement are evaluated in
// this arithmetic: error-free transformations TwoSum (Knuth, TAOCP vol. 2,
// 4.2.2) and TwoProduct via FMA, with the accurate (renormalising) addition
// of the double-double literature (e.g. Hida, Li, Bailey, "Algorithms for
// quad-double precision floating point arithmetic", ARITH 2001, restricted
// to two components). Relative error per operation is below ~2^-47.
#pragma once
#include "gla_common.cuh"

namespace gla {

struct df64 {
  float hi, lo;
};

GLA_DEV df64 df_make(float h, float l) {
  df64 r;
  r.hi = h;
  r.lo = l;
  return r;
}

// Exact: a + b = s + e.
GLA_DEV void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Exact when |a| >= |b| (or a == 0): a + b = s + e.
GLA_DEV void quick_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}

GLA_DEV df64 df_add(df64 a, df64 b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  df64 r;
  quick_two_sum(s, e, r.hi, r.lo);
  return r;
}

GLA_DEV df64 df_neg(df64 a) { return df_make(-a.hi, -a.lo); }

// acc + a * b (a, b double-float).
GLA_DEV df64 df_mac(df64 acc, df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float pe = fmaf(a.hi, b.hi, -p);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  float s, e;
  two_sum(acc.hi, p, s, e);
  e += pe + acc.lo;
  df64 r;
  quick_two_sum(s, e, r.hi, r.lo);
  return r;
}

// acc + a * b (b a plain float).
GLA_DEV df64 df_mac(df64 acc, df64 a, float b) {
  const float p = a.hi * b;
  float pe = fmaf(a.hi, b, -p);
  pe = fmaf(a.lo, b, pe);
  float s, e;
  two_sum(acc.hi, p, s, e);
  e += pe + acc.lo;
  df64 r;
  quick_two_sum(s, e, r.hi, r.lo);
  return r;
}

GLA_DEV df64 df_mul(df64 a, df64 b) { return df_mac(df_make(0.f, 0.f), a, b); }

// Conversions (FP64 instructions: use outside inner loops only).
GLA_DEV df64 df_from(double x) {
  const float h = (float)x;
  return df_make(h, (float)(x - (double)h));
}
GLA_DEV double df_to(df64 a) { return (double)a.hi + (double)a.lo; }

}  // namespace gla
