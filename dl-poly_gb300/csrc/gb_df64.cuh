// gb_df64.cuh - double-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi)/2), about 48 significant bits.  On GB300 the FP64
// pipe runs at 1/64 of the FP32 rate, so kernels that need FP64-level accuracy but
// not FP64 range evaluate their inner loops in this form on the FP32 pipes.
//
// The operations are the error-free transformations of the double-double literature
// (Knuth's two-sum, the FMA two-product; see Hida, Li and Bailey, "Library for
// double-double and quad-double arithmetic", 2007), written with the _rn intrinsics
// so the compiler cannot contract or reassociate them.
#ifndef GB_DF64_CUH
#define GB_DF64_CUH

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float hi, float lo) {
  df r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// s + e = a + b exactly
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df_make(s, e);
}

// the same for |a| >= |b|
__device__ __forceinline__ df quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// p + e = a * b exactly
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df_make(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ df df_add(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ df df_add_f(df a, float b) {
  const df s = two_sum(a.hi, b);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ __forceinline__ df df_neg(df a) { return df_make(-a.hi, -a.lo); }

__device__ __forceinline__ df df_mul(df a, df b) {
  const df p = two_prod(a.hi, b.hi);
  return quick_two_sum(p.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo)));
}

__device__ __forceinline__ df df_mul_f(df a, float b) {
  const df p = two_prod(a.hi, b);
  return quick_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

// a * b + c: the product's rounding error and cross terms join c's low part without
// first renormalising the product (14 FP32 operations instead of 18)
__device__ __forceinline__ df df_fma(df a, df b, df c) {
  const df p = two_prod(a.hi, b.hi);
  const float t = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  const df s = two_sum(p.hi, c.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(t, c.lo)));
}

__device__ __forceinline__ df df_sqr(df a) {
  const df p = two_prod(a.hi, a.hi);
  return quick_two_sum(p.hi, __fmaf_rn(__fmul_rn(2.0f, a.hi), a.lo, p.lo));
}

// 1/sqrt(a) for a > 0: FP32 seed and one Newton step whose residual 1 - a r^2 is formed
// in double-float (relative error about 4e-14)
__device__ __forceinline__ df df_rsqrt(df a) {
  const float r = rsqrtf(a.hi);
  const df ar2 = df_mul(a, two_prod(r, r));
  const float h = __fsub_rn(__fsub_rn(1.0f, ar2.hi), ar2.lo);
  return quick_two_sum(r, __fmul_rn(__fmul_rn(0.5f, r), h));
}

__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

__host__ __device__ inline void df_split(double v, float* hi, float* lo) {
  *hi = (float)v;
  *lo = (float)(v - (double)*hi);
}

// x^2 + y^2 + z^2: the squares' exact high parts summed by two two-sums, their rounding
// errors, cross terms and the sums' errors in one correction, renormalised once (31 FP32
// operations instead of the 40 of three squares and two additions)
__device__ __forceinline__ df df_norm2(df x, df y, df z) {
  const df px = two_prod(x.hi, x.hi), py = two_prod(y.hi, y.hi), pz = two_prod(z.hi, z.hi);
  const float cx = __fmaf_rn(__fadd_rn(x.hi, x.hi), x.lo, px.lo);
  const float cy = __fmaf_rn(__fadd_rn(y.hi, y.hi), y.lo, py.lo);
  const float cz = __fmaf_rn(__fadd_rn(z.hi, z.hi), z.lo, pz.lo);
  const df s1 = two_sum(px.hi, py.hi);
  const df s2 = two_sum(s1.hi, pz.hi);
  const float c = __fadd_rn(__fadd_rn(__fadd_rn(cx, cy), __fadd_rn(cz, s1.lo)), s2.lo);
  return quick_two_sum(s2.hi, c);
}

// running sum of many double-float terms: s carries the sum, c its rounding errors
struct dacc {
  float s, c;
};

__device__ __forceinline__ void dacc_add(dacc& a, df t) {
  const df u = two_sum(a.s, t.hi);
  a.s = u.hi;
  a.c = __fadd_rn(a.c, __fadd_rn(u.lo, t.lo));
}

__device__ __forceinline__ double dacc_value(const dacc& a) { return (double)a.s + (double)a.c; }

// a += x * y: the exact product's high part enters the compensated sum, its error term
// and the cross terms go straight to the correction (no renormalised product)
__device__ __forceinline__ void dacc_add_prod(dacc& a, df x, df y) {
  const df p = two_prod(x.hi, y.hi);
  const float t = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo));
  const df u = two_sum(a.s, p.hi);
  a.s = u.hi;
  a.c = __fadd_rn(a.c, __fadd_rn(u.lo, t));
}

// int64 fixed point (scale 2^40) of a double-float, each part rounded toward zero: the
// scaling by 2^40 is exact, and for |a| < 2^23 the hardware conversion gives what fix40
// gives.  The conversion runs on the FP64 unit, which the double-float kernels leave
// idle; they are bound by instruction issue, so two conversions beat the thirty-odd
// integer operations of fix40 there.
__device__ __forceinline__ long long fix40_df(df a) {
  return __float2ll_rz(__fmul_rn(a.hi, 1099511627776.0f)) + __float2ll_rz(__fmul_rn(a.lo, 1099511627776.0f));
}

// fix40 of the product a * b without renormalising it: the exact product's high part and
// the sum of its rounding error and cross terms, each scaled by 2^40 and truncated toward
// zero (the parts fix40_df truncates, up to where the renormalisation would split them)
__device__ __forceinline__ long long fix40_prod(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float t = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p)));
  return __float2ll_rz(__fmul_rn(p, 1099511627776.0f)) + __float2ll_rz(__fmul_rn(t, 1099511627776.0f));
}

#endif
