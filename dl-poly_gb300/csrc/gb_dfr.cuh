// gb_dfr.cuh - a double-float real type with arithmetic operators, so that code written
// once for a floating type T (the SPME splines, spreading, FFT passes and gather) can be
// instantiated in double-float: FP64-level accuracy on the FP32 pipes.  Built on the
// error-free transformations of gb_df64.cuh.
#ifndef GB_DFR_CUH
#define GB_DFR_CUH

#include "gb_df64.cuh"

struct dfr {
  float hi, lo;
  __host__ __device__ constexpr dfr() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr dfr(float h, float l) : hi(h), lo(l) {}
  // exact for |v| < 2^24
  __host__ __device__ constexpr dfr(int v) : hi((float)v), lo(0.f) {}
  // from a double: folds to constants for literals; at run time FP64 conversions
  __host__ __device__ dfr(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dfr to_dfr(df a) { return dfr(a.hi, a.lo); }
__device__ __forceinline__ df to_df(dfr a) { return df_make(a.hi, a.lo); }

__device__ __forceinline__ dfr operator+(dfr a, dfr b) { return to_dfr(df_add(to_df(a), to_df(b))); }
__device__ __forceinline__ dfr operator-(dfr a) { return dfr(-a.hi, -a.lo); }
__device__ __forceinline__ dfr operator-(dfr a, dfr b) { return to_dfr(df_add(to_df(a), df_make(-b.hi, -b.lo))); }
__device__ __forceinline__ dfr operator*(dfr a, dfr b) { return to_dfr(df_mul(to_df(a), to_df(b))); }
__device__ __forceinline__ dfr& operator+=(dfr& a, dfr b) { a = a + b; return a; }
__device__ __forceinline__ dfr& operator-=(dfr& a, dfr b) { a = a - b; return a; }
__device__ __forceinline__ dfr& operator*=(dfr& a, dfr b) { a = a * b; return a; }

// a / b: FP32 quotient, then one correction from the double-float remainder
__device__ __forceinline__ dfr operator/(dfr a, dfr b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df r = df_add(to_df(a), df_neg(df_mul_f(to_df(b), q1)));
  const float q2 = __fdiv_rn(r.hi, b.hi);
  return to_dfr(quick_two_sum(q1, q2));
}

// a * b + c
__device__ __forceinline__ dfr fma(dfr a, dfr b, dfr c) { return to_dfr(df_fma(to_df(a), to_df(b), to_df(c))); }

__device__ __forceinline__ bool nonzero_bits(dfr v) { return (__float_as_uint(v.hi) << 1) != 0u; }

struct dfc {
  dfr x, y;
};

__device__ __forceinline__ dfr shfl_xor_dfr(dfr v, int o) {
  return dfr(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}

// block sums of double-float values: reduced in double-float (no FP64 instruction per
// thread), one thread converts the NV block totals to FP64
template <int NV>
__device__ __forceinline__ void block_reduce_store(dfr (&v)[NV], double* out) {
  __shared__ dfr redd[32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += shfl_xor_dfr(v[k], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) redd[wid][k] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      dfr t = lane < nw ? redd[lane][k] : dfr();
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += shfl_xor_dfr(t, o);
      if (lane == 0) out[(size_t)blockIdx.x * NV + k] = (double)t;
    }
  }
}

#endif
