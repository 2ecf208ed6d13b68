// gb_fft.cuh - the SPME grid transform shared by gb_spme.cu and the
// constant-length instantiations (gb_fft_f32.cu, gb_fft_df.cu).
//
// An in-shared-memory Stockham FFT (radix 4, 3, 5, 2; the lengths
// 2^a 3^b 5^c that parallel_fft.F90:2031-2055 accepts) along x, y and z of the
// charge grid.  The x pass is real-to-complex; the z pass applies the
// influence function and accumulates the reciprocal stress
// (spme_construct_potential_grid_coul, ewald_spole.F90:1257-1386) between the
// forward and inverse z transforms.  Every kernel exists for any length
// (NC = 0, radices read from an FftPlan) and, for the lengths listed in the
// instantiating files, with the length NC fixed at compile time, so that every
// index division is by a constant and the radix loops unroll.
#pragma once
#include <type_traits>

#include "gb_common.cuh"
#include "gb_dfr.cuh"

namespace gbspme {

constexpr int TX = 4;  // columns per tile in the strided passes

struct FftPlan {
  int N;
  int nrad;
  int rad[16];
};

struct SpmeGeom {
  double rc[9];
  float rch[9], rcl[9];  // rc as double-floats
  double Kr[3];
  int K[3], B[3], nb[3], p;
};

// the five FFT kernels one grid launches, for working type T (complex T2)
template <typename T, typename T2>
struct FftKernels {
  void (*x_fwd)(const T*, T2*, FftPlan, const T2*, const T2*, int, int);
  void (*x_inv)(const T2*, T*, FftPlan, const T2*, const T2*, int, int);
  void (*y_fwd)(T2*, int, int, FftPlan, const T2*);
  void (*y_inv)(T2*, int, int, FftPlan, const T2*);
  void (*z_conv)(T2*, int, int, int, FftPlan, const T2*, const T*, const T*, SpmeGeom, double*);
};

// kernels for an x pass of half length M and y, z passes of lengths K2, K3:
// the constant-length instances where they were compiled, else the runtime-plan ones
template <typename T, typename T2>
FftKernels<T, T2> fft_kernels(int M, int K2, int K3);
template <>
FftKernels<double, double2> fft_kernels<double, double2>(int M, int K2, int K3);  // gb_spme.cu
template <>
FftKernels<float, float2> fft_kernels<float, float2>(int M, int K2, int K3);  // gb_fft_f32.cu
template <>
FftKernels<dfr, dfc> fft_kernels<dfr, dfc>(int M, int K2, int K3);  // gb_fft_df.cu

}  // namespace gbspme

namespace {

using namespace gbspme;

template <typename T> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };
template <> struct V2<dfr> { using t = dfc; };

template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// double-float a*b + c*d: both exact products' high parts in one two-sum, their rounding
// errors and cross terms in the correction, one renormalisation (19 FP32 operations
// instead of the 25 of two products and a sum)
__device__ __forceinline__ dfr df_prod_sum(dfr a, dfr b, dfr c, dfr d) {
  const df p = two_prod(a.hi, b.hi), q = two_prod(c.hi, d.hi);
  const float tp = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  const float tq = __fmaf_rn(c.hi, d.lo, __fmaf_rn(c.lo, d.hi, q.lo));
  const df s = two_sum(p.hi, q.hi);
  return to_dfr(quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(tp, tq))));
}
template <> __device__ __forceinline__ dfc cmul<dfc>(dfc a, dfc b) {
  dfc r;
  r.x = df_prod_sum(a.x, b.x, -a.y, b.y);
  r.y = df_prod_sum(a.x, b.y, a.y, b.x);
  return r;
}
// a + b and a - b left unnormalised (the two-sum of the high parts and the sum of the low
// parts): an intermediate of a butterfly, renormalised by the next addition
__device__ __forceinline__ dfr df_add_open(dfr a, dfr b) {
  const df s = two_sum(a.hi, b.hi);
  return dfr(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfc cadd_open(dfc a, dfc b) { dfc r; r.x = df_add_open(a.x, b.x); r.y = df_add_open(a.y, b.y); return r; }
__device__ __forceinline__ dfc csub_open(dfc a, dfc b) { dfc r; r.x = df_add_open(a.x, -b.x); r.y = df_add_open(a.y, -b.y); return r; }
template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { T2 r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { T2 r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// multiply by s*i
// multiply by S*i with S = +1 or -1 known at compile time (a free operand negation)
template <int S, typename T2> __device__ __forceinline__ T2 cmuli(T2 a) {
  T2 r;
  if (S > 0) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; }
  return r;
}

// x != 0 tested on the bit pattern (no FP64 compare instruction)
__device__ __forceinline__ bool nonzero_bits(double v) { return (__double_as_longlong(v) << 1) != 0; }
__device__ __forceinline__ bool nonzero_bits(float v) { return (__float_as_uint(v) << 1) != 0u; }


// radix-R butterfly of one Stockham stage (inputs already twiddled)
template <typename T, typename T2, int ISIGN, int R>
__device__ __forceinline__ void bfly(const T2 (&v)[5], T2 (&o)[5]) {
  if constexpr (R == 4 && std::is_same<T2, dfc>::value) {
    // double-float: the first level's sums stay unnormalised, the outputs are renormalised
    T2 a = cadd_open(v[0], v[2]), b = csub_open(v[0], v[2]), c = cadd_open(v[1], v[3]), d = csub_open(v[1], v[3]);
    T2 di = cmuli<ISIGN>(d);
    o[0] = cadd(a, c); o[2] = csub(a, c); o[1] = cadd(b, di); o[3] = csub(b, di);
  } else if constexpr (R == 4) {
    T2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]), c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
    T2 di = cmuli<ISIGN>(d);
    o[0] = cadd(a, c); o[2] = csub(a, c); o[1] = cadd(b, di); o[3] = csub(b, di);
  } else if constexpr (R == 2) {
    o[0] = cadd(v[0], v[1]); o[1] = csub(v[0], v[1]);
  } else if constexpr (R == 3) {
    const T h = (T)0.86602540378443864676;
    T2 t = cadd(v[1], v[2]), u = csub(v[1], v[2]);
    T2 m;
    m.x = v[0].x - (T)0.5 * t.x; m.y = v[0].y - (T)0.5 * t.y;
    T2 ui = cmuli<ISIGN>(u);
    ui.x *= h; ui.y *= h;
    o[0] = cadd(v[0], t); o[1] = cadd(m, ui); o[2] = csub(m, ui);
  } else {  // R == 5
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
    const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
    T2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]), t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    o[0] = cadd(v[0], cadd(t1, t2));
    T2 a1, a2, b1, b2;
    a1.x = v[0].x + c1 * t1.x + c2 * t2.x; a1.y = v[0].y + c1 * t1.y + c2 * t2.y;
    a2.x = v[0].x + c2 * t1.x + c1 * t2.x; a2.y = v[0].y + c2 * t1.y + c1 * t2.y;
    b1.x = s1 * t3.x + s2 * t4.x; b1.y = s1 * t3.y + s2 * t4.y;
    b2.x = s2 * t3.x - s1 * t4.x; b2.y = s2 * t3.y - s1 * t4.y;
    T2 ib1 = cmuli<ISIGN>(b1), ib2 = cmuli<ISIGN>(b2);
    o[1] = cadd(a1, ib1); o[4] = csub(a1, ib1); o[2] = cadd(a2, ib2); o[3] = csub(a2, ib2);
  }
}

// one Stockham stage over nlines lines of length N held in shared memory.
// The twiddle index r*k*step stays below N (k < Ns, r < R, step = N/(Ns R)).
template <typename T, typename T2, int ISIGN>
__device__ void fft_stage(const T2* __restrict__ in, T2* __restrict__ out, int N, int nlines, int R, int Ns,
                          const T2* __restrict__ tw) {
  const int T_ = N / R;
  const int total = nlines * T_;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int line = idx / T_;
    const int j = idx - line * T_;
    const int k = j % Ns;
    const T2* src = in + line * N;
    T2* dst = out + line * N;
    T2 v[5];
#pragma unroll 5
    for (int r = 0; r < 5; ++r)
      if (r < R) v[r] = src[j + r * T_];
    if (Ns > 1) {
      const int step = N / (Ns * R);
#pragma unroll 5
      for (int r = 1; r < 5; ++r) {
        if (r < R) {
          T2 w = tw[r * k * step];
          if (ISIGN < 0) w.y = -w.y;
          v[r] = cmul(v[r], w);
        }
      }
    }
    T2 o[5];
    if (R == 4) bfly<T, T2, ISIGN, 4>(v, o);
    else if (R == 2) bfly<T, T2, ISIGN, 2>(v, o);
    else if (R == 3) bfly<T, T2, ISIGN, 3>(v, o);
    else bfly<T, T2, ISIGN, 5>(v, o);
    const int base = (j / Ns) * Ns * R + k;
#pragma unroll 5
    for (int r = 0; r < 5; ++r)
      if (r < R) dst[base + r * Ns] = o[r];
  }
}

// full transform of nlines lines; returns the buffer holding the result
template <typename T, typename T2, int ISIGN>
__device__ T2* fft_lines(T2* a, T2* b, const FftPlan& pl, int nlines, const T2* tw) {
  int Ns = 1;
  for (int s = 0; s < pl.nrad; ++s) {
    __syncthreads();
    fft_stage<T, T2, ISIGN>(a, b, pl.N, nlines, pl.rad[s], Ns, tw);
    Ns *= pl.rad[s];
    T2* t = a; a = b; b = t;
  }
  __syncthreads();
  return a;
}

// The same stages with the length known at compile time: every index
// division and remainder is by a constant and the radix loops unroll.  The
// radix order (4s, then 3s, 5s, 2s) is make_plan's, so both forms of the
// transform perform the same arithmetic.
template <int M>
constexpr int next_radix() { return M % 4 == 0 ? 4 : (M % 3 == 0 ? 3 : (M % 5 == 0 ? 5 : 2)); }

template <typename T, typename T2, int ISIGN, int N, int R, int Ns>
__device__ __forceinline__ void fft_stage_ct(const T2* __restrict__ in, T2* __restrict__ out, int nlines,
                                             const T2* __restrict__ tw) {
  constexpr int T_ = N / R;
  constexpr int step = N / (Ns * R);
  const int total = nlines * T_;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int line = idx / T_;
    const int j = idx - line * T_;
    const int k = j % Ns;
    const T2* src = in + line * N;
    T2* dst = out + line * N;
    T2 v[5];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[j + r * T_];
    if constexpr (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        T2 w = tw[r * k * step];
        if (ISIGN < 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    T2 o[5];
    bfly<T, T2, ISIGN, R>(v, o);
    const int base = (j - k) * R + k;  // (j / Ns) Ns R + k
#pragma unroll
    for (int r = 0; r < R; ++r) dst[base + r * Ns] = o[r];
  }
}

template <typename T, typename T2, int ISIGN, int N, int Ns>
__device__ __forceinline__ T2* fft_ct(T2* a, T2* b, int nlines, const T2* tw) {
  if constexpr (Ns == N) {
    __syncthreads();
    return a;
  } else {
    constexpr int R = next_radix<N / Ns>();
    static_assert((N / Ns) % R == 0, "FFT lengths are 2^a 3^b 5^c");
    __syncthreads();
    fft_stage_ct<T, T2, ISIGN, N, R, Ns>(a, b, nlines, tw);
    return fft_ct<T, T2, ISIGN, N, Ns * R>(b, a, nlines, tw);
  }
}

// NC > 0: the compile-time transform of length NC (== pl.N); NC == 0: any length
template <typename T, typename T2, int ISIGN, int NC>
__device__ __forceinline__ T2* fft_run(T2* a, T2* b, const FftPlan& pl, int nlines, const T2* tw) {
  if constexpr (NC == 0) return fft_lines<T, T2, ISIGN>(a, b, pl, nlines, tw);
  else return fft_ct<T, T2, ISIGN, NC, 1>(a, b, nlines, tw);
}


// a reciprocal-cell entry in the working precision (double-floats from the stored split)
template <typename T>
__device__ __forceinline__ T rc_at(const SpmeGeom& sg, int k) { return (T)sg.rc[k]; }
template <>
__device__ __forceinline__ dfr rc_at<dfr>(const SpmeGeom& sg, int k) { return dfr(sg.rch[k], sg.rcl[k]); }

// ---------------------------------------------------------------- FFT passes
// The charge grid is real, so the x pass is a real-to-complex transform: a row
// of N = K1 reals is packed as M = N/2 complex values z_n = x_2n + i x_2n+1,
// transformed with the half-length complex FFT and split into the N/2+1
// non-redundant outputs
//   X_k = E_k + w^k O_k,  E_k = (Z_k + conj Z_{M-k}) / 2,  O_k = (Z_k - conj Z_{M-k}) / 2i,
// w = e^{+2 pi i/N} (the forward sign of the reference's transform).  The y and
// z passes then run on Kx = N/2+1 columns.  The inverse rebuilds
//   Z_k = (X_k + conj X_{M-k}) + i (X_k - conj X_{M-k}) w^{-k},  k < M,
// runs the half-length inverse and unpacks x_2n = Re z_n, x_2n+1 = Im z_n: the
// real part of the full inverse transform, as before.
template <typename T, typename T2, int NC>
__global__ void k_fft_x_fwd(const T* __restrict__ Q, T2* __restrict__ G, FftPlan pl, const T2* __restrict__ tw,
                            const T2* __restrict__ twN, int nrows, int lines) {
  extern __shared__ unsigned char smem_raw[];
  const int M = NC ? NC : pl.N, Kx = M + 1;
  T2* a = reinterpret_cast<T2*>(smem_raw);
  T2* b = a + lines * M;
  const size_t row0 = (size_t)blockIdx.x * lines;
  const int nl = (int)min((size_t)lines, (size_t)nrows - row0);
  const T2* Qc = reinterpret_cast<const T2*>(Q);
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) a[e] = Qc[row0 * M + e];
  T2* r = fft_run<T, T2, +1, NC>(a, b, pl, nl, tw);
  for (int e = threadIdx.x; e < nl * Kx; e += blockDim.x) {
    const int line = e / Kx, k = e - line * Kx;
    const T2 zk = r[line * M + (k == M ? 0 : k)];
    const T2 zc = r[line * M + (k == 0 ? 0 : M - k)];  // Z_{M-k}, conjugated below
    const T ex = (T)0.5 * (zk.x + zc.x), ey = (T)0.5 * (zk.y - zc.y);
    const T ox = (T)0.5 * (zk.y + zc.y), oy = (T)0.5 * (zc.x - zk.x);
    const T2 w = twN[k];
    T2 v;
    v.x = ex + (w.x * ox - w.y * oy);
    v.y = ey + (w.x * oy + w.y * ox);
    G[(row0 + line) * Kx + k] = v;
  }
}

template <typename T, typename T2, int NC>
__global__ void k_fft_x_inv(const T2* __restrict__ G, T* __restrict__ Q, FftPlan pl, const T2* __restrict__ tw,
                            const T2* __restrict__ twN, int nrows, int lines) {
  extern __shared__ unsigned char smem_raw[];
  const int M = NC ? NC : pl.N, Kx = M + 1;
  T2* a = reinterpret_cast<T2*>(smem_raw);
  T2* b = a + lines * M;
  const size_t row0 = (size_t)blockIdx.x * lines;
  const int nl = (int)min((size_t)lines, (size_t)nrows - row0);
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
    const int line = e / M, k = e - line * M;
    const T2 xk = G[(row0 + line) * Kx + k];
    const T2 xc = G[(row0 + line) * Kx + (M - k)];  // X_{M-k}, conjugated below
    const T ax = xk.x + xc.x, ay = xk.y - xc.y;     // X_k + conj X_{M-k}
    const T dx = xk.x - xc.x, dy = xk.y + xc.y;     // X_k - conj X_{M-k}
    const T2 w = twN[k];                            // w^{-k} = conj(w^k)
    const T bx = dx * w.x + dy * w.y, by = dy * w.x - dx * w.y;
    T2 v;
    v.x = ax - by;
    v.y = ay + bx;
    a[e] = v;
  }
  T2* r = fft_run<T, T2, -1, NC>(a, b, pl, nl, tw);
  T2* Qc = reinterpret_cast<T2*>(Q);
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) Qc[row0 * M + e] = r[e];
}

// Y pass (stride Kx): tile of TX columns x N lines, in place
template <typename T, typename T2, int ISIGN, int NC>
__global__ void k_fft_y(T2* __restrict__ G, int Kx, int K2_, FftPlan pl, const T2* __restrict__ tw) {
  extern __shared__ unsigned char smem_raw[];
  const int K2 = NC ? NC : K2_;
  T2* a = reinterpret_cast<T2*>(smem_raw);
  T2* b = a + TX * K2;
  const int ntx = (Kx + TX - 1) / TX;
  const int x0 = (blockIdx.x % ntx) * TX;
  const int zz = blockIdx.x / ntx;
  const int nt = min(TX, Kx - x0);
  T2* base = G + (size_t)zz * Kx * K2 + x0;
  for (int e = threadIdx.x; e < TX * K2; e += blockDim.x) {
    int yy = e / TX, t = e - yy * TX;
    T2 v; v.x = (T)0; v.y = (T)0;
    if (t < nt) v = base[(size_t)yy * Kx + t];
    a[t * K2 + yy] = v;
  }
  T2* r = fft_run<T, T2, ISIGN, NC>(a, b, pl, TX, tw);
  for (int e = threadIdx.x; e < TX * K2; e += blockDim.x) {
    int yy = e / TX, t = e - yy * TX;
    if (t < nt) base[(size_t)yy * Kx + t] = r[t * K2 + yy];
  }
}

// Z pass: forward z FFT, influence function + stress, inverse z FFT on the
// Kx = K1/2+1 columns of the half spectrum; columns 0 < x < K1/2 stand for
// themselves and their conjugate mirror, so they count twice in the stress
template <typename T, typename T2, int NC>
__global__ void k_fft_z_conv(T2* __restrict__ G, int K1, int K2, int K3_, FftPlan pl, const T2* __restrict__ tw,
                             const T* __restrict__ theta, const T* __restrict__ psi, SpmeGeom sg, double* blk) {
  extern __shared__ unsigned char smem_raw[];
  const int K3 = NC ? NC : K3_;
  T2* a = reinterpret_cast<T2*>(smem_raw);
  T2* b = a + TX * K3;
  const int Kx = K1 / 2 + 1;
  const int ntx = (Kx + TX - 1) / TX;
  const int x0 = (blockIdx.x % ntx) * TX;
  const int yy = blockIdx.x / ntx;
  const int nt = min(TX, Kx - x0);
  const size_t plane = (size_t)Kx * K2;
  T2* base = G + (size_t)yy * Kx + x0;
  for (int e = threadIdx.x; e < TX * K3; e += blockDim.x) {
    int zz = e / TX, t = e - zz * TX;
    T2 v; v.x = (T)0; v.y = (T)0;
    if (t < nt) v = base[(size_t)zz * plane + t];
    a[t * K3 + zz] = v;
  }
  // m_z = ll * rcell(9) for the cubic cell (gb_init accepts cubic cells only)
  T* rzt = reinterpret_cast<T*>(b + TX * K3);
  for (int zz = threadIdx.x; zz < K3; zz += blockDim.x) {
    int ll = zz; if (2 * ll > K3) ll -= K3;
    rzt[zz] = (T)ll * rc_at<T>(sg, 8);
  }
  T2* r = fft_run<T, T2, +1, NC>(a, b, pl, TX, tw);
  // Reciprocal stress sum_m m_a m_b psi |Q(m)|^2 (ewald_spole.F90:1362-1371): with
  // m = (mx, my, mz) and mx, my fixed along a z line, each line needs only
  // A = sum psi|Q|^2, B = sum mz psi|Q|^2, C = sum mz^2 psi|Q|^2.
  const int tpl = blockDim.x / TX;          // threads per line
  const int t = threadIdx.x / tpl;          // this thread's line
  // Bn: the z-Nyquist point (mz = +K3/2 for a point and its mirror alike) kept apart
  T A = 0, B = 0, Bn = 0, C = 0;
  if (t < nt) {
    const size_t line0 = (size_t)yy * Kx + x0 + t;
    T2* rl = r + t * K3;
    for (int zz = threadIdx.x - t * tpl; zz < K3; zz += tpl) {
      const size_t gi = line0 * K3 + zz;  // theta/psi are stored z-contiguous per (x,y) line
      const T th = theta[gi];
      T2 v = rl[zz];
      if (nonzero_bits(th)) {
        const T pv = psi[gi] * (v.x * v.x + v.y * v.y);
        const T u = pv * rzt[zz];
        A += pv;
        if (2 * zz == K3) Bn += u;
        else B += u;
        C = fma(u, rzt[zz], C);
        v.x *= th; v.y *= th;
      } else {
        v.x = (T)0; v.y = (T)0;
      }
      rl[zz] = v;
    }
  }
  // in the working precision T: the FP32 form issues no FP64 instruction here
  // A line 0 < jx < K1/2 stands for itself and its mirror m' = -m, except that
  // a Nyquist index (ky = K2/2, mz = K3/2) keeps its + sign in the mirror.
  // The mirror's share of m_a m_b psi|Q|^2 is then +/- the line's own:
  //   xx, yy, zz: +;  xy: - when ky is Nyquist;  xz: - for the Nyquist z point;
  //   yz: - when exactly one of ky and the z point is Nyquist.
  T st[6] = {0, 0, 0, 0, 0, 0};
  if (t < nt) {
    const int jx = x0 + t;
    int jj = jx; if (2 * jj > K1) jj -= K1;
    int kk = yy; if (2 * kk > K2) kk -= K2;
    const T rx = (T)jj * rc_at<T>(sg, 0), ry = (T)kk * rc_at<T>(sg, 4);
    if (jx == 0 || 2 * jx == K1) {  // the line holds its own mirror: the full-spectrum sums
      const T Ball = B + Bn;
      st[0] = rx * rx * A; st[1] = rx * ry * A; st[2] = rx * Ball;
      st[3] = ry * ry * A; st[4] = ry * Ball; st[5] = C;
    } else {
      const bool ny = 2 * yy == K2;
      st[0] = (T)2 * rx * rx * A;
      st[1] = ny ? (T)0 : (T)2 * rx * ry * A;
      st[2] = (T)2 * rx * B;
      st[3] = (T)2 * ry * ry * A;
      st[4] = (T)2 * ry * (ny ? Bn : B);
      st[5] = (T)2 * C;
    }
  }
  T2* o = (r == a) ? b : a;
  T2* r2 = fft_run<T, T2, -1, NC>(r, o, pl, TX, tw);
  for (int e = threadIdx.x; e < TX * K3; e += blockDim.x) {
    int zz = e / TX, t = e - zz * TX;
    if (t < nt) base[(size_t)zz * plane + t] = r2[t * K3 + zz];
  }
  block_reduce_store<6>(st, blk);
}


template <int... L>
struct FftLens {};

template <typename T, typename T2, int L>
void fft_take_x(FftKernels<T, T2>& k, int M) {
  if (M == L) {
    k.x_fwd = &k_fft_x_fwd<T, T2, L>;
    k.x_inv = &k_fft_x_inv<T, T2, L>;
  }
}

template <typename T, typename T2, int L>
void fft_take_yz(FftKernels<T, T2>& k, int K2, int K3) {
  if (K2 == L) {
    k.y_fwd = &k_fft_y<T, T2, +1, L>;
    k.y_inv = &k_fft_y<T, T2, -1, L>;
  }
  if (K3 == L) k.z_conv = &k_fft_z_conv<T, T2, L>;
}

// runtime-plan kernels, replaced pass by pass by the instances of lengths XL
// (x passes) and YL (y and z passes) that match
template <typename T, typename T2, int... XL, int... YL>
FftKernels<T, T2> fft_pick(FftLens<XL...>, FftLens<YL...>, int M, int K2, int K3) {
  FftKernels<T, T2> k{&k_fft_x_fwd<T, T2, 0>, &k_fft_x_inv<T, T2, 0>, &k_fft_y<T, T2, +1, 0>, &k_fft_y<T, T2, -1, 0>,
                      &k_fft_z_conv<T, T2, 0>};
  (fft_take_x<T, T2, XL>(k, M), ...);
  (fft_take_yz<T, T2, YL>(k, K2, K3), ...);
  return k;
}

}  // namespace
