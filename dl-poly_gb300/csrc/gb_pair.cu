// gb_pair.cu - real-space vdW + erfc-damped Coulomb pair forces.
//
// Follows the pair loop of two_body_forces (source/two_body.F90:339-606):
//   vdw_forces_tab        source/vdw.F90:1790-2024 (default, 3-point tables)
//   vdw_forces_direct     source/vdw.F90:1578-1788 (analytic 12-6 LJ)
//   ewald_real_forces_coul source/ewald_spole.F90:58-242 (tabulated erfc(ar)/r)
//   ewald_excl_forces     source/ewald_spole.F90:479-679 (direct A&S erfc)
// The 3-point interpolation of three_p_interp (numerics.F90:250-290) is the
// quadratic through table points k, k+1, k+2; it is evaluated here from its
// per-interval coefficients c0 + d*(c1 + d*c2), precomputed in FP64 from the
// same table values (identical polynomial, rounding differs by ~1e-16).
//
// FP64 form: one warp per local atom walks the reference half list.  Pairs
// with a halo image j are evaluated once, by the atom with the smaller global
// id, and applied to both atoms (the reference evaluates such a pair from both
// sides, each side keeping only its own force; the sum is the same).
// Mixed form: one warp per atom walks the same half list in FP32 and sums the
// pair forces as int64 fixed point (scale 2^40), the reaction on j with 64-bit
// integer atomics: order independent and bit-reproducible.
#include <cfloat>
#include <cmath>
#include <cstring>

#include "gb_common.cuh"
#include "gb_df64.cuh"
#include "gb_dfr.cuh"

namespace {

struct PairGeom {
  double rc2, rv2;           // cutoffs squared
  double rc2_lo, rc2_hi;     // band where sqrt(rsq) < rc is decided exactly
  double rv2_lo, rv2_hi;
  long long b_rc2_lo, b_rc2_hi, b_rv2_lo, b_rv2_hi, b_hi;  // the same bounds as IEEE bit patterns
  double rcut, rvdw;
  double erdr, vrdr;         // reciprocal table spacings
  double scaling;            // r4pie0 / eps
  int vdw_direct;
  int same_grid;             // erdr == vrdr: one table coordinate serves both tables
  int nsamples, max_grid, ntypes;
  // double-float kernel: cutoff bands on the FP32 high part of r^2 (1e-6 relative) and
  // the table spacings as double-floats
  float f_rc2_lo, f_rc2_hi, f_rv2_lo, f_rv2_hi, f_hi;
  float f_pre;  // FP32 prefilter on the high parts: f_hi plus a bound on their rounding
  float erdr_hi, erdr_lo, vrdr_hi, vrdr_lo, scal_hi, scal_lo;
};



__device__ __forceinline__ int vkey(int ai, int aj) {
  return ai > aj ? ai * (ai - 1) / 2 + aj : aj * (aj - 1) / 2 + ai;
}

// exact 3-point formula (numerics.F90:277-288), used for the first interval
__device__ double three_p_exact(const double* c, double d, double r) {
  // c holds (c0,c1,c2) of interval 0 built from (t0*?, t1, t2); rebuild points
  double p1 = c[0], p2 = c[0] + c[1] + c[2], p3 = c[0] + 2.0 * c[1] + 4.0 * c[2];
  p1 = p1 * r;
  double t1 = p1 + (p2 - p1) * d;
  double t2 = p2 + (p3 - p2) * (d - 1.0);
  return t1 + (t2 - t1) * d * 0.5;
}

template <int NV>
__device__ __forceinline__ void acc_store(double (&v)[NV], double* blk) {
  block_reduce_store<NV>(v, blk);
}

// --------------------------------------------------------------- FP64 form
// accumulator layout per block: engvdw, virvdw, engrl, virrl, str(6)
constexpr int NACC = 10;
constexpr int NACC_DF = 4;  // the double-float kernel: energies and virials (stress from k_pair_stress_fix)

__global__ void __launch_bounds__(256, 3) k_pair_fp64(int natms, const DevScalars* sc, const int* __restrict__ at_list,
                                                   const int* __restrict__ list, int ld,
                                                   const double* __restrict__ x, const double* __restrict__ y,
                                                   const double* __restrict__ z, const double* __restrict__ q,
                                                   const int* __restrict__ ltype, const int* __restrict__ ltg,
                                                   const int* __restrict__ src, const double* __restrict__ ecoef,
                                                   const double* __restrict__ vcoef, const int* __restrict__ vkind,
                                                   const double* __restrict__ veps, const double* __restrict__ vsig,
                                                   PairGeom pg, double* fx, double* fy, double* fz, double* blk,
                                                   unsigned long long* cnt) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double acc[NACC];
#pragma unroll
  for (int k = 0; k < NACC; ++k) acc[k] = 0.0;
  const int nlast = sc->nlast;
  // persistent warps walk the atoms in cell order (neighbouring atoms share j data in L1)
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nlast; w += nwarps) {
    const int i = at_list[w];
    if (i >= natms) continue;
    const double xi = x[i], yi = y[i], zi = z[i], qi = q[i] * pg.scaling;
    const bool qi_on = (__double_as_longlong(qi) & 0x7FFFFFFFFFFFFFFFll) >= DBL_MIN_BITS;
    const int ai = ltype[i], gi = ltg[i];
    const int* li = list + (size_t)i * ld + 3;
    const int n = li[0];
    double fix = 0.0, fiy = 0.0, fiz = 0.0;
    const int vstride = (pg.max_grid + 3) * 6;
    int nrc = 0;
    for (int m = lane + 1; m <= n; m += 32) {
      int j = li[m] - 1;
      int jf = j;  // atom receiving the reaction force
      if (j >= natms) {
        if (gi > ltg[j]) continue;  // evaluated from the other side
        jf = src[j];
      }
      // On this part an FP64 compare or conversion costs a full FP64 issue
      // slot, so range tests use the IEEE bit patterns (rsq >= 0 orders like
      // its bits) and the rsqrt seed is built with integer operations.
      const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
      const double rsq = dx * dx + dy * dy + dz * dz;
      const long long rb = __double_as_longlong(rsq);
      if (rb >= pg.b_hi) continue;
      // 1/r: FP32 rsqrt of the truncated value, one FP64 Newton step (rel. error < 1e-13)
      double rinv = flt_to_dbl(rsqrtf(dbl_to_flt_trunc(rsq)));
      rinv = rinv * fma(-0.5 * rsq * rinv, rinv, 1.5);
      const double rrr = rsq * rinv;
      const bool in_c = rb < pg.b_rc2_lo || (rb < pg.b_rc2_hi && sqrt(rsq) < pg.rcut);
      const bool in_v = rb < pg.b_rv2_lo || (rb < pg.b_rv2_hi && sqrt(rsq) < pg.rvdw);
      const double qj = q[j];
      const bool do_c = in_c && qi_on && ((__double_as_longlong(qj) & 0x7FFFFFFFFFFFFFFFll) > DBL_MIN_BITS);
      int key = -1;
      if (in_v) {
        key = vkey(ai, ltype[j]) - 1;
        if (vkind[key] == 0) key = -1;
      }
      if (!do_c && key < 0) continue;
      // shared table coordinate (the erfc and vdW grids coincide when rvdw == rcut);
      // k = Int(ppp) without FP64 conversions: FP32 floor of the truncated value
      // (never above ppp), exact double of k from its bits, one fix-up step
      const double ppp = rrr * pg.erdr;
      int k = (int)dbl_to_flt_trunc(ppp);
      double d = ppp - int_to_dbl(k);
      if (__double_as_longlong(d) >= ONE_BITS) { ++k; d -= 1.0; }
      double gam = 0.0, ee = 0.0, ev = 0.0, gvir_c = 0.0, gvir_v = 0.0;
      // real-space Coulomb (ewald_spole.F90:131-176)
      if (do_c) {
        const double* c = ecoef + (size_t)k * 6;
        const double pre = qi * qj;
        double eg, ec;
        if (k > 0) {
          eg = pre * fma(d, fma(d, c[5], c[4]), c[3]);
          ec = pre * fma(d, fma(d, c[2], c[1]), c[0]);
        } else {
          eg = pre * three_p_exact(c + 3, d, rrr);
          ec = pre * three_p_exact(c, d, rrr);
        }
        gam = eg;
        ee = ec;
        gvir_c = eg;
      }
      // van der Waals (vdw.F90:1881-1962 tabulated / :1670-1700 direct)
      if (key >= 0) {
        const double r_rsq = rinv * rinv;
        double gv, e;
        if (pg.vdw_direct) {
          const double sr = vsig[key] * rinv;
          const double s2 = sr * sr, s6 = s2 * s2 * s2;
          e = 4.0 * veps[key] * s6 * (s6 - 1.0);
          gv = 24.0 * veps[key] * s6 * (2.0 * s6 - 1.0) * r_rsq;
        } else {
          int kv = k;
          double dv = d;
          if (!pg.same_grid) {
            const double pv = rrr * pg.vrdr;
            kv = (int)pv;
            dv = pv - (double)kv;
          }
          const double* c = vcoef + (size_t)key * vstride + (size_t)kv * 6;
          if (kv > 0) {
            gv = fma(dv, fma(dv, c[2], c[1]), c[0]) * r_rsq;
            e = fma(dv, fma(dv, c[5], c[4]), c[3]);
          } else {
            gv = three_p_exact(c, dv, rrr) * r_rsq;
            e = three_p_exact(c + 3, dv, rrr);
          }
        }
        gam += gv;
        ev = e;
        gvir_v = gv;
      }
      ++nrc;
      // reaction force on j (negations fold into the operands: no extra FP64 op)
      const double nfx = (-gam) * dx, nfy = (-gam) * dy, nfz = (-gam) * dz;
      fix -= nfx; fiy -= nfy; fiz -= nfz;
      atomicAdd(&fx[jf], nfx);
      atomicAdd(&fy[jf], nfy);
      atomicAdd(&fz[jf], nfz);
      acc[0] += ev;
      acc[1] = fma(-gvir_v, rsq, acc[1]);
      acc[2] += ee;
      acc[3] = fma(-gvir_c, rsq, acc[3]);
      acc[4] = fma(-dx, nfx, acc[4]); acc[5] = fma(-dx, nfy, acc[5]); acc[6] = fma(-dx, nfz, acc[6]);
      acc[7] = fma(-dy, nfy, acc[7]); acc[8] = fma(-dy, nfz, acc[8]); acc[9] = fma(-dz, nfz, acc[9]);
    }
    fix = warp_sum(fix); fiy = warp_sum(fiy); fiz = warp_sum(fiz);
    nrc = warp_sumi(nrc);
    if (lane == 0) {
      atomicAdd(&fx[i], fix);
      atomicAdd(&fy[i], fiy);
      atomicAdd(&fz[i], fiz);
      atomicAdd(&cnt[0], (unsigned long long)n);
      atomicAdd(&cnt[1], (unsigned long long)nrc);
    }
  }
  block_reduce_store<NACC>(acc, blk);
}

// exclusion correction (FP64), one thread per atom over its excluded section
// In the mixed form the same FP64 kernel writes fixed-point forces (fixp != 0):
// the intramolecular exclusion terms cancel against the reciprocal energy
// (tens of millions of internal units for water), so they stay in FP64.
__global__ void k_excl_fp64(int natms, const int* list, int ld, const double* x, const double* y, const double* z,
                            const double* q, const int* ltg, const int* src, double alpha, double scaling,
                            double rcut, double* fx, double* fy, double* fz, double* blk,
                            unsigned long long* fixp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (i < natms) {
    const int* li = list + (size_t)i * ld + 3;
    int lim = li[-1] - li[0];
    double chgea = q[i];
    if (lim > 0 && fabs(chgea) > DBL_MIN) {
      chgea *= scaling;
      const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741, a4 = -1.453152027,
                   a5 = 1.061405429, pp = 0.3275911, r10 = 0.1, r216 = 1.0 / 216.0, r42 = 1.0 / 42.0,
                   rr3 = 1.0 / 3.0, sqrpi = 1.7724538509055160273;
      double fix = 0, fiy = 0, fiz = 0;
      for (int m = 1; m <= lim; ++m) {
        int j = li[li[0] + m] - 1;
        double xx = x[i] - x[j], yy = y[i] - y[j], zz = z[i] - z[j];
        double rrr = sqrt(xx * xx + yy * yy + zz * zz);
        double chgprd = q[j];
        if (fabs(chgprd) > DBL_MIN && rrr < rcut) {
          chgprd *= chgea;
          double rsq = rrr * rrr, alpr = rrr * alpha, alpr2 = alpr * alpr, erfr, egamma;
          if (alpr < 1.0e-2) {
            erfr = 2.0 * chgprd * (alpha / sqrpi) * (1.0 + alpr2 * (-rr3 + alpr2 * (r10 + alpr2 * (-r42 + alpr2 * r216))));
            egamma = -4.0 * chgprd * (alpha * alpha * alpha / sqrpi) *
                     (rr3 + alpr2 * (-2.0 * r10 + alpr2 * (3.0 * r42 - 4.0 * alpr2 * r216)));
          } else {
            double exp1 = exp(-(alpha * rrr) * (alpha * rrr));
            double tt = 1.0 / (1.0 + pp * alpha * rrr);
            erfr = chgprd * (1.0 - tt * (a1 + tt * (a2 + tt * (a3 + tt * (a4 + tt * a5)))) * exp1) / rrr;
            egamma = -(erfr - 2.0 * chgprd * (alpha / sqrpi) * exp1) / rsq;
          }
          double fx_ = egamma * xx, fy_ = egamma * yy, fz_ = egamma * zz;
          fix += fx_; fiy += fy_; fiz += fz_;
          if (j < natms) {
            if (fixp) {
              const double sc = 1099511627776.0;
              atomicAdd(&fixp[3 * j + 0], (unsigned long long)(-__double2ll_rn(fx_ * sc)));
              atomicAdd(&fixp[3 * j + 1], (unsigned long long)(-__double2ll_rn(fy_ * sc)));
              atomicAdd(&fixp[3 * j + 2], (unsigned long long)(-__double2ll_rn(fz_ * sc)));
            } else {
              atomicAdd(&fx[j], -fx_); atomicAdd(&fy[j], -fy_); atomicAdd(&fz[j], -fz_);
            }
          }
          if (j < natms || ltg[i] < ltg[j]) {
            acc[0] -= erfr;
            acc[1] -= egamma * rsq;
            acc[2] += xx * fx_; acc[3] += xx * fy_; acc[4] += xx * fz_;
            acc[5] += yy * fy_; acc[6] += yy * fz_; acc[7] += zz * fz_;
          }
        }
      }
      if (fixp) {
        const double sc = 1099511627776.0;
        atomicAdd(&fixp[3 * i + 0], (unsigned long long)__double2ll_rn(fix * sc));
        atomicAdd(&fixp[3 * i + 1], (unsigned long long)__double2ll_rn(fiy * sc));
        atomicAdd(&fixp[3 * i + 2], (unsigned long long)__double2ll_rn(fiz * sc));
      } else {
        atomicAdd(&fx[i], fix); atomicAdd(&fy[i], fiy); atomicAdd(&fz[i], fiz);
      }
    }
  }
  block_reduce_store<8>(acc, blk);
}

// -------------------------------------------------------------- mixed form
// FP32 arithmetic, int64 fixed-point force sums; energies and virials are
// summed per lane in FP32 (compensated) and reduced in FP64.  The erfc and LJ
// functions are evaluated directly: on this part FP32 math and MUFU are far
// cheaper than the random table reads the FP64 form's exact interpolation needs.
constexpr float AS_A1 = 0.254829592f, AS_A2 = -0.284496736f, AS_A3 = 1.421413741f, AS_A4 = -1.453152027f,
                AS_A5 = 1.061405429f, AS_P = 0.3275911f;
constexpr int MAX_KEYS = 64;
constexpr int MAX_TYPES = 10;  // 55 type-pair keys
__constant__ float4 c_lj[MAX_KEYS];
// Mixed form on the half list: each pair is evaluated once and its force goes
// to i (per-lane int64 sums) and, negated, to j (one 64-bit integer atomic
// per component).  Integer addition is associative, so the forces are the
// same whatever the order the warps and atomics run in.  Halo pairs are
// evaluated from the side with the smaller global id and applied to the
// image's source atom, as in the FP64 kernel.
__global__ void __launch_bounds__(256, 4) k_pair_mixed_half(int natms, const DevScalars* sc,
                                                         const int* __restrict__ at_list,
                                                         const int* __restrict__ list, int ld,
                                                         const float4* __restrict__ xf, const float4* __restrict__ xlo,
                                                         const int* __restrict__ ltype, const int* __restrict__ ltg,
                                                         const int* __restrict__ src, int ntypes, float rc2, float rv2,
                                                         float alpha, float alpha2rsqrpi, float scaling,
                                                         unsigned long long* fixp, double* blk,
                                                         unsigned long long* cnt) {
  __shared__ float4 s_lj[MAX_TYPES * MAX_TYPES];
  for (int e = threadIdx.x; e < ntypes * ntypes; e += blockDim.x) {
    const int ai = e / ntypes + 1, aj = e % ntypes + 1;
    s_lj[e] = c_lj[vkey(ai, aj) - 1];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  // lane k < NACC keeps the compensated running sum of quantity k over the
  // warp's atoms (2 registers instead of 2 x NACC per lane)
  float a_k = 0.f, c_k = 0.f;
  unsigned long long n_list = 0, n_rc = 0;
  const int nlast = sc->nlast;
  // persistent warps walk the atoms in cell order (neighbouring atoms share j data in L1)
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nlast; w += nwarps) {
    const int i = at_list[w];
    if (i >= natms) continue;
    const float4 pi = xf[i];
    const float4 li = xlo[i];
    const float qi = pi.w * scaling;
    const int row = (ltype[i] - 1) * ntypes - 1;
    const int gi = ltg[i];
    const int* lst = list + (size_t)i * ld + 3;
    const int n = lst[0];
    long long sx = 0, sy = 0, sz = 0;
    float t[NACC];
#pragma unroll
    for (int k = 0; k < NACC; ++k) t[k] = 0.f;
    for (int m = lane + 1; m <= n; m += 32) {
      const int j = lst[m] - 1;
      int jf = j;
      if (j >= natms) {
        if (gi > ltg[j]) continue;  // evaluated from the other side
        jf = src[j];
      }
      const float4 pj = xf[j];
      const float4 lj = xlo[j];
      const float dx = (pi.x - pj.x) + (li.x - lj.x), dy = (pi.y - pj.y) + (li.y - lj.y),
                  dz = (pi.z - pj.z) + (li.z - lj.z);
      const float rsq = dx * dx + dy * dy + dz * dz;
      if (rsq >= rc2 && rsq >= rv2) continue;
      const float rinv = rsqrtf(rsq);
      const float rrr = rsq * rinv;
      const float r2i = rinv * rinv;
      float gam = 0.f;
      if (rsq < rc2 && pj.w != 0.f) {
        const float x = alpha * rrr;
        const float ex = __expf(-x * x);
        const float tt = __frcp_rn(fmaf(AS_P, x, 1.0f));
        const float poly = tt * fmaf(tt, fmaf(tt, fmaf(tt, fmaf(tt, AS_A5, AS_A4), AS_A3), AS_A2), AS_A1);
        const float pre = qi * pj.w;
        const float ec = pre * poly * ex * rinv;
        const float eg = fmaf(pre * alpha2rsqrpi, ex, ec) * r2i;
        gam += eg;
        t[2] += ec;
        t[3] = fmaf(-eg, rsq, t[3]);
      }
      if (rsq < rv2) {
        const float4 lj6 = s_lj[row + __float_as_int(lj.w)];  // xlo.w holds the type
        if (lj6.w != 0.f) {
          const float s2 = lj6.z * r2i;
          const float s6 = s2 * s2 * s2;
          const float gv = lj6.y * s6 * fmaf(2.0f, s6, -1.0f) * r2i;
          gam += gv;
          t[0] = fmaf(lj6.x * s6, s6 - 1.0f, t[0]);
          t[1] = fmaf(-gv, rsq, t[1]);
        }
      }
      ++n_rc;
      const float fx_ = gam * dx, fy_ = gam * dy, fz_ = gam * dz;
      const long long ix = fix40(fx_), iy = fix40(fy_), iz = fix40(fz_);
      sx += ix; sy += iy; sz += iz;
      atomicAdd(&fixp[3 * jf + 0], (unsigned long long)(-ix));
      atomicAdd(&fixp[3 * jf + 1], (unsigned long long)(-iy));
      atomicAdd(&fixp[3 * jf + 2], (unsigned long long)(-iz));
      t[4] = fmaf(dx, fx_, t[4]); t[5] = fmaf(dx, fy_, t[5]); t[6] = fmaf(dx, fz_, t[6]);
      t[7] = fmaf(dy, fy_, t[7]); t[8] = fmaf(dy, fz_, t[8]); t[9] = fmaf(dz, fz_, t[9]);
    }
#pragma unroll
    for (int k = 0; k < NACC; ++k) {
      const float v = warp_sumf(t[k]);  // this atom's share, in every lane
      if (lane == k) {
        const float y = v - c_k, tt = a_k + y;
        c_k = (tt - a_k) - y;
        a_k = tt;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
      sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    if (lane == 0) {
      atomicAdd(&fixp[3 * i + 0], (unsigned long long)sx);
      atomicAdd(&fixp[3 * i + 1], (unsigned long long)sy);
      atomicAdd(&fixp[3 * i + 2], (unsigned long long)sz);
      n_list += (unsigned long long)n;
    }
  }
  double acc[NACC];
  const double own = (double)a_k - (double)c_k;
#pragma unroll
  for (int k = 0; k < NACC; ++k) acc[k] = (lane == k) ? own : 0.0;
  n_rc = (unsigned long long)warp_sumi((int)n_rc);
  if (lane == 0) {
    atomicAdd(&cnt[0], n_list);
    atomicAdd(&cnt[1], n_rc);
  }
  block_reduce_store<NACC>(acc, blk);
}

inline int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// ===================================================================== host
// per-key LJ constants for the mixed form (4 eps, 24 eps, sigma^2)
void pair_setup() {
  if (g.nkey > MAX_KEYS || g.p.ntypes > MAX_TYPES) throw (int)GB_ERR_ARG;
  float4 lj[MAX_KEYS];
  for (int k = 0; k < MAX_KEYS; ++k) lj[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k = 0; k < g.nkey; ++k) {
    const double e = g.h_vdw_eps[k], s = g.h_vdw_sig[k];
    const float present = g.h_vdw_kind[k] != 0 ? 1.f : 0.f;
    lj[k] = make_float4((float)(4.0 * e), (float)(24.0 * e), (float)(s * s), present);
  }
  GB_CUDA(cudaMemcpyToSymbol(c_lj, lj, sizeof(lj)));
}

// ------------------------------------------------------- FP64 form, double-float
// The FP64 form's pair loop on the FP32 pipes: positions as FP32 hi + lo pairs (48
// bits), the separation formed with an exact two-sum, r^2, 1/r, the table coordinate and
// the three-point polynomials in double-float; pair forces summed as int64 fixed point
// (2^40) with 64-bit integer atomics for j, energies and virials in double-float running
// sums.  Pairs whose r^2 lies within 1e-6 of a cutoff squared, and pairs in the first
// table interval, take the FP64 formulas of k_pair_fp64 (exact cutoff decisions).
// Measured against the FP64 oracle: forces and energies agree to ~1e-13.

// per interval of a double-float table: (c0 hi, c0 lo, c1 hi, c1 lo) of the energy and
// of the force polynomial, then (c2 hi, c2 lo) of both; c0 + d (c1 + d c2) in double-float
// throughout (near the repulsive wall of a 12-6 table the quadratic term reaches 1e-3 of
// the value, so it needs the full precision too)
__device__ __forceinline__ df poly_df(float4 c01, float c2h, float c2l, df d) {
  const df t = df_fma(d, df_make(c2h, c2l), df_make(c01.z, c01.w));
  return df_fma(d, t, df_make(c01.x, c01.y));
}

// FP64 terms of one pair, as k_pair_fp64 evaluates them (slow path)
__device__ void pair_terms_fp64(const PairGeom& pg, double dx, double dy, double dz, double qi, double qj, int ai,
                                int aj, const double* ecoef, const double* vcoef, const int* vkind, const double* veps,
                                const double* vsig, double* gam, double* ee, double* ev, double* gvc, double* gvv,
                                bool* any) {
  *gam = *ee = *ev = *gvc = *gvv = 0.0;
  *any = false;
  const double rsq = dx * dx + dy * dy + dz * dz;
  const double rrr = sqrt(rsq);
  const bool in_c = rrr < pg.rcut && qi != 0.0 && qj != 0.0;
  int key = -1;
  if (rrr < pg.rvdw) {
    key = vkey(ai, aj) - 1;
    if (vkind[key] == 0) key = -1;
  }
  if (!in_c && key < 0) return;
  *any = true;
  if (in_c) {
    const double ppp = rrr * pg.erdr;
    const int k = (int)ppp;
    const double d = ppp - (double)k;
    const double* c = ecoef + (size_t)k * 6;
    const double pre = qi * qj;
    double eg, ec;
    if (k > 0) {
      eg = pre * fma(d, fma(d, c[5], c[4]), c[3]);
      ec = pre * fma(d, fma(d, c[2], c[1]), c[0]);
    } else {
      eg = pre * three_p_exact(c + 3, d, rrr);
      ec = pre * three_p_exact(c, d, rrr);
    }
    *gam = eg; *ee = ec; *gvc = eg;
  }
  if (key >= 0) {
    const double rinv = 1.0 / rrr, r_rsq = rinv * rinv;
    double gv, e;
    if (pg.vdw_direct) {
      const double sr = vsig[key] * rinv;
      const double s2 = sr * sr, s6 = s2 * s2 * s2;
      e = 4.0 * veps[key] * s6 * (s6 - 1.0);
      gv = 24.0 * veps[key] * s6 * (2.0 * s6 - 1.0) * r_rsq;
    } else {
      const double pv = rrr * pg.vrdr;
      const int kv = (int)pv;
      const double dv = pv - (double)kv;
      const double* c = vcoef + (size_t)key * (pg.max_grid + 3) * 6 + (size_t)kv * 6;
      if (kv > 0) {
        gv = fma(dv, fma(dv, c[2], c[1]), c[0]) * r_rsq;
        e = fma(dv, fma(dv, c[5], c[4]), c[3]);
      } else {
        gv = three_p_exact(c, dv, rrr) * r_rsq;
        e = three_p_exact(c + 3, dv, rrr);
      }
    }
    *gam += gv; *ev = e; *gvv = gv;
  }
}

// table coordinate of a double-float r: k = Int(ppp) and d = ppp - k in double-float
__device__ __forceinline__ int table_coord(df rrr, float sh, float sl, df* d) {
  const df ppp = df_mul(rrr, df_make(sh, sl));
  int k = (int)ppp.hi;                                   // ppp >= 0: truncation
  if ((float)k == ppp.hi && ppp.lo < 0.0f) --k;          // hi integral, value just below it
  *d = quick_two_sum(__fsub_rn(ppp.hi, (float)k), ppp.lo);
  return k;
}

// per-warp queue of pairs inside the outer cutoff: neighbour index and double-float r^2
struct PairQueue {
  int j[64];
};
constexpr int PAIR_DF_NT = 256;  // threads of a k_pair_df64 CTA

// the pair terms of one queued pair (ewald_spole.F90:131-176, vdw.F90:1881-1962), its
// fixed-point forces and the running energy, virial and stress sums
__device__ __forceinline__ void pair_terms_df64(const PairGeom& pg, int i, int j, int jf, int ai, int aj, df qi,
                                                bool qi_on, float2 qj2, df dx, df dy, df dz, df rsq,
                                                const double* __restrict__ x, const double* __restrict__ y,
                                                const double* __restrict__ z, const double* __restrict__ q,
                                                const float4* __restrict__ etab, const float4* __restrict__ vtab,
                                                const double* __restrict__ ecoef, const double* __restrict__ vcoef,
                                                const int* __restrict__ vkind, const double* __restrict__ veps,
                                                const double* __restrict__ vsig, int vstride,
                                                unsigned long long* fixp, dacc (&acc)[NACC_DF], long long& sx,
                                                long long& sy, long long& sz, unsigned long long& n_rc) {
  const bool band = (rsq.hi >= pg.f_rc2_lo && rsq.hi <= pg.f_rc2_hi) ||
                    (rsq.hi >= pg.f_rv2_lo && rsq.hi <= pg.f_rv2_hi);
  const bool in_c = qi_on && qj2.x != 0.0f && rsq.hi < pg.f_rc2_lo;
  int key = -1;
  if (rsq.hi < pg.f_rv2_lo) {
    key = vkey(ai, aj) - 1;
    if (vkind[key] == 0) key = -1;
  }
  df gam = df_make(0.f, 0.f), ee = gam, ev = gam, gvc = gam, gvv = gam;
  bool slow = band;
  if (!slow && (in_c || key >= 0)) {
    const df rinv = df_rsqrt(rsq);
    const df rrr = df_mul(rsq, rinv);
    df d;
    const int k = table_coord(rrr, pg.erdr_hi, pg.erdr_lo, &d);
    int kv = k;
    df dv = d;
    if (!pg.same_grid && key >= 0) kv = table_coord(rrr, pg.vrdr_hi, pg.vrdr_lo, &dv);
    if (k == 0 || (key >= 0 && kv == 0)) {
      slow = true;  // first interval: the exact three-point formula, in FP64
    } else {
      if (in_c) {  // real-space Coulomb
        const float4* c = etab + (size_t)k * 3;
        const float4 e01 = c[0], d01 = c[1], c2 = c[2];
        const df pre = df_mul(qi, df_make(qj2.x, qj2.y));
        gvc = df_mul(pre, poly_df(d01, c2.z, c2.w, d));
        ee = df_mul(pre, poly_df(e01, c2.x, c2.y, d));
        gam = gvc;
      }
      if (key >= 0) {  // van der Waals, tabulated
        const df r_rsq = df_sqr(rinv);
        if (pg.vdw_direct) {
          slow = true;
        } else {
          const float4* c = vtab + (size_t)key * vstride + (size_t)kv * 3;
          const float4 f01 = c[0], v01 = c[1], c2 = c[2];
          gvv = df_mul(poly_df(f01, c2.x, c2.y, dv), r_rsq);
          ev = poly_df(v01, c2.z, c2.w, dv);
          gam = df_add(gam, gvv);
        }
      }
    }
  }
  if (slow) {
    double g64, e64c, e64v, gc64, gv64;
    bool any;
    pair_terms_fp64(pg, x[i] - x[j], y[i] - y[j], z[i] - z[j], q[i] * pg.scaling, q[j], ai, aj, ecoef, vcoef,
                    vkind, veps, vsig, &g64, &e64c, &e64v, &gc64, &gv64, &any);
    if (!any) return;
    float h, l;
    df_split(g64, &h, &l); gam = df_make(h, l);
    df_split(e64c, &h, &l); ee = df_make(h, l);
    df_split(e64v, &h, &l); ev = df_make(h, l);
    df_split(gc64, &h, &l); gvc = df_make(h, l);
    df_split(gv64, &h, &l); gvv = df_make(h, l);
  } else if (!in_c && key < 0) {
    return;
  }
  ++n_rc;
  const df fxx = df_mul(gam, dx), fyy = df_mul(gam, dy), fzz = df_mul(gam, dz);
  const long long ix = fix40_df(fxx), iy = fix40_df(fyy), iz = fix40_df(fzz);
  sx += ix; sy += iy; sz += iz;
  atomicAdd(&fixp[3 * jf + 0], (unsigned long long)(-ix));
  atomicAdd(&fixp[3 * jf + 1], (unsigned long long)(-iy));
  atomicAdd(&fixp[3 * jf + 2], (unsigned long long)(-iz));
  dacc_add(acc[0], ev);
  dacc_add_prod(acc[1], df_neg(gvv), rsq);
  dacc_add(acc[2], ee);
  dacc_add_prod(acc[3], df_neg(gvc), rsq);
}

__global__ void __launch_bounds__(PAIR_DF_NT, 4) k_pair_df64(int natms, const DevScalars* sc, const int* __restrict__ at_list,
                                                   const int* __restrict__ list, int ld,
                                                   const float4* __restrict__ xf, const float4* __restrict__ xlo,
                                                   const float2* __restrict__ qdf, const double* __restrict__ x,
                                                   const double* __restrict__ y, const double* __restrict__ z,
                                                   const double* __restrict__ q, const int* __restrict__ ltg,
                                                   const int* __restrict__ src, const float4* __restrict__ etab,
                                                   const float4* __restrict__ vtab, const double* __restrict__ ecoef,
                                                   const double* __restrict__ vcoef, const int* __restrict__ vkind,
                                                   const double* __restrict__ veps, const double* __restrict__ vsig,
                                                   PairGeom pg, unsigned long long* fixp, double* blk,
                                                   unsigned long long* cnt) {
  __shared__ PairQueue pq[PAIR_DF_NT / 32];
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  dacc acc[NACC_DF];
#pragma unroll
  for (int k = 0; k < NACC_DF; ++k) { acc[k].s = 0.f; acc[k].c = 0.f; }
  unsigned long long n_list = 0, n_rc = 0;
  const int nlast = sc->nlast;
  const int vstride = (pg.max_grid + 3) * 3;  // float4 per key
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nlast; w += nwarps) {
    const int i = at_list[w];
    if (i >= natms) continue;
    const float4 pi = xf[i], li = xlo[i];
    const float2 qi2 = qdf[i];
    const df qi = df_mul(df_make(qi2.x, qi2.y), df_make(pg.scal_hi, pg.scal_lo));  // q_i r4pie0/eps
    const bool qi_on = qi2.x != 0.0f;
    const int ai = __float_as_int(li.w), gi = ltg[i];
    const int* lst = list + (size_t)i * ld + 3;
    const int n = lst[0];
    long long sx = 0, sy = 0, sz = 0;
    // Pass 1 over 32 entries at a time: an FP32 r^2 of the coordinates' high parts, with
    // a bound on their rounding added to the outer cutoff, so that every entry inside
    // the cutoff (and a few just outside) joins this warp's queue (ballot compaction).
    // Pass 2, the exact separation and the pair terms, runs on 32 queued pairs at a
    // time with every lane busy.  The queue holds < 64 pairs.
    int nq = 0;  // queued pairs (uniform over the warp)
    for (int base = 0;; base += 32) {
      const bool more = base < n;
      if (more) {
        const int m = base + lane + 1;
        bool keep = false;
        int j = 0;
        if (m <= n) {
          j = lst[m] - 1;
          if (j < natms || gi <= ltg[j]) {  // halo pairs are evaluated from the smaller id
            const float4 pj = xf[j];
            const float ex = pi.x - pj.x, ey = pi.y - pj.y, ez = pi.z - pj.z;
            keep = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= pg.f_pre;
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (keep) {
          const int slot = nq + __popc(bal & ((1u << lane) - 1u));
          pq[wq].j[slot] = j;
        }
        nq += __popc(bal);
        __syncwarp();
      }
      if (nq >= 32 || (!more && nq > 0)) {
        const int take = min(nq, 32);
        const int slot = nq - take + lane;
        if (lane < take) {
          const int j = pq[wq].j[slot];
          // separation: exact difference of the high parts plus the difference of the low parts
          const float4 pj = xf[j], lj = xlo[j];
          const int aj = __float_as_int(lj.w);
          const df ex = two_sum(pi.x, -pj.x), ey = two_sum(pi.y, -pj.y), ez = two_sum(pi.z, -pj.z);
          const df dx = quick_two_sum(ex.hi, __fadd_rn(ex.lo, __fsub_rn(li.x, lj.x)));
          const df dy = quick_two_sum(ey.hi, __fadd_rn(ey.lo, __fsub_rn(li.y, lj.y)));
          const df dz = quick_two_sum(ez.hi, __fadd_rn(ez.lo, __fsub_rn(li.z, lj.z)));
          const df rsq = df_norm2(dx, dy, dz);
          if (rsq.hi <= pg.f_hi) {
            const int jf = j;  // an image's force stays in its own slot until k_fold_images
            const float2 qj2 = qdf[j];
            pair_terms_df64(pg, i, j, jf, ai, aj, qi, qi_on, qj2, dx, dy, dz, rsq, x, y, z, q, etab, vtab, ecoef,
                            vcoef, vkind, veps, vsig, vstride, fixp, acc, sx, sy, sz, n_rc);
          }
        }
        nq -= take;
        __syncwarp();  // the taken slots are read before the next pass appends over them
      }
      if (!more && nq == 0) break;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
      sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    if (lane == 0) {
      atomicAdd(&fixp[3 * i + 0], (unsigned long long)sx);
      atomicAdd(&fixp[3 * i + 1], (unsigned long long)sy);
      atomicAdd(&fixp[3 * i + 2], (unsigned long long)sz);
      n_list += (unsigned long long)n;
    }
  }
  dfr out[NACC_DF];
#pragma unroll
  for (int k = 0; k < NACC_DF; ++k) out[k] = to_dfr(two_sum(acc[k].s, acc[k].c));
  n_rc = (unsigned long long)warp_sumi((int)n_rc);
  if (lane == 0) {
    atomicAdd(&cnt[0], n_list);
    atomicAdd(&cnt[1], n_rc);
  }
  block_reduce_store<NACC_DF>(out, blk);
}

// ------------------------------------------------------- sorted-position kernels
// The pair loop over the list's partners in cell (sorted) order.  The list build writes,
// beside list(k, i), spos(k, i): the partner's position in the cell-sorted arrays, or -1
// for an entry of the backward halo pass (that pair is also listed, in its forward
// pass, by the partner atom and is evaluated there).  Persistent warps walk the local
// atoms in sorted order, so the warps of a CTA work on one cell and read the same
// neighbour cells: the partner data (FP32 high parts with the charge, remainders, type)
// are contiguous runs that L1 holds, not gathers by atom index.  Pair forces go to
// per-sorted-position int64 fixed-point sums (64-bit integer reductions: the result does
// not depend on their order); k_slot_stress_fold sums the stress and moves them to atoms.
// CTA size by form (measured at 262,144 ions, each CTA on a contiguous run of the local
// atoms; pair time per launch and MD step with SPME on the side stream, 1024-thread CTAs
// (one per SM) / 256-thread CTAs (four per SM)): double-float 1.192 / 1.285 ms, step 2.77 /
// 2.84 ms; mixed 0.687 / 0.687 ms, step 1.52 / 1.48 ms (the side stream's kernels find room
// beside the smaller CTAs).  GB_PAIR_NT=256 or 1024 sets it for both forms.
constexpr int PAIR_SORTED_NT = 1024;

struct PairSortedArgs {
  int natms;
  const int* at_list;
  const int* loc_sp;  // the local atoms' sorted positions, in sorted order
  const int* list;
  int ld;
  const int* spos;
  int ldt;
  const float4* xhs;
  const float4* xls;
  const unsigned char* tys;
  const uint2* xlh;  // mixed form: remainders and type in 8 bytes (pair_lo_type)
  const double *x, *y, *z, *q;  // FP64 by atom index: the exact pair evaluation near a cutoff
  const float4* etab;
  int netab;  // float4 entries of etab (the FP64 form copies the table into shared memory)
  const float4* vtab;
  const double* ecoef;
  const double* vcoef;
  const int* vkind;
  const double* veps;
  const double* vsig;
  int ntypes;
  float rc2, rv2, alpha, a2rp, scaling;  // mixed form
  unsigned long long* fixs;
  double* blk;
  unsigned long long* cnt;
  const DevScalars* sc;
};

// The FP64 form's terms of one pair (the arithmetic of pair_terms_df64, partner data
// passed in); jp is the partner's sorted position, whose atom index the exact FP64
// evaluation near a cutoff looks up.
// Returns false when the pair exerts no force.
__device__ __forceinline__ bool pair_df64_eval(const PairGeom& pg, const PairSortedArgs& A, const float4* etab,
                                               int i, int jp, int ai,
                                               int aj, df qi, bool qi_on, float qjh, float qjl, df dx, df dy, df dz,
                                               df rsq, dacc (&acc)[NACC_DF], long long& ix, long long& iy,
                                               long long& iz) {
  const bool band = (rsq.hi >= pg.f_rc2_lo && rsq.hi <= pg.f_rc2_hi) ||
                    (rsq.hi >= pg.f_rv2_lo && rsq.hi <= pg.f_rv2_hi);
  const bool in_c = qi_on && qjh != 0.0f && rsq.hi < pg.f_rc2_lo;
  int key = -1;
  if (rsq.hi < pg.f_rv2_lo) {
    key = vkey(ai, aj) - 1;
    if (A.vkind[key] == 0) key = -1;
  }
  // wv: the vdW virial term -gvv r^2 (-G(r) of the table itself on the fast path)
  df gam = df_make(0.f, 0.f), ee = gam, ev = gam, gvc = gam, gvv = gam, wv = gam;
  bool slow = band;
  if (!slow && (in_c || key >= 0)) {
    const df rinv = df_rsqrt(rsq);
    const df rrr = df_mul(rsq, rinv);
    df d;
    const int k = table_coord(rrr, pg.erdr_hi, pg.erdr_lo, &d);
    int kv = k;
    df dv = d;
    if (!pg.same_grid && key >= 0) kv = table_coord(rrr, pg.vrdr_hi, pg.vrdr_lo, &dv);
    if (k == 0 || (key >= 0 && kv == 0)) {
      slow = true;  // first interval: the exact three-point formula, in FP64
    } else {
      if (in_c) {
        const float4* c = etab + k * 3;
        const float4 e01 = c[0], d01 = c[1], c2 = c[2];
        const df pre = df_mul(qi, df_make(qjh, qjl));
        gvc = df_mul(pre, poly_df(d01, c2.z, c2.w, d));
        ee = df_mul(pre, poly_df(e01, c2.x, c2.y, d));
        gam = gvc;
      }
      if (key >= 0) {
        const df r_rsq = df_sqr(rinv);
        if (pg.vdw_direct) {
          slow = true;
        } else {
          const float4* c = A.vtab + (size_t)key * ((pg.max_grid + 3) * 3) + (size_t)kv * 3;
          const float4 f01 = c[0], v01 = c[1], c2 = c[2];
          const df G = poly_df(f01, c2.x, c2.y, dv);
          gvv = df_mul(G, r_rsq);
          wv = df_neg(G);
          ev = poly_df(v01, c2.z, c2.w, dv);
          gam = df_add(gam, gvv);
        }
      }
    }
  }
  if (slow) {
    double g64, e64c, e64v, gc64, gv64;
    bool any;
    const int j = A.at_list[jp];
    pair_terms_fp64(pg, A.x[i] - A.x[j], A.y[i] - A.y[j], A.z[i] - A.z[j], A.q[i] * pg.scaling, A.q[j], ai, aj,
                    A.ecoef, A.vcoef, A.vkind, A.veps, A.vsig, &g64, &e64c, &e64v, &gc64, &gv64, &any);
    if (!any) return false;
    float h, l;
    df_split(g64, &h, &l); gam = df_make(h, l);
    df_split(e64c, &h, &l); ee = df_make(h, l);
    df_split(e64v, &h, &l); ev = df_make(h, l);
    df_split(gc64, &h, &l); gvc = df_make(h, l);
    df_split(gv64, &h, &l); gvv = df_make(h, l);
    wv = df_neg(df_mul(gvv, rsq));
  } else if (!in_c && key < 0) {
    return false;
  }
  ix = fix40_prod(gam, dx);
  iy = fix40_prod(gam, dy);
  iz = fix40_prod(gam, dz);
  dacc_add(acc[0], ev);
  dacc_add(acc[1], wv);
  dacc_add(acc[2], ee);
  dacc_add_prod(acc[3], df_neg(gvc), rsq);
  return true;
}

// The mixed form's terms of one pair (FP32, analytic erfc and 12-6 LJ, as k_pair_mixed_half).
// The four energy and virial terms go to the lane's FP32 sums of the current atom (e4:
// vdW energy, vdW virial, Coulomb energy, Coulomb virial), which enter the compensated
// running sums once per atom; the forces leave as 2^40 fixed point, truncated toward zero
// by the hardware float-to-int64 conversion (the value fix40 forms with integer operations).
__device__ __forceinline__ long long fix40_cvt(float x) { return __float2ll_rz(__fmul_rn(x, 1099511627776.0f)); }

__device__ __forceinline__ bool pair_mixed_eval(const PairSortedArgs& A, const float4* s_lj, int row, int aj,
                                                float qi, float qj, float dx, float dy, float dz, float (&e4)[4],
                                                long long& ix, long long& iy, long long& iz) {
  const float rsq = dx * dx + dy * dy + dz * dz;
  if (rsq >= A.rc2 && rsq >= A.rv2) return false;
  const float rinv = rsqrtf(rsq);
  const float rrr = rsq * rinv;
  const float r2i = rinv * rinv;
  float gam = 0.f;
  bool any = false;
  if (rsq < A.rc2 && qj != 0.f) {
    const float x = A.alpha * rrr;
    const float ex = __expf(-x * x);
    const float tt = __frcp_rn(fmaf(AS_P, x, 1.0f));
    const float poly = tt * fmaf(tt, fmaf(tt, fmaf(tt, fmaf(tt, AS_A5, AS_A4), AS_A3), AS_A2), AS_A1);
    const float pre = qi * qj;
    const float ec = pre * poly * ex * rinv;
    const float eg = fmaf(pre * A.a2rp, ex, ec) * r2i;
    gam += eg;
    e4[2] += ec;
    e4[3] -= eg * rsq;
    any = true;
  }
  if (rsq < A.rv2) {
    const float4 lj6 = s_lj[row + aj];
    if (lj6.w != 0.f) {
      const float s2 = lj6.z * r2i;
      const float s6 = s2 * s2 * s2;
      const float gv = lj6.y * s6 * fmaf(2.0f, s6, -1.0f) * r2i;
      gam += gv;
      e4[0] += lj6.x * s6 * (s6 - 1.0f);
      e4[1] -= gv * rsq;
      any = true;
    }
  }
  if (!any) return false;
  ix = fix40_cvt(gam * dx);
  iy = fix40_cvt(gam * dy);
  iz = fix40_cvt(gam * dz);
  return true;
}

template <int N>
struct PairQueueN {
  int j[N];
};

template <int MIXED, int U, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_pair_sorted(PairSortedArgs A, PairGeom pg) {
  __shared__ PairQueueN<32 * (U + 1)> pq[NT / 32];
  __shared__ float4 s_lj[MIXED ? MAX_TYPES * MAX_TYPES : 1];
  extern __shared__ float4 s_etab[];  // FP64 form: the double-float erfc table
  if (MIXED) {
    for (int e = threadIdx.x; e < A.ntypes * A.ntypes; e += blockDim.x) {
      const int ai = e / A.ntypes + 1, aj = e % A.ntypes + 1;
      s_lj[e] = c_lj[vkey(ai, aj) - 1];
    }
    __syncthreads();
  } else {
    for (int e = threadIdx.x; e < A.netab; e += blockDim.x) s_etab[e] = A.etab[e];
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  dacc acc[NACC_DF];
#pragma unroll
  for (int k = 0; k < NACC_DF; ++k) { acc[k].s = 0.f; acc[k].c = 0.f; }
  unsigned long long n_list = 0, n_rc = 0;
  // Each CTA takes an equal, contiguous run of the local atoms in sorted (cell) order, its
  // warps NT / 32 consecutive atoms at a time: the partners of the atoms in flight are the
  // same few link cells, and the next atoms' mostly the same, which the SM's L1 holds.
  const int per = (A.natms + gridDim.x - 1) / gridDim.x;
  const int a_end = min(A.natms, (int)(blockIdx.x + 1) * per);
  for (int a = blockIdx.x * per + wq; a < a_end; a += NT / 32) {
    const int p = A.loc_sp[a];
    const int i = A.at_list[p];
    const float4 pi = A.xhs[p];
    float4 li;
    int ai;
    if (MIXED) {
      pair_lo_type(A.xlh[p], li.x, li.y, li.z, ai);
      li.w = 0.f;
    } else {
      li = A.xls[p];
      ai = A.tys[p];
    }
    const df qi = df_mul(df_make(pi.w, li.w), df_make(pg.scal_hi, pg.scal_lo));  // q_i r4pie0/eps
    const bool qi_on = pi.w != 0.0f;
    const float qi32 = pi.w * A.scaling;
    const int ljrow = (ai - 1) * A.ntypes - 1;
    const int n = A.list[(size_t)i * A.ld + 3];
    const int* sp = A.spos + (size_t)i * A.ldt;
    long long sx = 0, sy = 0, sz = 0;
    float e4[4] = {0.f, 0.f, 0.f, 0.f};  // mixed form: this atom's energy and virial terms
    // pass 1, 32 U entries at a time (U per lane, their loads in flight together): an FP32
    // r^2 of the high parts against the outer cutoff plus a bound on their rounding queues
    // the candidates (ballot compaction); pass 2 evaluates 32 queued pairs at a time with
    // every lane busy.  The queue holds < 32 (U + 1) pairs.
    int nq = 0;
    for (int base = 0;; base += 32 * U) {
      const bool more = base < n;
      if (more) {
        int jv[U];
        float4 pv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int m = base + 32 * u + lane + 1;
          jv[u] = m <= n ? sp[m] : -1;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) pv[u] = jv[u] >= 0 ? A.xhs[jv[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
        const unsigned lt = (1u << lane) - 1u;
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const float ex = pi.x - pv[u].x, ey = pi.y - pv[u].y, ez = pi.z - pv[u].z;
          const bool keep = jv[u] >= 0 && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= pg.f_pre;
          const unsigned b = __ballot_sync(0xffffffffu, keep);
          if (keep) pq[wq].j[nq + __popc(b & lt)] = jv[u];
          nq += __popc(b);
        }
        __syncwarp();
      }
      while (nq >= 32 || (!more && nq > 0)) {
        const int take = min(nq, 32);
        if (lane < take) {
          const int j = pq[wq].j[nq - take + lane];
          const float4 pj = A.xhs[j];
          float4 lj;
          int aj;
          if (MIXED) {
            pair_lo_type(A.xlh[j], lj.x, lj.y, lj.z, aj);
            lj.w = 0.f;
          } else {
            lj = A.xls[j];
            aj = A.tys[j];
          }
          long long ix = 0, iy = 0, iz = 0;
          bool hit;
          if (MIXED) {
            const float dx = (pi.x - pj.x) + (li.x - lj.x), dy = (pi.y - pj.y) + (li.y - lj.y),
                        dz = (pi.z - pj.z) + (li.z - lj.z);
            hit = pair_mixed_eval(A, s_lj, ljrow, aj, qi32, pj.w, dx, dy, dz, e4, ix, iy, iz);
          } else {
            const df ex = two_sum(pi.x, -pj.x), ey = two_sum(pi.y, -pj.y), ez = two_sum(pi.z, -pj.z);
            const df dx = quick_two_sum(ex.hi, __fadd_rn(ex.lo, __fsub_rn(li.x, lj.x)));
            const df dy = quick_two_sum(ey.hi, __fadd_rn(ey.lo, __fsub_rn(li.y, lj.y)));
            const df dz = quick_two_sum(ez.hi, __fadd_rn(ez.lo, __fsub_rn(li.z, lj.z)));
            const df rsq = df_norm2(dx, dy, dz);
            hit = rsq.hi <= pg.f_hi && pair_df64_eval(pg, A, s_etab, i, j, ai, aj, qi, qi_on, pj.w, lj.w, dx,
                                                      dy, dz, rsq, acc, ix, iy, iz);
          }
          if (hit) {
            ++n_rc;
            sx += ix; sy += iy; sz += iz;
            atomicAdd(&A.fixs[3 * (size_t)j + 0], (unsigned long long)(-ix));
            atomicAdd(&A.fixs[3 * (size_t)j + 1], (unsigned long long)(-iy));
            atomicAdd(&A.fixs[3 * (size_t)j + 2], (unsigned long long)(-iz));
          }
        }
        nq -= take;
        __syncwarp();  // the taken slots are read before the next pass appends over them
      }
      if (!more) break;
    }
    if (MIXED) {
#pragma unroll
      for (int q = 0; q < 4; ++q) dacc_add(acc[q], df_make(e4[q], 0.f));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
      sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    if (lane == 0) {
      atomicAdd(&A.fixs[3 * (size_t)p + 0], (unsigned long long)sx);
      atomicAdd(&A.fixs[3 * (size_t)p + 1], (unsigned long long)sy);
      atomicAdd(&A.fixs[3 * (size_t)p + 2], (unsigned long long)sz);
      n_list += (unsigned long long)n;
    }
  }
  dfr out[NACC_DF];
#pragma unroll
  for (int k = 0; k < NACC_DF; ++k) out[k] = to_dfr(two_sum(acc[k].s, acc[k].c));
  n_rc = (unsigned long long)warp_sumi((int)n_rc);
  if (lane == 0) {
    if (n_list) atomicAdd(&A.cnt[0], n_list);
    if (n_rc) atomicAdd(&A.cnt[1], n_rc);
  }
  block_reduce_store<NACC_DF>(out, A.blk);
}

// Pair stress from the per-sorted-position forces (sum over slots of x (x) F, every halo
// image at its own position, in FP64 from the exact fixed-point forces), then each
// slot's force onto its atom (a halo image's onto its source): integer sums.
__global__ void k_slot_stress_fold(int natms, const DevScalars* sc, const int* __restrict__ at_list,
                                   const int* __restrict__ src, const double* __restrict__ x,
                                   const double* __restrict__ y, const double* __restrict__ z,
                                   const long long* __restrict__ fixs, unsigned long long* fixp, double* blk) {
  const int nlast = sc->nlast;
  const double s = 1.0 / 1099511627776.0;
  double st[6] = {0, 0, 0, 0, 0, 0};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nlast; p += gridDim.x * blockDim.x) {
    const long long f0 = fixs[3 * (size_t)p], f1 = fixs[3 * (size_t)p + 1], f2 = fixs[3 * (size_t)p + 2];
    if ((f0 | f1 | f2) == 0) continue;
    const int a = at_list[p];
    const double fa = (double)f0 * s, fb = (double)f1 * s, fc = (double)f2 * s;
    const double xa = x[a], ya = y[a], za = z[a];
    st[0] = fma(xa, fa, st[0]); st[1] = fma(xa, fb, st[1]); st[2] = fma(xa, fc, st[2]);
    st[3] = fma(ya, fb, st[3]); st[4] = fma(ya, fc, st[4]); st[5] = fma(za, fc, st[5]);
    const int tgt = a < natms ? a : src[a];
    atomicAdd(&fixp[3 * tgt + 0], (unsigned long long)f0);
    atomicAdd(&fixp[3 * tgt + 1], (unsigned long long)f1);
    atomicAdd(&fixp[3 * tgt + 2], (unsigned long long)f2);
  }
  block_reduce_store<6>(st, blk);
}

// Pair stress of the double-float kernel from its per-slot forces: with every image's
// force kept in the image's own slot, sum over pairs of d (x) f = sum over slots of
// x (x) F (each pair's f enters its two slots with opposite signs, and d is the
// difference of the two slots' positions), summed in FP64 from the exact fixed-point
// forces.  Components xx, xy, xz, yy, yz, zz, as the per-pair sums of the FP64 kernels.
__global__ void k_pair_stress_fix(const DevScalars* sc, const double* __restrict__ x, const double* __restrict__ y,
                                  const double* __restrict__ z, const long long* __restrict__ fixp, double* blk) {
  const int nlast = sc->nlast;
  const double s = 1.0 / 1099511627776.0;
  double st[6] = {0, 0, 0, 0, 0, 0};
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < nlast; a += gridDim.x * blockDim.x) {
    const double fa = (double)fixp[3 * a] * s, fb = (double)fixp[3 * a + 1] * s, fc = (double)fixp[3 * a + 2] * s;
    const double xa = x[a], ya = y[a], za = z[a];
    st[0] = fma(xa, fa, st[0]); st[1] = fma(xa, fb, st[1]); st[2] = fma(xa, fc, st[2]);
    st[3] = fma(ya, fb, st[3]); st[4] = fma(ya, fc, st[4]); st[5] = fma(za, fc, st[5]);
  }
  block_reduce_store<6>(st, blk);
}

// image forces of the double-float kernel onto their source atoms (integer sums:
// the order of the atomics does not matter)
__global__ void k_fold_images(int natms, const DevScalars* sc, const int* __restrict__ src,
                              unsigned long long* fixp) {
  const int h = natms + blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= sc->nlast) return;
  const int i = src[h];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const unsigned long long v = fixp[3 * h + c];
    if (v) atomicAdd(&fixp[3 * i + c], v);
  }
}

// FP64 form: forces of the other terms are in fx; add the double-float pair kernel's
// fixed-point sums
__global__ void k_fix_add_fp64(int n, const long long* fixp, double* fx, double* fy, double* fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = 1.0 / 1099511627776.0;
  fx[i] += (double)fixp[3 * i] * s;
  fy[i] += (double)fixp[3 * i + 1] * s;
  fz[i] += (double)fixp[3 * i + 2] * s;
}

namespace {

// double-float cutoff bands, the FP32 prefilter bound and the split spacings
void pair_geom_df(PairGeom& pg) {
  pg.f_rc2_lo = (float)(pg.rc2 * (1.0 - 1e-6));
  pg.f_rc2_hi = (float)(pg.rc2 * (1.0 + 1e-6));
  pg.f_rv2_lo = (float)(pg.rv2 * (1.0 - 1e-6));
  pg.f_rv2_hi = (float)(pg.rv2 * (1.0 + 1e-6));
  pg.f_hi = std::max(pg.f_rc2_hi, pg.f_rv2_hi);
  // |x - (float)x| <= u for every coordinate: R = twice the summed cell-vector lengths
  // bounds the local atoms (reduced coordinates within +-(1/2 + drift)) and their halo
  // images (the halo is under half a cell wide)
  double R = 0.0;
  for (int v = 0; v < 3; ++v)
    R += std::sqrt(g.cell[3 * v] * g.cell[3 * v] + g.cell[3 * v + 1] * g.cell[3 * v + 1] +
                   g.cell[3 * v + 2] * g.cell[3 * v + 2]);
  R *= 2.0;
  const double u = std::ldexp(1.0, std::ilogb(R) - 23);
  const double eps = std::ldexp(1.0, -23);
  const double D = std::sqrt((double)pg.f_hi) + 1.0;
  const double dlt = 2.0 * u + eps * (D + 2.0 * u);  // error of a separation component
  const double band = 4.0 * (2.0 * std::sqrt(3.0) * D * dlt + 3.0 * dlt * dlt) + 8.0 * eps * D * D;
  pg.f_pre = std::nextafter((float)((double)pg.f_hi + band), 3.0e38f);
  df_split(pg.erdr, &pg.erdr_hi, &pg.erdr_lo);
  df_split(pg.vrdr, &pg.vrdr_hi, &pg.vrdr_lo);
  df_split(pg.scaling, &pg.scal_hi, &pg.scal_lo);
}

// The sorted-position pair kernels (both forms) with the exclusion correction; results
// into g.sc->acc like the per-atom kernels.
void pair_forces_sorted(PairGeom& pg, int nb2) {
  cudaStream_t st = g.stream;
  pair_geom_df(pg);
  const bool mixed = g.precision == GB_MIXED;
  PairSortedArgs A;
  A.natms = g.natms;
  A.at_list = g.at_list;
  A.loc_sp = g.loc_sp;
  A.list = g.list; A.ld = g.ld; A.spos = g.spos; A.ldt = g.ldt;
  A.xhs = g.xhs; A.xls = g.xls; A.tys = g.tys; A.xlh = g.xlh;
  A.x = g.x; A.y = g.y; A.z = g.z; A.q = g.chge;
  A.etab = g.erfc_df; A.vtab = g.vdw_df; A.ecoef = g.erfc_coef; A.vcoef = g.vdw_coef;
  A.netab = (g.nsamples + 1) * 3;
  A.vkind = g.vdw_kind; A.veps = g.vdw_eps; A.vsig = g.vdw_sig;
  A.ntypes = g.p.ntypes;
  A.rc2 = (float)pg.rc2; A.rv2 = (float)pg.rv2; A.alpha = (float)g.p.alpha;
  A.a2rp = (float)(g.p.alpha * 2.0 / std::sqrt(3.14159265358979323846264338327950288));
  A.scaling = (float)pg.scaling;
  A.fixs = (unsigned long long*)g.fixs;
  A.cnt = &g.sc->npairs_list;
  A.sc = g.sc;
  // four list entries per lane in the filter pass (measured at 262,144 ions, pair time
  // per launch for 1 / 2 / 4 entries: double-float 1.46 / 1.37 / 1.34 ms, mixed 0.81 /
  // 0.76 / 0.74 ms)
  void (*kern)(PairSortedArgs, PairGeom) = nullptr;
  int nt = PAIR_SORTED_NT;
  if (g.pair_nt == 256 || (g.pair_nt == 0 && mixed)) {
    nt = 256;
    kern = mixed ? k_pair_sorted<1, 4, 256> : k_pair_sorted<0, 4, 256>;
  } else {
    kern = mixed ? k_pair_sorted<1, 4, 1024> : k_pair_sorted<0, 4, 1024>;
  }
  // the FP64 form reads its erfc table from shared memory
  const size_t dsm = mixed ? 0 : sizeof(float4) * (size_t)A.netab;
  if (dsm > 0) GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm));
  int occ = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, nt, dsm));
  // The CTAs take equal contiguous runs of the local atoms: one resident set of CTAs
  // (the double-float form), or short-lived CTAs of 16 atoms per warp (the mixed form: they
  // retire through the step, so the side stream's SPME kernels take their places and the
  // last runs balance the load; measured at 262,144 ions, mixed pair 0.682 -> 0.646 ms and
  // step 1.481 -> 1.460 ms; for the double-float form they were slower at every length).
  // GB_PAIR_APW sets the atoms per warp (0: one resident set).
  int apw = mixed ? 16 : 0;
  if (g.pair_apw >= 0) apw = g.pair_apw;
  // a small system keeps at least one CTA per resident slot (fewer atoms per warp)
  if (apw > 0) apw = std::max(1, std::min(apw, g.natms / ((nt / 32) * std::max(1, occ) * g.nsm)));
  const int nb = apw > 0 ? std::max(1, nblocks((long long)g.natms, (nt / 32) * apw))
                         : std::max(1, std::min(nblocks((long long)g.mxatms * 32, nt), occ * g.nsm));
  const int nbs = std::max(1, std::min(nblocks(g.mxatms, 256), 4 * g.nsm));  // stress blocks
  double* blk = gb_blkacc(nb * NACC_DF + nbs * 6 + nb2 * 8);
  double* blks = blk + (size_t)nb * NACC_DF;
  double* blk2 = blks + (size_t)nbs * 6;
  A.blk = blk;
  GB_CUDA(cudaMemsetAsync(g.fixs, 0, sizeof(long long) * 3 * (size_t)g.mxatms, st));
  if (!mixed) GB_CUDA(cudaMemsetAsync(g.fixp, 0, sizeof(long long) * 3 * (size_t)g.mxatms, st));
  prof_begin(P_PAIR);
  kern<<<nb, nt, dsm, st>>>(A, pg);
  GB_LAUNCHED();
  run_side_hook();  // side-stream work enqueued behind the pair kernel's launch
  side_join();  // the reciprocal-space forces are in place before the pair forces join them
  k_slot_stress_fold<<<nbs, 256, 0, st>>>(g.natms, g.sc, g.at_list, g.src, g.x, g.y, g.z, g.fixs,
                                          (unsigned long long*)g.fixp, blks);
  GB_LAUNCHED();
  if (!mixed) {
    k_fix_add_fp64<<<nblocks(g.natms, 256), 256, 0, st>>>(g.natms, g.fixp, g.fx, g.fy, g.fz);
    GB_LAUNCHED();
  }
  prof_end(P_PAIR);
  gb_reduce_blocks(blk, nb, NACC_DF, &g.sc->acc[A_PAIR]);
  gb_reduce_blocks(blks, nbs, 6, &g.sc->acc[A_PAIR + NACC_DF]);
  if (g.lbook) {
    prof_begin(P_EXCL);
    k_excl_fp64<<<nb2, 128, 0, st>>>(g.natms, g.list, g.ld, g.x, g.y, g.z, g.chge, g.ltg, g.src, g.p.alpha,
                                     g.scaling, g.p.rcut, g.fx, g.fy, g.fz, blk2,
                                     mixed ? (unsigned long long*)g.fixp : nullptr);
    GB_LAUNCHED();
    prof_end(P_EXCL);
    gb_reduce_blocks(blk2, nb2, 8, &g.sc->acc[A_EXCL]);
  }
}

}  // namespace

// eng6: engrl, virrl, engex, virex, engvdw, virvdw; stress9 accumulates.
void pair_forces(double* eng6, double* stress9) {
  PairGeom pg;
  pg.rcut = g.p.rcut;
  pg.rvdw = g.p.rvdw;
  pg.rc2 = g.p.rcut * g.p.rcut;
  pg.rv2 = g.p.rvdw * g.p.rvdw;
  // decide sqrt(rsq) < rc exactly only inside a narrow band around rc^2
  pg.rc2_lo = pg.rc2 * (1.0 - 1e-12);
  pg.rc2_hi = std::max(pg.rc2, pg.rv2) * (1.0 + 1e-12);
  pg.rv2_lo = pg.rv2 * (1.0 - 1e-12);
  pg.rv2_hi = pg.rv2 * (1.0 + 1e-12);
  auto bits = [](double v) { long long b; std::memcpy(&b, &v, 8); return b; };
  pg.b_rc2_lo = bits(pg.rc2_lo);
  pg.b_rc2_hi = bits(pg.rc2 * (1.0 + 1e-12));
  pg.b_rv2_lo = bits(pg.rv2_lo);
  pg.b_rv2_hi = bits(pg.rv2_hi);
  pg.b_hi = bits(pg.rc2_hi);
  pg.erdr = g.erfc_rdr;
  pg.vrdr = g.vdw_rdr;
  pg.scaling = g.scaling;
  pg.vdw_direct = g.p.vdw_direct;
  pg.same_grid = (g.erfc_rdr == g.vdw_rdr) ? 1 : 0;
  pg.nsamples = g.nsamples;
  pg.max_grid = g.max_grid;
  pg.ntypes = g.p.ntypes;
  cudaStream_t st = g.stream;
  const int T = 256;
  const int nb2 = nblocks(g.natms, 128);
  GB_CUDA(cudaMemsetAsync(&g.sc->npairs_list, 0, 2 * sizeof(unsigned long long), st));
  const bool sorted = g.spos_valid && g.use_sorted && !(g.precision == GB_FP64 && g.fp64_native);
  if (!sorted) {  // the atom-index kernels write the force arrays directly
    run_side_hook();
    side_join();
  }
  if (sorted) {
    pair_forces_sorted(pg, nb2);
  } else if (g.precision == GB_FP64 && !g.fp64_native) {
    // double-float bands and spacings
    pg.f_rc2_lo = (float)(pg.rc2 * (1.0 - 1e-6));
    pg.f_rc2_hi = (float)(pg.rc2 * (1.0 + 1e-6));
    pg.f_rv2_lo = (float)(pg.rv2 * (1.0 - 1e-6));
    pg.f_rv2_hi = (float)(pg.rv2 * (1.0 + 1e-6));
    pg.f_hi = std::max(pg.f_rc2_hi, pg.f_rv2_hi);
    {
      // |x - (float)x| <= u for every coordinate: R = twice the summed cell-vector
      // lengths bounds the local atoms (reduced coordinates within +-(1/2 + drift)) and
      // their halo images (the halo is under half a cell wide)
      double R = 0.0;
      for (int v = 0; v < 3; ++v)
        R += std::sqrt(g.cell[3 * v] * g.cell[3 * v] + g.cell[3 * v + 1] * g.cell[3 * v + 1] +
                       g.cell[3 * v + 2] * g.cell[3 * v + 2]);
      R *= 2.0;
      const double u = std::ldexp(1.0, std::ilogb(R) - 23);
      const double eps = std::ldexp(1.0, -23);
      const double D = std::sqrt((double)pg.f_hi) + 1.0;
      const double dlt = 2.0 * u + eps * (D + 2.0 * u);  // error of a separation component
      const double band = 4.0 * (2.0 * std::sqrt(3.0) * D * dlt + 3.0 * dlt * dlt) + 8.0 * eps * D * D;
      pg.f_pre = std::nextafter((float)((double)pg.f_hi + band), 3.0e38f);
    }
    df_split(pg.erdr, &pg.erdr_hi, &pg.erdr_lo);
    df_split(pg.vrdr, &pg.vrdr_hi, &pg.vrdr_lo);
    df_split(pg.scaling, &pg.scal_hi, &pg.scal_lo);
    static int occdf = 0;
    if (!occdf) GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occdf, k_pair_df64, PAIR_DF_NT, 0));
    int nb = std::max(1, std::min(nblocks((long long)g.mxatms * 32, PAIR_DF_NT), occdf * g.nsm));
    const int nbs = std::max(1, std::min(nblocks(g.mxatms, 256), 4 * g.nsm));  // stress blocks
    double* blk = gb_blkacc(nb * NACC + nb2 * 8 + nbs * 6);
    double* blks = blk + (size_t)nb * NACC + (size_t)nb2 * 8;
    // local atoms and halo images: an image's force is folded onto its source after the stress sum
    GB_CUDA(cudaMemsetAsync(g.fixp, 0, sizeof(long long) * 3 * (size_t)g.mxatms, st));
    prof_begin(P_PAIR);
    k_pair_df64<<<nb, PAIR_DF_NT, 0, st>>>(g.natms, g.sc, g.at_list, g.list, g.ld, g.xf, g.xlo, g.qdf, g.x, g.y, g.z, g.chge,
                                  g.ltg, g.src, g.erfc_df, g.vdw_df, g.erfc_coef, g.vdw_coef, g.vdw_kind, g.vdw_eps,
                                  g.vdw_sig, pg, (unsigned long long*)g.fixp, blk, &g.sc->npairs_list);
    GB_LAUNCHED();
    k_pair_stress_fix<<<nbs, 256, 0, st>>>(g.sc, g.x, g.y, g.z, g.fixp, blks);
    GB_LAUNCHED();
    k_fold_images<<<std::max(1, nblocks(g.mxatms - g.natms, 256)), 256, 0, st>>>(g.natms, g.sc, g.src,
                                                                    (unsigned long long*)g.fixp);
    GB_LAUNCHED();
    k_fix_add_fp64<<<nblocks(g.natms, 256), 256, 0, st>>>(g.natms, g.fixp, g.fx, g.fy, g.fz);
    GB_LAUNCHED();
    prof_end(P_PAIR);
    gb_reduce_blocks(blk, nb, NACC_DF, &g.sc->acc[A_PAIR]);
    gb_reduce_blocks(blks, nbs, 6, &g.sc->acc[A_PAIR + NACC_DF]);
    if (g.lbook) {
      double* blk2 = blk + (size_t)nb * NACC;
      prof_begin(P_EXCL);
      k_excl_fp64<<<nb2, 128, 0, st>>>(g.natms, g.list, g.ld, g.x, g.y, g.z, g.chge, g.ltg, g.src, g.p.alpha,
                                       g.scaling, g.p.rcut, g.fx, g.fy, g.fz, blk2, nullptr);
      GB_LAUNCHED();
      prof_end(P_EXCL);
      gb_reduce_blocks(blk2, nb2, 8, &g.sc->acc[A_EXCL]);
    }
  } else if (g.precision == GB_FP64) {
    static int occ64 = 0;
    if (!occ64) GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, k_pair_fp64, T, 0));
    int nb = std::max(1, std::min(nblocks((long long)g.mxatms * 32, T), occ64 * g.nsm));
    double* blk = gb_blkacc(nb * NACC + nb2 * 8);
    prof_begin(P_PAIR);
    k_pair_fp64<<<nb, T, 0, st>>>(g.natms, g.sc, g.at_list, g.list, g.ld, g.x, g.y, g.z, g.chge, g.ltype, g.ltg,
                                  g.src, g.erfc_coef, g.vdw_coef, g.vdw_kind, g.vdw_eps, g.vdw_sig, pg, g.fx, g.fy,
                                  g.fz, blk, &g.sc->npairs_list);
    GB_LAUNCHED();
    prof_end(P_PAIR);
    gb_reduce_blocks(blk, nb, NACC, &g.sc->acc[A_PAIR]);
    if (g.lbook) {
      double* blk2 = blk + (size_t)nb * NACC;
      prof_begin(P_EXCL);
      k_excl_fp64<<<nb2, 128, 0, st>>>(g.natms, g.list, g.ld, g.x, g.y, g.z, g.chge, g.ltg, g.src, g.p.alpha,
                                       g.scaling, g.p.rcut, g.fx, g.fy, g.fz, blk2, nullptr);
      GB_LAUNCHED();
      prof_end(P_EXCL);
      gb_reduce_blocks(blk2, nb2, 8, &g.sc->acc[A_EXCL]);
    }
  } else {
    static int occ32 = 0;
    if (!occ32) GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ32, k_pair_mixed_half, T, 0));
    int nb = std::max(1, std::min(nblocks((long long)g.mxatms * 32, T), occ32 * g.nsm));
    double* blk = gb_blkacc(nb * NACC + nb2 * 8);
    prof_begin(P_PAIR);
    const double a2rp = g.p.alpha * 2.0 / std::sqrt(3.14159265358979323846264338327950288);
    k_pair_mixed_half<<<nb, T, 0, st>>>(g.natms, g.sc, g.at_list, g.list, g.ld, g.xf, g.xlo, g.ltype, g.ltg, g.src,
                                        g.p.ntypes, (float)pg.rc2, (float)pg.rv2, (float)g.p.alpha, (float)a2rp,
                                        (float)pg.scaling, (unsigned long long*)g.fixp, blk, &g.sc->npairs_list);
    GB_LAUNCHED();
    prof_end(P_PAIR);
    gb_reduce_blocks(blk, nb, NACC, &g.sc->acc[A_PAIR]);
    if (g.lbook) {
      double* blk2 = blk + (size_t)nb * NACC;
      prof_begin(P_EXCL);
      k_excl_fp64<<<nb2, 128, 0, st>>>(g.natms, g.list, g.ld, g.x, g.y, g.z, g.chge, g.ltg, g.src, g.p.alpha,
                                       g.scaling, g.p.rcut, g.fx, g.fy, g.fz, blk2, (unsigned long long*)g.fixp);
      GB_LAUNCHED();
      prof_end(P_EXCL);
      gb_reduce_blocks(blk2, nb2, 8, &g.sc->acc[A_EXCL]);
    }
  }
  if (g.defer_scalars) return;  // the MD loop reads the sums after its last step
  gb_sync_scalars();
  pair_scalars(g.hsc, eng6, stress9);
}

// engrl, virrl, engex, virex, engvdw, virvdw and the pair stress from the device sums
void pair_scalars(const DevScalars* h, double* eng6, double* stress9) {
  double res[NACC];
  double ex[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < NACC; ++k) res[k] = h->acc[A_PAIR + k];
  if (g.lbook) for (int k = 0; k < 8; ++k) ex[k] = h->acc[A_EXCL + k];
  eng6[0] = res[2]; eng6[1] = res[3];
  eng6[2] = ex[0]; eng6[3] = ex[1];
  eng6[4] = res[0]; eng6[5] = res[1];
  double s6[6];
  for (int k = 0; k < 6; ++k) s6[k] = res[4 + k] + ex[2 + k];
  stress9[0] += s6[0]; stress9[1] += s6[1]; stress9[2] += s6[2];
  stress9[3] += s6[1]; stress9[4] += s6[3]; stress9[5] += s6[4];
  stress9[6] += s6[2]; stress9[7] += s6[4]; stress9[8] += s6[5];
}
