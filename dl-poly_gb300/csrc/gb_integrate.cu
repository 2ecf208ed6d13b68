// gb_integrate.cu - NVE velocity Verlet, SHAKE/RATTLE, kinetic stress and the
// Verlet-list displacement check on the device.
//
// Follows:
//   nve_0_vv            source/nve.F90:38-235 (stage 1 :131-174, stage 2 :198-217)
//   constraints_tags    source/constraints.F90:438-586
//   constraints_shake_vv source/constraints.F90:777-1030, apply_shake :1071-1200
//   constraints_rattle  source/constraints.F90:587-775, apply_rattle :1032-1069
//   kinstress           source/kinetics.F90:218-262
//   vnl_check           source/neighbours.F90:123-296
// SHAKE and RATTLE are Jacobi iterations with one global convergence test per
// sweep, exactly as the reference: a cooperative-grid kernel runs the sweeps
// with grid-wide barriers, at most shake_maxit of them, and returns the
// iteration count and a status bit instead of spinning.  Per-atom corrections
// are summed in constraint order from a per-atom constraint table, and applied
// listot(i) times, so positions round as the reference's do.
#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>
#include <cstdlib>

#include "gb_common.cuh"

namespace cg = cooperative_groups;

namespace {

inline int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ double image1(double d, double c, double a) {
  // images, cubic branch (numerics.F90:1527-1532): d - c*Anint(a*d)
  return sub_rn(d, mul_rn(c, round(mul_rn(a, d))));
}

// Velocity Verlet stages (nve.F90:127-217).  hdw[i] = (tstep/2) / weight(i), formed once
// with the same correctly rounded division the reference performs each step, and 0 for
// an atom with weight <= 1e-6 (which the stages skip): the stages then read one array
// instead of dividing on the FP64 unit.
__global__ void k_vv1(int n, const double* __restrict__ hdw, double tstep, const double* __restrict__ fx,
                      const double* __restrict__ fy, const double* __restrict__ fz, double* vx, double* vy, double* vz,
                      double* x, double* y, double* z) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double tmp = hdw[i];
  if (tmp > 0.0) {
    vx[i] = vx[i] + tmp * fx[i];
    vy[i] = vy[i] + tmp * fy[i];
    vz[i] = vz[i] + tmp * fz[i];
    x[i] = x[i] + tstep * vx[i];
    y[i] = y[i] + tstep * vy[i];
    z[i] = z[i] + tstep * vz[i];
  }
}

__global__ void k_vv2(int n, const double* __restrict__ hdw, const double* __restrict__ fx,
                      const double* __restrict__ fy, const double* __restrict__ fz, double* vx, double* vy,
                      double* vz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double tmp = hdw[i];
  if (tmp > 0.0) {
    vx[i] = vx[i] + tmp * fx[i];
    vy[i] = vy[i] + tmp * fy[i];
    vz[i] = vz[i] + tmp * fz[i];
  }
}

// m v (x) v summed over the atoms (kinetics.F90:218-262): a grid-stride loop, so each
// thread reduces its own atoms in registers and the FP64 block reduction runs once per
// thread rather than once per atom (the FP64 unit bounds this kernel)
__global__ void k_kinstress(int n, const double* w, const int* lfrzn, const double* vx, const double* vy,
                            const double* vz, double* blk) {
  double a[6] = {0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (lfrzn[i] != 0) continue;
    const double m = w[i], u = vx[i], v = vy[i], t = vz[i];
    a[0] += m * u * u; a[1] += m * u * v; a[2] += m * u * t;
    a[3] += m * v * v; a[4] += m * v * t; a[5] += m * t * t;
  }
  block_reduce_store<6>(a, blk);
}

// largest |r - r_checkpoint|^2 with minimum image, over a grid-stride loop; the caller takes
// the square root of the maximum (the square root is monotone and correctly rounded, so
// it equals the largest of the per-atom square roots); doubles >= 0 order as their bits
__global__ void k_maxdisp(int n, const double* x, const double* y, const double* z, const double* xb,
                          const double* yb, const double* zb, double c0, double a0, unsigned long long* out) {
  double r2 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double dx = image1(x[i] - xb[i], c0, a0), dy = image1(y[i] - yb[i], c0, a0),
                 dz = image1(z[i] - zb[i], c0, a0);
    r2 = fmax(r2, dx * dx + dy * dy + dz * dz);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r2 = fmax(r2, __shfl_xor_sync(0xffffffffu, r2, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(r2));
}

__global__ void k_zero3(int n, double* a, double* b, double* c) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { a[i] = 0.0; b[i] = 0.0; c[i] = 0.0; }
}

__global__ void k_fix_to_fp64(int n, const long long* fixp, double* fx, double* fy, double* fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = 1.0 / 1099511627776.0;
  fx[i] = (double)fixp[3 * i] * s;
  fy[i] = (double)fixp[3 * i + 1] * s;
  fz[i] = (double)fixp[3 * i + 2] * s;
}

// constraints_tags: bond vectors at the start of the stage (min image)
__global__ void k_con_tags(int nc, const int* ci, const int* cj, const double* x, const double* y, const double* z,
                           double c0, double a0, double* dxx, double* dyy, double* dzz) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  int i = ci[k], j = cj[k];
  dxx[k] = image1(x[i] - x[j], c0, a0);
  dyy[k] = image1(y[i] - y[j], c0, a0);
  dzz[k] = image1(z[i] - z[j], c0, a0);
}

struct ConArgs {
  int nc, natms, maxit;
  const int *ci, *cj, *listot, *astart, *alist, *lfrzn;
  const double* d0;
  double *dxx, *dyy, *dzz, *dxt, *dyt, *dzt, *dt2, *gam;
  double *x, *y, *z, *vx, *vy, *vz;
  const double* w;
  double tstep, tol, c0, a0;
  int* flags;      // maxit+1 ints, zeroed
  DevScalars* sc;
  double* blk;     // per-block stress partials (6)
};

// constraints_shake_vv: Jacobi sweeps until every |d^2 - d0^2|/2 < tol*d0
__global__ void k_shake(ConArgs A) {
  cg::grid_group grid = cg::this_grid();
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  const double tstep2 = A.tstep * A.tstep;
  double st[6] = {0, 0, 0, 0, 0, 0};
  int it = 0;
  bool safe = false;
  while (!safe && it < A.maxit) {
    ++it;
    for (int k = tid; k < A.nc; k += nth) {
      int i = A.ci[k], j = A.cj[k];
      double dx = image1(A.x[i] - A.x[j], A.c0, A.a0);
      double dy = image1(A.y[i] - A.y[j], A.c0, A.a0);
      double dz = image1(A.z[i] - A.z[j], A.c0, A.a0);
      A.dxt[k] = dx; A.dyt[k] = dy; A.dzt[k] = dz;
      double d0 = A.d0[k];
      double d2 = dx * dx + dy * dy + dz * dz - d0 * d0;
      A.dt2[k] = d2;
      if (!(0.5 * fabs(d2) < A.tol * d0)) A.flags[it] = 1;
    }
    grid.sync();
    safe = (A.flags[it] == 0);
    if (!safe) {
      for (int k = tid; k < A.nc; k += nth) {
        int i = A.ci[k], j = A.cj[k];
        double amti = tstep2 / A.w[i], amtj = tstep2 / A.w[j];
        if (A.lfrzn[i] != 0) amti = 0.0;
        if (A.lfrzn[j] != 0) amtj = 0.0;
        double gamma = A.dt2[k] / ((amti + amtj) * (A.dxx[k] * A.dxt[k] + A.dyy[k] * A.dyt[k] + A.dzz[k] * A.dzt[k]));
        A.gam[k] = gamma;
        st[0] -= gamma * A.dxx[k] * A.dxx[k]; st[1] -= gamma * A.dxx[k] * A.dyy[k];
        st[2] -= gamma * A.dxx[k] * A.dzz[k]; st[3] -= gamma * A.dyy[k] * A.dyy[k];
        st[4] -= gamma * A.dyy[k] * A.dzz[k]; st[5] -= gamma * A.dzz[k] * A.dzz[k];
      }
      grid.sync();
      for (int i = tid; i < A.natms; i += nth) {
        const int s = A.astart[i], e = A.astart[i + 1];
        if (s == e || A.lfrzn[i] != 0) continue;
        double xt = 0.0, yt = 0.0, zt = 0.0;
        const double amt = tstep2 / A.w[i];
        for (int t = s; t < e; ++t) {
          int code = A.alist[t];
          int k = code >> 1;
          double g = A.gam[k];
          double f = (code & 1) ? 0.5 * g * amt : -0.5 * g * amt;
          xt += A.dxx[k] * f; yt += A.dyy[k] * f; zt += A.dzz[k] * f;
        }
        const double dli = 1.0 / (double)A.listot[i];
        double px = A.x[i], py = A.y[i], pz = A.z[i];
        for (int r = 0; r < A.listot[i]; ++r) { px += xt * dli; py += yt * dli; pz += zt * dli; }
        A.x[i] = px; A.y[i] = py; A.z[i] = pz;
      }
      grid.sync();
    }
  }
  if (tid == 0) {
    A.sc->shake_iters = it;
    if (!safe) A.sc->status |= ST_SHAKE_FAIL;
  }
  block_reduce_store<6>(st, A.blk);
}

// constraints_rattle: normalise the bond vectors, then Jacobi sweeps on v
__global__ void k_rattle(ConArgs A) {
  cg::grid_group grid = cg::this_grid();
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  for (int k = tid; k < A.nc; k += nth) {
    double dis = 1.0 / sqrt(A.dxx[k] * A.dxx[k] + A.dyy[k] * A.dyy[k] + A.dzz[k] * A.dzz[k]);
    A.dxx[k] *= dis; A.dyy[k] *= dis; A.dzz[k] *= dis;
  }
  grid.sync();
  int it = 0;
  bool safe = false;
  while (!safe && it < A.maxit) {
    ++it;
    for (int k = tid; k < A.nc; k += nth) {
      int i = A.ci[k], j = A.cj[k];
      double amti = A.tstep / A.w[i], amtj = A.tstep / A.w[j];
      if (A.lfrzn[i] != 0) amti = 0.0;
      if (A.lfrzn[j] != 0) amtj = 0.0;
      double gamma = A.dxx[k] * (A.vx[i] - A.vx[j]) + A.dyy[k] * (A.vy[i] - A.vy[j]) + A.dzz[k] * (A.vz[i] - A.vz[j]);
      if (!(0.5 * A.tstep * fabs(gamma) < A.tol)) A.flags[it] = 1;
      A.gam[k] = gamma / (amti + amtj);
    }
    grid.sync();
    safe = (A.flags[it] == 0);
    if (!safe) {
      for (int i = tid; i < A.natms; i += nth) {
        const int s = A.astart[i], e = A.astart[i + 1];
        if (s == e || A.lfrzn[i] != 0) continue;
        double xt = 0.0, yt = 0.0, zt = 0.0;
        const double amt = A.tstep / A.w[i];
        for (int t = s; t < e; ++t) {
          int code = A.alist[t];
          int k = code >> 1;
          double g = A.gam[k];
          double f = (code & 1) ? g * amt : -g * amt;
          xt += A.dxx[k] * f; yt += A.dyy[k] * f; zt += A.dzz[k] * f;
        }
        const double dli = 1.0 / (double)A.listot[i];
        double px = A.vx[i], py = A.vy[i], pz = A.vz[i];
        for (int r = 0; r < A.listot[i]; ++r) { px += xt * dli; py += yt * dli; pz += zt * dli; }
        A.vx[i] = px; A.vy[i] = py; A.vz[i] = pz;
      }
      grid.sync();
    }
  }
  if (tid == 0) {
    A.sc->rattle_iters = it;
    if (!safe) A.sc->status |= ST_RATTLE_FAIL;
  }
}

// ------------------------------------------------- cluster-local SHAKE/RATTLE
// When every connected group of constraints (a "cluster": a rigid water, a
// small molecule) has at most CL_MAXA atoms and CL_MAXC constraints, the
// Jacobi sweeps of different clusters are independent: sweep `it` of a cluster
// reads only that cluster's atoms.  One thread then owns a cluster and runs
// its sweeps in registers; the only global quantity is the convergence test,
// "every constraint of every cluster passes at sweep it".  Sweeps run in
// chunks of CL_CHUNK: each cluster records the sweeps at which it fails in a
// per-sweep flag word and applies every update of the chunk, saving the state
// after each sweep in a per-cluster ring; one grid barrier per chunk then gives
// the first sweep N at which nobody failed, and each cluster keeps the state
// saved after sweep N-1.  Every update uses the per-sweep kernel's arithmetic,
// so the result and the iteration count are those of the reference's global
// sweeps (constraints.F90:898-969 and 1032-1071).
//
// FP64 instructions are expensive on this part, so tests that need no
// arithmetic are done on the IEEE bit patterns: the minimum image of a bond
// shorter than a quarter cell is the bond itself (round(d/L) = 0 exactly), and
// the tolerance tests 0.5|x| < t are |x| < 2t, an integer compare of the
// magnitudes' bits.
constexpr int CL_MAXA = 4, CL_MAXC = 6, CL_CHUNK = 8;
constexpr int CL_RING = CL_CHUNK + 1;       // state at chunk start + after each sweep
constexpr int CL_SLOT = 3 * CL_MAXA + CL_MAXC;  // doubles per ring slot: state, then sweep gammas

struct ClusterTab {
  int atom[CL_MAXA];   // global atom ids, -1 padding
  int con[CL_MAXC];    // global constraint ids in ascending order, -1 padding
  int pair[CL_MAXC];   // local ends: li | lj << 4
  int alist[CL_MAXA];  // per local atom: count | entries (local constraint << 1 | j end) in 4-bit fields from bit 4
  int meta;            // na | nc << 4
};

__device__ __forceinline__ void warp_flag(bool fail, int* flag) {
  const unsigned m = __activemask();
  const unsigned b = __ballot_sync(m, fail);
  if (b && (threadIdx.x & 31) == __ffs(m) - 1) atomicOr(flag, 1);
}

__device__ __forceinline__ long long absbits(double v) { return __double_as_longlong(v) & 0x7fffffffffffffffll; }

// d - c*Anint(a*d), skipping the FP64 work when |d| < quarter (bits) makes the shift zero
__device__ __forceinline__ double image_short(double d, long long quarter_bits, double c, double a) {
  if (absbits(d) < quarter_bits) return d;
  return image1(d, c, a);
}

// register-array reads with a runtime index, as selects (no local-memory copy)
template <int N>
__device__ __forceinline__ double sel(const double (&a)[N], int i) {
  double r = a[0];
#pragma unroll
  for (int k = 1; k < N; ++k) r = (i == k) ? a[k] : r;
  return r;
}

// per-cluster constants and state (positions for SHAKE, velocities for RATTLE)
template <int MA, int MC>
struct ClData {
  int na, nc;
  double x[MA], y[MA], z[MA];
  double bx[MC], by[MC], bz[MC];
  double d0sq[MC];          // SHAKE: d0^2
  long long tolb[MC];       // bits of the tolerance bound on |d2| (SHAKE) or |gamma| (RATTLE)
  double msum[MC];          // amt_i + amt_j
  double hm[MA];            // per-atom update factor: 0.5 amt (SHAKE) or amt (RATTLE)
  double dli[MA];           // 1 / listot
  bool active[MA];          // has constraints and is not frozen
};

template <int MA, int MC>
__device__ __forceinline__ void cl_load(const ConArgs& A, const ClusterTab& T, bool rattle, ClData<MA, MC>& D) {
  D.na = T.meta & 15;
  D.nc = (T.meta >> 4) & 15;
  const double amt_num = rattle ? A.tstep : A.tstep * A.tstep;
  double amt[MA];
#pragma unroll
  for (int a = 0; a < MA; ++a) {
    D.x[a] = D.y[a] = D.z[a] = 0.0;
    amt[a] = 0.0; D.hm[a] = 0.0; D.dli[a] = 1.0; D.active[a] = false;
    if (a < D.na) {
      const int i = T.atom[a];
      if (rattle) { D.x[a] = A.vx[i]; D.y[a] = A.vy[i]; D.z[a] = A.vz[i]; }
      else { D.x[a] = A.x[i]; D.y[a] = A.y[i]; D.z[a] = A.z[i]; }
      const bool frz = A.lfrzn[i] != 0;
      amt[a] = frz ? 0.0 : amt_num / A.w[i];
      const int cnt = T.alist[a] & 15;
      D.active[a] = !frz && cnt > 0;
      D.hm[a] = rattle ? amt[a] : 0.5 * amt[a];
      D.dli[a] = 1.0 / (double)(cnt > 0 ? cnt : 1);
    }
  }
#pragma unroll
  for (int c = 0; c < MC; ++c) {
    D.bx[c] = D.by[c] = D.bz[c] = 0.0; D.d0sq[c] = 0.0; D.tolb[c] = 0; D.msum[c] = 1.0;
    if (c < D.nc) {
      const int k = T.con[c];
      const int li = T.pair[c] & 15, lj = T.pair[c] >> 4;
      double ux = A.dxx[k], uy = A.dyy[k], uz = A.dzz[k];
      if (rattle) {
        const double dis = 1.0 / sqrt(ux * ux + uy * uy + uz * uz);
        ux *= dis; uy *= dis; uz *= dis;
        // 0.5 tstep |gamma| < tol  <=>  |gamma| < (2 tol) / tstep, evaluated as the kernel does: 0.5*tstep*|g| < tol
        D.tolb[c] = 0;  // unused: RATTLE keeps the FP64 comparison (tstep scaling is not exact)
      } else {
        const double d0 = A.d0[k];
        D.d0sq[c] = d0 * d0;
        D.tolb[c] = __double_as_longlong(2.0 * (A.tol * d0));  // 0.5|d2| < tol d0  <=>  |d2| < 2 (tol d0)
      }
      D.bx[c] = ux; D.by[c] = uy; D.bz[c] = uz;
      D.msum[c] = sel(amt, li) + sel(amt, lj);
    }
  }
}

// one sweep: tests (returns true when a constraint fails), gammas, update of the state
template <int MA, int MC>
__device__ __forceinline__ bool cl_sweep(const ConArgs& A, const ClusterTab& T, bool rattle, long long quarter,
                                         ClData<MA, MC>& D, double (&gam)[MC]) {
  bool fail = false;
#pragma unroll
  for (int c = 0; c < MC; ++c) {
    gam[c] = 0.0;
    if (c < D.nc) {
      const int li = T.pair[c] & 15, lj = T.pair[c] >> 4;
      if (rattle) {
        const double gamma = D.bx[c] * (sel(D.x, li) - sel(D.x, lj)) + D.by[c] * (sel(D.y, li) - sel(D.y, lj)) +
                             D.bz[c] * (sel(D.z, li) - sel(D.z, lj));
        if (!(0.5 * A.tstep * fabs(gamma) < A.tol)) fail = true;
        gam[c] = gamma / D.msum[c];
      } else {
        const double dx = image_short(sel(D.x, li) - sel(D.x, lj), quarter, A.c0, A.a0);
        const double dy = image_short(sel(D.y, li) - sel(D.y, lj), quarter, A.c0, A.a0);
        const double dz = image_short(sel(D.z, li) - sel(D.z, lj), quarter, A.c0, A.a0);
        const double d2 = dx * dx + dy * dy + dz * dz - D.d0sq[c];
        if (!(absbits(d2) < D.tolb[c])) fail = true;
        gam[c] = d2 / (D.msum[c] * (D.bx[c] * dx + D.by[c] * dy + D.bz[c] * dz));
      }
    }
  }
#pragma unroll
  for (int a = 0; a < MA; ++a) {
    if (!D.active[a]) continue;
    const int al = T.alist[a], cnt = al & 15;
    double xt = 0.0, yt = 0.0, zt = 0.0;
#pragma unroll
    for (int e = 0; e < MC; ++e) {
      if (e < cnt) {
        const int code = (al >> (4 + 4 * e)) & 15, c = code >> 1;
        const double gh = sel(gam, c) * D.hm[a];
        const double f = (code & 1) ? gh : -gh;
        xt += sel(D.bx, c) * f; yt += sel(D.by, c) * f; zt += sel(D.bz, c) * f;
      }
    }
    double px = D.x[a], py = D.y[a], pz = D.z[a];
    for (int r = 0; r < cnt; ++r) { px += xt * D.dli[a]; py += yt * D.dli[a]; pz += zt * D.dli[a]; }
    D.x[a] = px; D.y[a] = py; D.z[a] = pz;
  }
  return fail;
}

template <int MA, int MC>
__device__ __forceinline__ void ring_put(double* slot, const ClData<MA, MC>& D, const double (&gam)[MC]) {
#pragma unroll
  for (int a = 0; a < MA; ++a) { slot[3 * a] = D.x[a]; slot[3 * a + 1] = D.y[a]; slot[3 * a + 2] = D.z[a]; }
#pragma unroll
  for (int c = 0; c < MC; ++c) slot[3 * CL_MAXA + c] = gam[c];
}

// SHAKE (rattle = false) or RATTLE (rattle = true) over all clusters; gsum
// (MC doubles per cluster) holds the committed gamma sums of SHAKE for
// the constraint stress
template <int MA, int MC>
__global__ void __launch_bounds__(128) k_constrain_cl(ConArgs A, const ClusterTab* __restrict__ tabs, int ncl,
                                                      double* __restrict__ ring, double* __restrict__ gsum,
                                                      int rattle_i) {
  cg::grid_group grid = cg::this_grid();
  const bool rattle = rattle_i != 0;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  const long long quarter = __double_as_longlong(0.25 * A.c0);
  int it0 = 0, nfinal = -1;
  for (;;) {
    for (int cl = tid; cl < ncl; cl += nth) {
      const ClusterTab T = tabs[cl];
      ClData<MA, MC> D;
      cl_load(A, T, rattle, D);
      double* rg = ring + (size_t)cl * CL_RING * CL_SLOT;
      double gam[MC];
#pragma unroll
      for (int c = 0; c < MC; ++c) gam[c] = 0.0;
      ring_put(rg, D, gam);
      for (int s_ = 1; s_ <= CL_CHUNK; ++s_) {
        if (it0 + s_ > A.maxit) break;
        const bool fail = cl_sweep(A, T, rattle, quarter, D, gam);
        warp_flag(fail, &A.flags[it0 + s_]);
        ring_put(rg + s_ * CL_SLOT, D, gam);
      }
    }
    grid.sync();
    for (int s_ = 1; s_ <= CL_CHUNK && it0 + s_ <= A.maxit; ++s_)
      if (A.flags[it0 + s_] == 0) { nfinal = it0 + s_; break; }
    // committed sweeps of this chunk: all of them, or those before nfinal
    const int last = nfinal > 0 ? nfinal - 1 - it0 : (A.maxit - it0 < CL_CHUNK ? A.maxit - it0 : CL_CHUNK);
    for (int cl = tid; cl < ncl; cl += nth) {
      const ClusterTab T = tabs[cl];
      const int na = T.meta & 15, nc = (T.meta >> 4) & 15;
      const double* rg = ring + (size_t)cl * CL_RING * CL_SLOT;
      const double* fin = rg + last * CL_SLOT;
#pragma unroll
      for (int a = 0; a < MA; ++a) {
        if (a < na) {
          const int i = T.atom[a];
          if (rattle) { A.vx[i] = fin[3 * a]; A.vy[i] = fin[3 * a + 1]; A.vz[i] = fin[3 * a + 2]; }
          else { A.x[i] = fin[3 * a]; A.y[i] = fin[3 * a + 1]; A.z[i] = fin[3 * a + 2]; }
        }
      }
      if (!rattle) {
        for (int s_ = 1; s_ <= last; ++s_)
#pragma unroll
          for (int c = 0; c < MC; ++c)
            if (c < nc) gsum[(size_t)cl * CL_MAXC + c] += rg[s_ * CL_SLOT + 3 * CL_MAXA + c];
      }
    }
    if (nfinal > 0) break;
    it0 += CL_CHUNK;
    if (it0 >= A.maxit) break;
    // no barrier needed here: a cluster is always handled by the same thread
  }
  if (tid == 0) {
    if (rattle) {
      A.sc->rattle_iters = nfinal > 0 ? nfinal : A.maxit;
      if (nfinal < 0) A.sc->status |= ST_RATTLE_FAIL;
    } else {
      A.sc->shake_iters = nfinal > 0 ? nfinal : A.maxit;
      if (nfinal < 0) A.sc->status |= ST_SHAKE_FAIL;
    }
  }
  if (!rattle) {
    // constraint stress: every committed update adds -gamma b b^T, b fixed during SHAKE
    double st[6] = {0, 0, 0, 0, 0, 0};
    for (int cl = tid; cl < ncl; cl += nth) {
      const ClusterTab T = tabs[cl];
      const int nc = (T.meta >> 4) & 15;
#pragma unroll
      for (int c = 0; c < MC; ++c) {
        if (c >= nc) continue;
        const int k = T.con[c];
        const double g = gsum[(size_t)cl * CL_MAXC + c];
        const double bx = A.dxx[k], by = A.dyy[k], bz = A.dzz[k];
        st[0] -= g * bx * bx; st[1] -= g * bx * by; st[2] -= g * bx * bz;
        st[3] -= g * by * by; st[4] -= g * by * bz; st[5] -= g * bz * bz;
      }
    }
    block_reduce_store<6>(st, A.blk);
  }
}

// apply_shake epilogue: v += dr/dt, f += dr/dt * m/(dt/2) for constrained atoms
__global__ void k_shake_post(int n, const int* astart, const int* lfrzn, double rstep, double hstep, const double* w,
                             const double* x, const double* y, const double* z, const double* ox, const double* oy,
                             const double* oz, double* vx, double* vy, double* vz, double* fx, double* fy,
                             double* fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (astart[i + 1] == astart[i] || lfrzn[i] != 0) return;
  double xt = (x[i] - ox[i]) * rstep, yt = (y[i] - oy[i]) * rstep, zt = (z[i] - oz[i]) * rstep;
  vx[i] += xt; vy[i] += yt; vz[i] += zt;
  double tmp = w[i] / hstep;
  fx[i] += xt * tmp; fy[i] += yt * tmp; fz[i] += zt * tmp;
}

__global__ void k_copy3(int n, const double* a, const double* b, const double* c, double* oa, double* ob, double* oc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { oa[i] = a[i]; ob[i] = b[i]; oc[i] = c[i]; }
}

int* d_flags = nullptr;
int coop_blocks_shake = 0, coop_blocks_rattle = 0;
// cluster-local path (used when every constraint cluster is small)
ClusterTab* d_cltab = nullptr;
double* d_clring = nullptr;  // per-cluster state ring (CL_RING slots of CL_SLOT doubles)
double* d_clgsum = nullptr;  // per-cluster committed SHAKE gamma sums
int n_clusters = 0, coop_blocks_cl = 0;
constexpr int CL_THREADS = 128;  // small blocks spread the clusters over every SM
const void* cl_kernel = nullptr;  // k_constrain_cl instantiation for the largest cluster

// connected constraint clusters; false when one exceeds CL_MAXA atoms or CL_MAXC constraints
bool build_clusters(const std::vector<int>& ci, const std::vector<int>& cj, std::vector<ClusterTab>& out) {
  const int n = g.natms, nc = (int)ci.size();
  std::vector<int> parent(n);
  for (int i = 0; i < n; ++i) parent[i] = i;
  auto find = [&](int a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
  };
  for (int k = 0; k < nc; ++k) {
    const int a = find(ci[k]), b = find(cj[k]);
    if (a != b) parent[std::max(a, b)] = std::min(a, b);
  }
  std::vector<int> root_id(n, -1);
  out.clear();
  std::vector<std::vector<int>> atoms, cons;
  for (int k = 0; k < nc; ++k) {  // clusters in order of their first constraint; constraints ascending
    const int r = find(ci[k]);
    if (root_id[r] < 0) {
      root_id[r] = (int)atoms.size();
      atoms.emplace_back();
      cons.emplace_back();
    }
    cons[root_id[r]].push_back(k);
  }
  for (size_t c = 0; c < cons.size(); ++c) {
    for (int k : cons[c])
      for (int e : {ci[k], cj[k]})
        if (std::find(atoms[c].begin(), atoms[c].end(), e) == atoms[c].end()) atoms[c].push_back(e);
    if ((int)atoms[c].size() > CL_MAXA || (int)cons[c].size() > CL_MAXC) return false;
  }
  out.resize(cons.size());
  for (size_t c = 0; c < cons.size(); ++c) {
    ClusterTab& T = out[c];
    for (int a = 0; a < CL_MAXA; ++a) { T.atom[a] = -1; T.alist[a] = 0; }
    for (int q = 0; q < CL_MAXC; ++q) { T.con[q] = -1; T.pair[q] = 0; }
    const int na = (int)atoms[c].size(), ncl = (int)cons[c].size();
    for (int a = 0; a < na; ++a) T.atom[a] = atoms[c][a];
    auto local = [&](int gid) { return (int)(std::find(atoms[c].begin(), atoms[c].end(), gid) - atoms[c].begin()); };
    for (int q = 0; q < ncl; ++q) {
      const int k = cons[c][q];
      T.con[q] = k;
      const int li = local(ci[k]), lj = local(cj[k]);
      T.pair[q] = li | (lj << 4);
      // per-atom entries in constraint order, as the global per-atom table holds them
      for (int end = 0; end < 2; ++end) {
        const int la = end ? lj : li;
        const int cnt = T.alist[la] & 15;
        T.alist[la] = (T.alist[la] & ~15) | (cnt + 1);
        T.alist[la] |= ((q << 1) | end) << (4 + 4 * cnt);
      }
    }
    T.meta = na | (ncl << 4);
  }
  return true;
}

}  // namespace

// ===================================================================== host
void integ_setup_constraints(const int32_t* listcon, const double* prmcon) {
  const int nc = g.ntcons;
  if (nc == 0) return;
  std::vector<int> ci(nc), cj(nc), lt(g.natms, 0);
  std::vector<double> d0(nc);
  for (int k = 0; k < nc; ++k) {
    ci[k] = listcon[3 * k + 1] - 1;
    cj[k] = listcon[3 * k + 2] - 1;
    d0[k] = prmcon[listcon[3 * k] - 1];
    lt[ci[k]]++; lt[cj[k]]++;
  }
  // per-atom constraint table in constraint order; bit 0 = atom is the j end
  std::vector<int> start(g.natms + 1, 0), list;
  for (int i = 0; i < g.natms; ++i) start[i + 1] = start[i] + lt[i];
  list.resize(start[g.natms]);
  std::vector<int> fill(g.natms, 0);
  for (int k = 0; k < nc; ++k) {
    list[start[ci[k]] + fill[ci[k]]++] = (k << 1) | 0;
    list[start[cj[k]] + fill[cj[k]]++] = (k << 1) | 1;
  }
  GB_CUDA(cudaMalloc(&g.con_i, sizeof(int) * nc));
  GB_CUDA(cudaMalloc(&g.con_j, sizeof(int) * nc));
  GB_CUDA(cudaMalloc(&g.con_d0, sizeof(double) * nc));
  GB_CUDA(cudaMalloc(&g.listot, sizeof(int) * g.natms));
  GB_CUDA(cudaMalloc(&g.acon_start, sizeof(int) * (g.natms + 1)));
  GB_CUDA(cudaMalloc(&g.acon_list, sizeof(int) * std::max<size_t>(1, list.size())));
  for (double** p : {&g.dxx, &g.dyy, &g.dzz, &g.dxt, &g.dyt, &g.dzt, &g.dt2, &g.gam})
    GB_CUDA(cudaMalloc(p, sizeof(double) * nc));
  GB_CUDA(cudaMemcpy(g.con_i, ci.data(), sizeof(int) * nc, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(g.con_j, cj.data(), sizeof(int) * nc, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(g.con_d0, d0.data(), sizeof(double) * nc, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(g.listot, lt.data(), sizeof(int) * g.natms, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(g.acon_start, start.data(), sizeof(int) * (g.natms + 1), cudaMemcpyHostToDevice));
  if (!list.empty())
    GB_CUDA(cudaMemcpy(g.acon_list, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice));
  if (d_flags) cudaFree(d_flags);
  GB_CUDA(cudaMalloc(&d_flags, sizeof(int) * (g.p.shake_maxit + CL_CHUNK + 2)));
  int bps = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_shake, 256, 0));
  coop_blocks_shake = std::max(1, std::min(bps * g.nsm, nblocks(std::max(nc, g.natms), 256)));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_rattle, 256, 0));
  coop_blocks_rattle = std::max(1, std::min(bps * g.nsm, nblocks(std::max(nc, g.natms), 256)));
  // cluster-local sweeps when every cluster is small (GB_SHAKE_GLOBAL=1 keeps the per-sweep kernels)
  if (d_cltab) { cudaFree(d_cltab); d_cltab = nullptr; }
  if (d_clring) { cudaFree(d_clring); d_clring = nullptr; }
  if (d_clgsum) { cudaFree(d_clgsum); d_clgsum = nullptr; }
  n_clusters = 0;
  const char* env = std::getenv("GB_SHAKE_GLOBAL");
  std::vector<ClusterTab> tabs;
  if (!(env && env[0] == '1') && build_clusters(ci, cj, tabs)) {
    n_clusters = (int)tabs.size();
    GB_CUDA(cudaMalloc(&d_cltab, sizeof(ClusterTab) * tabs.size()));
    GB_CUDA(cudaMemcpy(d_cltab, tabs.data(), sizeof(ClusterTab) * tabs.size(), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMalloc(&d_clring, sizeof(double) * CL_RING * CL_SLOT * tabs.size()));
    GB_CUDA(cudaMalloc(&d_clgsum, sizeof(double) * CL_MAXC * tabs.size()));
    // rigid 3-site molecules get register arrays sized 3 x 3 (more resident warps)
    bool small = true;
    for (const ClusterTab& T : tabs)
      if ((T.meta & 15) > 3 || ((T.meta >> 4) & 15) > 3) small = false;
    cl_kernel = small ? (const void*)k_constrain_cl<3, 3> : (const void*)k_constrain_cl<CL_MAXA, CL_MAXC>;
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, cl_kernel, CL_THREADS, 0));
    coop_blocks_cl = std::max(1, std::min(bps * g.nsm, nblocks(n_clusters, CL_THREADS)));
  }
}

void integ_zero_forces() {
  if (g.precision == GB_FP64) {
    k_zero3<<<nblocks(g.natms, 256), 256, 0, g.stream>>>(g.natms, g.fx, g.fy, g.fz);
    GB_LAUNCHED();
  } else {
    GB_CUDA(cudaMemsetAsync(g.fixp, 0, sizeof(long long) * 3 * (size_t)g.natms, g.stream));
  }
}

void integ_forces_to_fp64() {
  k_fix_to_fp64<<<nblocks(g.natms, 256), 256, 0, g.stream>>>(g.natms, g.fixp, g.fx, g.fy, g.fz);
  GB_LAUNCHED();
}

void integ_vnl_launch() {
  GB_CUDA(cudaMemsetAsync(&g.sc->maxdisp, 0, sizeof(double), g.stream));
  k_maxdisp<<<std::min(nblocks(g.natms, 256), 2 * g.nsm), 256, 0, g.stream>>>(
      g.natms, g.x, g.y, g.z, g.xbg, g.ybg, g.zbg, g.cell[0], 1.0 / g.cell[0], (unsigned long long*)&g.sc->maxdisp);
  GB_LAUNCHED();
}

int integ_vnl_result() { return std::sqrt(g.hsc->maxdisp) >= std::nextafter(0.5, 0.0) * g.p.rpad ? 1 : 0; }

int integ_vnl_check() {
  integ_vnl_launch();
  gb_sync_scalars();
  return integ_vnl_result();
}

static void con_args(ConArgs& A) {
  A.nc = g.ntcons; A.natms = g.natms; A.maxit = g.p.shake_maxit;
  A.ci = g.con_i; A.cj = g.con_j; A.listot = g.listot; A.astart = g.acon_start; A.alist = g.acon_list;
  A.lfrzn = g.lfrzn; A.d0 = g.con_d0;
  A.dxx = g.dxx; A.dyy = g.dyy; A.dzz = g.dzz; A.dxt = g.dxt; A.dyt = g.dyt; A.dzt = g.dzt;
  A.dt2 = g.dt2; A.gam = g.gam;
  A.x = g.x; A.y = g.y; A.z = g.z; A.vx = g.vx; A.vy = g.vy; A.vz = g.vz; A.w = g.weight;
  A.tstep = g.p.tstep; A.tol = g.p.shake_tol; A.c0 = g.cell[0]; A.a0 = 1.0 / g.cell[0];
  A.flags = d_flags; A.sc = g.sc; A.blk = nullptr;
}

// constraints_tags (constraints.F90:438-586): old bond vectors from the current positions
void integ_con_tags() {
  if (g.ntcons <= 0) return;
  k_con_tags<<<nblocks(g.ntcons, 256), 256, 0, g.stream>>>(g.ntcons, g.con_i, g.con_j, g.x, g.y, g.z, g.cell[0],
                                                             1.0 / g.cell[0], g.dxx, g.dyy, g.dzz);
  GB_LAUNCHED();
}

// apply_shake (constraints.F90:1071-1200): the current positions are the unconstrained
// ones (oxt); SHAKE against the bond vectors of the last integ_con_tags, then the velocity
// and force corrections.  Throws GB_ERR_SHAKE when the iteration does not converge.
void integ_shake(int* iters, double* vircon, double* strcon) {
  if (iters) *iters = 0;
  if (g.ntcons <= 0) return;
  cudaStream_t st = g.stream;
  const int n = g.natms;
  const double tstep = g.p.tstep, hstep = 0.5 * tstep, rstep = 1.0 / tstep;
  k_copy3<<<nblocks(n, 256), 256, 0, st>>>(n, g.x, g.y, g.z, g.ox, g.oy, g.oz);
  GB_LAUNCHED();
  GB_CUDA(cudaMemsetAsync(d_flags, 0, sizeof(int) * (g.p.shake_maxit + CL_CHUNK + 2), st));
  ConArgs A;
  con_args(A);
  const int nbs = n_clusters ? coop_blocks_cl : coop_blocks_shake;
  A.blk = gb_blkacc(nbs * 6);
  prof_begin(P_SHAKE);
  if (n_clusters) {
    const ClusterTab* tabs = d_cltab;
    int ncl = n_clusters, rattle = 0;
    double *ring = d_clring, *gsum = d_clgsum;
    GB_CUDA(cudaMemsetAsync(d_clgsum, 0, sizeof(double) * CL_MAXC * n_clusters, st));
    void* args[] = {&A, &tabs, &ncl, &ring, &gsum, &rattle};
    GB_CUDA(cudaLaunchCooperativeKernel(cl_kernel, nbs, CL_THREADS, args, 0, st));
  } else {
    void* args[] = {&A};
    GB_CUDA(cudaLaunchCooperativeKernel((void*)k_shake, nbs, 256, args, 0, st));
  }
  GB_LAUNCHED();
  prof_end(P_SHAKE);
  gb_reduce_blocks(A.blk, nbs, 6, &g.sc->acc[A_STRCON]);
  k_shake_post<<<nblocks(n, 256), 256, 0, st>>>(n, g.acon_start, g.lfrzn, rstep, hstep, g.weight, g.x, g.y, g.z,
                                                 g.ox, g.oy, g.oz, g.vx, g.vy, g.vz, g.fx, g.fy, g.fz);
  GB_LAUNCHED();
  gb_sync_scalars();
  if (iters) *iters = g.hsc->shake_iters;
  const double* s = &g.hsc->acc[A_STRCON];
  double str[9] = {s[0], s[1], s[2], s[1], s[3], s[4], s[2], s[4], s[5]};
  if (strcon) for (int k = 0; k < 9; ++k) strcon[k] = str[k];
  if (vircon) *vircon = -(str[0] + str[4] + str[8]);
  if (g.hsc->status & ST_SHAKE_FAIL) throw (int)GB_ERR_SHAKE;
}

// apply_rattle with kit = 1 (constraints.F90:1032-1069 -> constraints_rattle :587-775) on
// the current velocities, against the bond vectors of the last integ_con_tags.  The
// status is read by the caller (ST_RATTLE_FAIL).
void integ_rattle_launch() {
  if (g.ntcons <= 0) return;
  cudaStream_t st = g.stream;
  GB_CUDA(cudaMemsetAsync(d_flags, 0, sizeof(int) * (g.p.shake_maxit + CL_CHUNK + 2), st));
  ConArgs A;
  con_args(A);
  prof_begin(P_RATTLE);
  if (n_clusters) {
    const ClusterTab* tabs = d_cltab;
    int ncl = n_clusters, rattle = 1;
    double *ring = d_clring, *gsum = d_clgsum;
    void* args[] = {&A, &tabs, &ncl, &ring, &gsum, &rattle};
    GB_CUDA(cudaLaunchCooperativeKernel(cl_kernel, coop_blocks_cl, CL_THREADS, args, 0, st));
  } else {
    void* args[] = {&A};
    GB_CUDA(cudaLaunchCooperativeKernel((void*)k_rattle, coop_blocks_rattle, 256, args, 0, st));
  }
  GB_LAUNCHED();
  prof_end(P_RATTLE);
}

void integ_vv(int stage, double* strkin, double* engke, int* iters, double* vircon, double* strcon) {
  cudaStream_t st = g.stream;
  const int n = g.natms;
  const double tstep = g.p.tstep, hstep = 0.5 * tstep;
  if (iters) *iters = 0;
  integ_con_tags();
  if (stage == 1) {
    prof_begin(P_VV);
    if (!thermo_vv1(hstep, tstep)) {
      k_vv1<<<nblocks(n, 256), 256, 0, st>>>(n, g.hdw, tstep, g.fx, g.fy, g.fz, g.vx, g.vy, g.vz, g.x, g.y, g.z);
      GB_LAUNCHED();
    }
    prof_end(P_VV);
    integ_shake(iters, vircon, strcon);
  } else {
    prof_begin(P_VV);
    k_vv2<<<nblocks(n, 256), 256, 0, st>>>(n, g.hdw, g.fx, g.fy, g.fz, g.vx, g.vy, g.vz);
    GB_LAUNCHED();
    prof_end(P_VV);
    integ_rattle_launch();
    if (!thermo_vv2_finish(strkin, engke)) {
      const int nb = std::min(nblocks(n, 256), 2 * g.nsm);
      double* blk = gb_blkacc(nb * 6);
      k_kinstress<<<nb, 256, 0, st>>>(n, g.weight, g.lfrzn, g.vx, g.vy, g.vz, blk);
      GB_LAUNCHED();
      gb_reduce_blocks(blk, nb, 6, &g.sc->acc[A_STRKIN]);
      if (g.defer_scalars) return;  // the MD loop reads the sums after its last step
      gb_sync_scalars();
      kin_scalars(g.hsc, strkin, engke);
    }
    if (iters && g.ntcons > 0) *iters = g.hsc->rattle_iters;
    if (g.ntcons > 0 && (g.hsc->status & ST_RATTLE_FAIL)) throw (int)GB_ERR_RATTLE;
    if (g.hsc->status & ST_RNG) throw (int)GB_ERR_RNG;
    if (g.hsc->status & ST_DEVICE_WAIT) throw (int)GB_ERR_DEVICE_WAIT;
  }
}

// kinetic stress (symmetric 3x3) and kinetic energy from the device sums
void kin_scalars(const DevScalars* h, double* strkin, double* engke) {
  const double* s = &h->acc[A_STRKIN];
  double sk[9] = {s[0], s[1], s[2], s[1], s[3], s[4], s[2], s[4], s[5]};
  if (strkin) for (int k = 0; k < 9; ++k) strkin[k] = sk[k];
  if (engke) *engke = 0.5 * (sk[0] + sk[4] + sk[8]);
}
