// gb_metal.cu - tabulated embedded-atom (EAM) metal forces on the device: the
// two passes of the reference (local density, then forces) over the Verlet list.
//
// Follows:
//   metal_table_read          source/metal.F90:1489-1925 (tab = 1, 'eam': pair, dens, embe tables)
//   metal_table_derivatives   source/metal.F90:2807-2897 (five-point derivative of each table)
//   metal_ld_compute          source/metal.F90:897-1257 (embedding F(rho), F'(rho), error 507)
//   metal_ld_collect_eam      source/metal.F90:2207-2516 (density pass, error 506)
//   metal_ld_set_halo         source/metal.F90:3146 (F'(rho) on the halo images)
//   metal_forces              source/metal.F90:193-895 (tabulated EAM branch)
// in the serial build without HALF_HALO (the default), whose bookkeeping is: a
// pair across the cell boundary is listed from both sides; each side adds only
// to its own local atom, and its energy is counted from the side with the smaller
// global id.  Here such a pair is evaluated once, from that side, and applied to
// both atoms, which gives the same sums.
//
// Every table value is interpolated with the reference's three-point formula
// (the l-1, l, l+1 points, its branch on ppp < 0 and l == 5).  Forces are summed
// in FP64 (the FP64 form; metals are not offered in the mixed form).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "gb_common.cuh"

namespace {

inline int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ double interp3(const double* v, int l, double ppp);
__device__ __forceinline__ double interp3_raw(const double* v, int l, double ppp) { return interp3(v, l, ppp); }

struct MetTab {
  int n;          // Nint(buffer(1)) = ngrid + 4; 0 = no table
  int off;        // values at v[off + i], i = 1..n (Fortran index), derivatives at d[off + i]
  double r0;      // start - 5*dr
  double rmax;    // finish
  double dr;
  double rdr;     // 1/dr as the reference forms it
  int grid;       // tables with the same (r0, rdr, n) share a grid id: one index serves them all
  int listed;     // pair tables: the FIELD 'metal' directive lists this type pair (keypot 0)
  double nr0rdr;  // -r0 * rdr: x = r * rdr + nr0rdr
  long long b_lo, b_hi;  // r <= rmax decided on rsq bits outside [rmax^2 (1 -+ 1e-12)]
};

// r <= rmax as the reference decides it (correctly rounded sqrt), from the bits of rsq
// except inside a narrow band around rmax^2
__device__ __forceinline__ bool within(long long rb, long long lo, long long hi, double rsq, double rmax) {
  return rb < lo || (rb <= hi && sqrt(rsq) <= rmax);
}

// The three-point formula is the quadratic through (l-1, l, l+1) in both of its
// ppp branches, so the force passes evaluate it from per-point coefficients
// c0 + p (c1 + p c2), c0 = v_l, c1 = (v_{l+1} - v_{l-1})/2, c2 = (v_{l+1} - 2 v_l + v_{l-1})/2
// (two FMAs).  Entry l = 5 holds the linear form the reference uses there for
// ppp >= 0; the rare l = 5, ppp < 0 case and the density's negative fall-back read
// the raw values.
struct Coef {
  double c0, c1, c2, pad;
};

__device__ __forceinline__ double qeval(const Coef* c, int l, double p) {
  const double2 a = *reinterpret_cast<const double2*>(&c[l].c0);
  const double b = c[l].c2;
  return fma(p, fma(p, b, a.y), a.x);
}

// l = Nint((r - r0) / dr) clamped to [5, n-1] and ppp: the nearest integer comes from
// adding 1.5*2^52 (no FP64 conversion); false if the reference's l < 5 guard fires
__device__ __forceinline__ bool qindex(const MetTab& t, double r, int* l, double* ppp) {
  const double x = fma(r, t.rdr, t.nr0rdr);
  const double big = 6755399441055744.0;
  const double tt = x + big;
  int k = __double2loint(tt);
  double kd = tt - big;
  bool ok = true;
  if (k > t.n - 1) { k = t.n - 1; kd = (double)k; }
  if (k < 5) { ok = false; k = 6; kd = 6.0; }
  *l = k;
  *ppp = x - kd;
  return ok;
}

__device__ __forceinline__ double qeval_full(const Coef* c, const double* raw, int l, double p) {
  if (l == 5 && p < 0.0) return interp3_raw(raw, l, p);
  return qeval(c, l, p);
}

// metal_ld_compute / metal_forces interpolation: index l and fraction ppp
__device__ __forceinline__ bool tab_index(const MetTab& t, double r, int* l, double* ppp) {
  const double rr1 = r - t.r0;
  int k = min((int)round(rr1 * t.rdr), t.n - 1);
  bool ok = true;
  if (k < 5) { ok = false; k = 6; }
  *l = k;
  *ppp = rr1 * t.rdr - (double)k;
  return ok;
}

__device__ __forceinline__ double interp3(const double* v, int l, double ppp) {
  const double vk0 = v[l - 1], vk1 = v[l], vk2 = v[l + 1];
  const double t1 = vk1 + ppp * (vk1 - vk0);
  const double t2 = vk1 + ppp * (vk2 - vk1);
  if (ppp < 0.0) return t1 + 0.5 * (t2 - t1) * (ppp + 1.0);
  if (l == 5) return t2;
  return t2 + 0.5 * (t2 - t1) * (ppp - 1.0);
}

// density: the same formula, but a negative result falls back to t1 / t2
__device__ __forceinline__ double interp3_density(const double* v, int l, double ppp) {
  const double vk0 = v[l - 1], vk1 = v[l], vk2 = v[l + 1];
  const double t1 = vk1 + ppp * (vk1 - vk0);
  const double t2 = vk1 + ppp * (vk2 - vk1);
  if (ppp < 0.0) {
    const double d = t1 + 0.5 * (t2 - t1) * (ppp + 1.0);
    return d < 0.0 ? t1 : d;
  }
  if (l == 5) return t2;
  const double d = t2 + 0.5 * (t2 - t1) * (ppp - 1.0);
  return d < 0.0 ? t2 : d;
}

struct MetArgs {
  const MetTab* tab;    // [nkey pair | ntypes density | ntypes embedding]
  const double* v;      // table values (column 1), Fortran-indexed from off
  const double* d;      // column 2: -r dV/dr, -r drho/dr, dF/drho
  const Coef* cv;       // quadratic coefficients of column 1 (same offsets)
  const Coef* cd;       // and of column 2
  const int* listed;    // per pair key: 1 if the FIELD lists it (keypot = 0), else 0 (keypot = -1)
  int nkey, ntypes, ntab;
  double rcut;
  long long b_rc_lo, b_rc_hi;   // rcut^2 band as bit patterns
};

constexpr int MAX_TAB = 64;  // tables staged in shared memory (ntypes <= 8)

__device__ __forceinline__ void stage_tables(const MetArgs& A, MetTab* st) {
  for (int k = threadIdx.x; k < A.ntab; k += blockDim.x) st[k] = A.tab[k];
  __syncthreads();
}

// density from one species table; a negative quadratic falls back to t1 / t2 (metal_ld_collect_eam)
__device__ __forceinline__ double density_at(const MetArgs& A, const MetTab& t, int l, double p) {
  double dens = qeval_full(A.cv + t.off, A.v + t.off, l, p);
  const long long db = __double_as_longlong(dens);
  if (db < 0 && db != (long long)0x8000000000000000ull) dens = interp3_density(A.v + t.off, l, p);  // < 0
  return dens;
}

// r from rsq: seeded 1/sqrt (exact sqrt for a zero or subnormal rsq, which the table
// guards then reject)
__device__ __forceinline__ double dist_from(double rsq, long long rb, double* rinv) {
  if (rb < DBL_MIN_BITS) { *rinv = 0.0; return sqrt(rsq); }
  *rinv = rsqrt_seeded(rsq);
  return rsq * (*rinv);
}

__global__ void __launch_bounds__(256) k_metal_density(int natms, const DevScalars* sc, const int* __restrict__ at_list,
                                                       const int* __restrict__ list, int ld, const double* __restrict__ x,
                                                       const double* __restrict__ y, const double* __restrict__ z,
                                                       const int* __restrict__ ltype, const int* __restrict__ ltg,
                                                       const int* __restrict__ src, MetArgs A, double* rho,
                                                       int* status) {
  __shared__ MetTab tabs[MAX_TAB];
  stage_tables(A, tabs);
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nlast = sc->nlast;
  bool bad = false;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nlast; w += nwarps) {
    const int i = at_list[w];
    if (i >= natms) continue;
    const double xi = x[i], yi = y[i], zi = z[i];
    const int ai = ltype[i], gi = ltg[i];
    const MetTab& ti = tabs[A.nkey + ai - 1];
    const int* li = list + (size_t)i * ld + 3;
    const int n = li[0];
    double rho_i = 0.0;
    for (int m = lane + 1; m <= n; m += 32) {
      const int j = li[m] - 1;
      int jf = j;
      if (j >= natms) {
        if (gi > ltg[j]) continue;  // counted from the other side
        jf = src[j];
      }
      const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
      const double rsq = dx * dx + dy * dy + dz * dz;
      const long long rb = __double_as_longlong(rsq);
      const int aj = ltype[j];
      const MetTab& tj = tabs[A.nkey + aj - 1];
      const bool in_j = tj.n > 5 && within(rb, tj.b_lo, tj.b_hi, rsq, tj.rmax);
      const bool in_i = ai != aj && ti.n > 5 && within(rb, ti.b_lo, ti.b_hi, rsq, ti.rmax);
      if (!in_j && !in_i) continue;
      double rinv;
      const double r = dist_from(rsq, rb, &rinv);
      // to i from j's species table, to j from i's (metal_ld_collect_eam)
      int l = 0;
      double p = 0.0;
      int gl = -1;
      double to_j = 0.0;
      if (in_j) {
        if (!qindex(tj, r, &l, &p)) bad = true;
        gl = tj.grid;
        const double dens = density_at(A, tj, l, p);
        rho_i += dens;
        if (ai == aj) to_j = dens;
      }
      if (in_i) {
        if (ti.grid != gl && !qindex(ti, r, &l, &p)) bad = true;
        to_j = density_at(A, ti, l, p);
      }
      if ((__double_as_longlong(to_j) & 0x7FFFFFFFFFFFFFFFll) != 0) atomicAdd(&rho[jf], to_j);
    }
    rho_i = warp_sum(rho_i);
    if (lane == 0 && rho_i != 0.0) atomicAdd(&rho[i], rho_i);
  }
  if (bad) atomicOr(status, ST_METAL_TABLE);
}

// embedding energy and F'(rho) (metal_ld_compute, tab > 0, rho grid)
__global__ void k_metal_embed(int natms, const int* ltype, MetArgs A, double* rho, double* blk, int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e[1] = {0.0};
  int st = 0;
  if (i < natms) {
    const MetTab& t = A.tab[A.nkey + A.ntypes + ltype[i] - 1];
    if (t.n > 0) {
      const double rhosqr = rho[i];
      if (rhosqr >= t.r0 + 5.0 * t.dr) {
        if (rhosqr <= t.rmax) {
          int l;
          double p;
          if (!tab_index(t, rhosqr, &l, &p)) st |= ST_METAL_DENSITY;
          e[0] = interp3(A.v + t.off, l, p);
          rho[i] = interp3(A.d + t.off, l, p);
        } else {  // beyond the table: F at its last point, F' = 0
          e[0] = A.v[t.off + t.n];
          rho[i] = 0.0;
        }
      } else {
        st |= ST_METAL_DENSITY;
      }
    }
  }
  if (st) atomicOr(status, st);
  block_reduce_store<1>(e, blk);
}

// metal_ld_set_halo: images carry F'(rho) of their source atom
__global__ void k_metal_halo(int natms, const DevScalars* sc, const int* src, double* rho) {
  const int k = natms + blockIdx.x * blockDim.x + threadIdx.x;
  if (k < sc->nlast) rho[k] = rho[src[k]];
}

constexpr int MACC = 8;  // engmet, virmet, stress (6)

__global__ void __launch_bounds__(256, 3) k_metal_forces(int natms, const DevScalars* sc, const int* __restrict__ at_list,
                                                      const int* __restrict__ list, int ld, const double* __restrict__ x,
                                                      const double* __restrict__ y, const double* __restrict__ z,
                                                      const int* __restrict__ ltype, const int* __restrict__ ltg,
                                                      const int* __restrict__ src, MetArgs A,
                                                      const double* __restrict__ rho, double* fx, double* fy, double* fz,
                                                      double* blk, int* status, unsigned long long* cnt) {
  __shared__ MetTab tabs[MAX_TAB];
  stage_tables(A, tabs);
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nlast = sc->nlast;
  double acc[MACC];
#pragma unroll
  for (int k = 0; k < MACC; ++k) acc[k] = 0.0;
  bool bad = false;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nlast; w += nwarps) {
    const int i = at_list[w];
    if (i >= natms) continue;
    const double xi = x[i], yi = y[i], zi = z[i], rho_i = rho[i];
    const int ai = ltype[i], gi = ltg[i];
    const MetTab& ti = tabs[A.nkey + ai - 1];
    const int* li = list + (size_t)i * ld + 3;
    const int n = li[0];
    double fix = 0.0, fiy = 0.0, fiz = 0.0;
    int nrc = 0;
    for (int m = lane + 1; m <= n; m += 32) {
      const int j = li[m] - 1;
      int jf = j;
      if (j >= natms) {
        if (gi > ltg[j]) continue;
        jf = src[j];
      }
      const int aj = ltype[j];
      const int key = (ai > aj ? ai * (ai - 1) / 2 + aj : aj * (aj - 1) / 2 + ai) - 1;
      const MetTab& tp = tabs[key];
      if (!tp.listed) continue;  // keypot = -1
      const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
      const double rsq = dx * dx + dy * dy + dz * dz;
      const long long rb = __double_as_longlong(rsq);
      if (!within(rb, A.b_rc_lo, A.b_rc_hi, rsq, A.rcut)) continue;   // rrr <= met%rcut
      ++nrc;
      double rinv;
      const double rrr = dist_from(rsq, rb, &rinv);
      const double inv_rsq = rinv * rinv;
      double eng = 0.0, gamma1 = 0.0, gamma2 = 0.0, gamma3 = 0.0;
      int l = 0, gl = -1;
      double p = 0.0;
      if (tp.n > 0 && within(rb, tp.b_lo, tp.b_hi, rsq, tp.rmax)) {
        if (!qindex(tp, rrr, &l, &p)) bad = true;
        gl = tp.grid;
        gamma1 = qeval_full(A.cd + tp.off, A.d + tp.off, l, p);
        eng = qeval_full(A.cv + tp.off, A.v + tp.off, l, p);
      }
      const MetTab& tj = tabs[A.nkey + aj - 1];
      if (tj.n > 0 && ti.n > 5 && within(rb, tj.b_lo, tj.b_hi, rsq, tj.rmax)) {
        if (tj.grid != gl && !qindex(tj, rrr, &l, &p)) bad = true;
        gl = tj.grid;
        gamma2 = qeval_full(A.cd + tj.off, A.d + tj.off, l, p);
      }
      if (ai == aj) {
        gamma3 = gamma2;
      } else if (ti.n > 5 && within(rb, ti.b_lo, ti.b_hi, rsq, ti.rmax)) {
        if (ti.grid != gl && !qindex(ti, rrr, &l, &p)) bad = true;
        gamma3 = qeval_full(A.cd + ti.off, A.d + ti.off, l, p);
      }
      const double num = gamma1 + (gamma2 * rho_i + gamma3 * rho[j]);  // gamma * rsq
      const double gamma = num * inv_rsq;
      const double fxx = gamma * dx, fyy = gamma * dy, fzz = gamma * dz;
      fix += fxx; fiy += fyy; fiz += fzz;
      atomicAdd(&fx[jf], -fxx);
      atomicAdd(&fy[jf], -fyy);
      atomicAdd(&fz[jf], -fzz);
      acc[0] += eng;
      acc[1] -= num;
      acc[2] = fma(dx, fxx, acc[2]); acc[3] = fma(dx, fyy, acc[3]); acc[4] = fma(dx, fzz, acc[4]);
      acc[5] = fma(dy, fyy, acc[5]); acc[6] = fma(dy, fzz, acc[6]); acc[7] = fma(dz, fzz, acc[7]);
    }
    fix = warp_sum(fix); fiy = warp_sum(fiy); fiz = warp_sum(fiz);
    if (cnt) nrc = warp_sumi(nrc);
    if (lane == 0) {
      atomicAdd(&fx[i], fix);
      atomicAdd(&fy[i], fiy);
      atomicAdd(&fz[i], fiz);
      if (cnt) {  // list entries walked and pairs inside the cutoff, when no pair kernel counts them
        atomicAdd(&cnt[0], (unsigned long long)n);
        atomicAdd(&cnt[1], (unsigned long long)nrc);
      }
    }
  }
  if (bad) atomicOr(status, ST_METAL_TABLE);
  block_reduce_store<MACC>(acc, blk);
}

// ------------------------------------------------------------------- host state
MetTab* d_tab = nullptr;
double* d_val = nullptr;
double* d_der = nullptr;
Coef* d_cv = nullptr;
Coef* d_cd = nullptr;
int* d_listed = nullptr;
double* d_rho = nullptr;
int n_key = 0, n_tab = 0, occ_dens = 0, occ_force = 0;

// metal_table_derivatives: five-point derivative on the normalised neighbours
void table_derivatives(const std::vector<double>& buf, std::vector<double>& der) {
  // buf and der are Fortran-indexed (element 0 unused), buf(1..4) the header
  const double delmet = buf[4];
  const int v_end = (int)std::lround(buf[1]);
  const int i_start = 5 + 2, i_end = v_end - 2;
  for (int i = i_start; i <= i_end; ++i) {
    double aa0 = buf[i], f0, f1, f2, f3, f4;
    if (std::fabs(aa0) <= DBL_MIN) {
      f0 = f1 = f2 = f3 = f4 = 0.0;
    } else {
      f0 = buf[i - 2] / aa0;
      f1 = buf[i - 1] / aa0;
      f2 = 1.0;
      f3 = buf[i + 1] / aa0;
      f4 = buf[i + 2] / aa0;
    }
    const double d1y = (f1 - f0);
    const double d2y = (f2 - f1) - (f1 - f0);
    const double d3y = (f3 - f0) + 3.0 * (f1 - f2);
    const double d4y = (f4 - f3) + 3.0 * (f2 - f3) + 3.0 * (f2 - f1) + (f0 - f1);
    aa0 = aa0 / delmet;
    const double aa4 = d4y / 24.0;
    const double aa3 = (d3y + 12.0 * aa4) / 6.0;
    const double aa2 = (d2y + 6.0 * aa3 - 14.0 * aa4) / 2.0;
    const double aa1 = d1y + 3.0 * aa2 - 7.0 * aa3 + 15.0 * aa4;
    der[i] = aa1 * aa0;
    if (i == i_start) {
      der[i_start - 2] = (aa1 - 4.0 * aa2 + 12.0 * aa3 - 32.0 * aa4) * aa0;
      der[i_start - 1] = (aa1 - 2.0 * aa2 + 3.0 * aa3 - 4.0 * aa4) * aa0;
    } else if (i == i_end) {
      der[i_end + 1] = (aa1 + 2.0 * aa2 + 3.0 * aa3 + 4.0 * aa4) * aa0;
      der[i_end + 2] = (aa1 + 4.0 * aa2 + 12.0 * aa3 + 32.0 * aa4) * aa0;
    }
  }
}

}  // namespace

void metal_free() {
  void* p[] = {d_tab, d_val, d_der, d_cv, d_cd, d_listed, d_rho};
  for (void* q : p)
    if (q) cudaFree(q);
  d_tab = nullptr; d_val = nullptr; d_der = nullptr; d_cv = nullptr; d_cd = nullptr; d_listed = nullptr;
  d_rho = nullptr;
  n_key = n_tab = 0;
  g.has_metal = false;
}

bool metal_active() { return g.has_metal; }

// kind[k] 1 = pair (types t1, t2), 2 = density (type t1), 3 = embedding (type t1);
// values in the units of the tables after the FIELD energy unit is applied
// (pair and embedding energies in internal units)
int metal_setup(int ntab, const int32_t* kind, const int32_t* t1, const int32_t* t2, const int32_t* ngrid,
                const double* start, const double* finish, const double* values, const int32_t* listed) {
  metal_free();
  const int nt = g.p.ntypes;
  n_key = nt * (nt + 1) / 2;
  n_tab = n_key + 2 * nt;
  if (n_tab > 64) return GB_ERR_ARG;  // MAX_TAB tables (8 species)
  std::vector<MetTab> tab(n_tab);
  for (auto& t : tab) {
    t.n = 0; t.off = 0; t.r0 = t.rmax = t.dr = t.rdr = t.nr0rdr = 0.0; t.grid = -1; t.listed = 0;
    t.b_lo = t.b_hi = 0;
  }
  std::vector<double> val(1, 0.0), der(1, 0.0);
  size_t pos = 0;
  for (int k = 0; k < ntab; ++k) {
    const int ng = ngrid[k];
    if (ng < 5 || kind[k] < 1 || kind[k] > 3 || t1[k] < 1 || t1[k] > nt) return GB_ERR_ARG;
    int id;
    if (kind[k] == 1) {
      if (t2[k] < 1 || t2[k] > nt) return GB_ERR_ARG;
      const int a = std::max(t1[k], t2[k]), b = std::min(t1[k], t2[k]);
      id = a * (a - 1) / 2 + b - 1;
    } else {
      id = n_key + (kind[k] == 2 ? 0 : nt) + t1[k] - 1;
    }
    // metal_table_read: buffer(1) = ngrid + 4, buffer(4) = dr, buffer(2) = start - 5 dr, buffer(3) = finish
    std::vector<double> buf(ng + 5 + 1, 0.0), d(ng + 5 + 1, 0.0);
    buf[1] = (double)(ng + 4);
    buf[4] = (finish[k] - start[k]) / (double)(ng - 1);
    buf[2] = start[k] - 5.0 * buf[4];
    buf[3] = finish[k];
    for (int i = 0; i < ng; ++i) buf[5 + i] = values[pos + i];
    pos += ng;
    table_derivatives(buf, d);
    for (int i = 1; i <= 4; ++i) d[i] = kind[k] == 2 ? 0.0 : buf[i];  // header copies; zero for density
    if (kind[k] != 3)  // pair and density: column 2 holds -r d/dr
      for (int i = 5; i <= ng + 4; ++i) d[i] = -((double)i * buf[4] + buf[2]) * d[i];
    MetTab& t = tab[id];
    t.n = ng + 4;
    t.off = (int)val.size() - 1;
    t.r0 = buf[2];
    t.rmax = buf[3];
    t.dr = buf[4];
    t.rdr = 1.0 / buf[4];
    // entries 1..n+1 as the reference's arrays hold them: the header in 1..4 (an
    // interpolation at l = 5 reads entry 4), the values, then zeros
    for (int i = 1; i <= ng + 5; ++i) {
      val.push_back(buf[i]);
      der.push_back(d[i]);
    }
  }
  // quadratic coefficients per point (entry l = 5: the reference's linear form for ppp >= 0)
  std::vector<Coef> cv(val.size()), cd(der.size());
  for (auto& c : cv) c = Coef{0, 0, 0, 0};
  for (auto& c : cd) c = Coef{0, 0, 0, 0};
  for (int id = 0; id < n_tab; ++id) {
    const MetTab& t = tab[id];
    if (t.n == 0) continue;
    for (int l = 5; l <= t.n - 1; ++l) {
      for (int col = 0; col < 2; ++col) {
        const std::vector<double>& w = col ? der : val;
        const double v0 = w[t.off + l - 1], v1 = w[t.off + l], v2 = w[t.off + l + 1];
        Coef& c = col ? cd[t.off + l] : cv[t.off + l];
        if (l == 5) c = Coef{v1, v2 - v1, 0.0, 0.0};
        else c = Coef{v1, 0.5 * (v2 - v0), 0.5 * ((v2 - v1) - (v1 - v0)), 0.0};
      }
    }
  }
  // grid ids: tables on the same grid share one index computation
  int ngrid_ids = 0;
  for (int id = 0; id < n_tab; ++id) {
    if (tab[id].n == 0) continue;
    for (int o = 0; o < id && tab[id].grid < 0; ++o)
      if (tab[o].n == tab[id].n && tab[o].r0 == tab[id].r0 && tab[o].rdr == tab[id].rdr) tab[id].grid = tab[o].grid;
    if (tab[id].grid < 0) tab[id].grid = ngrid_ids++;
  }
  std::vector<int> lst(n_key, 0);
  for (int k = 0; k < n_key; ++k) lst[k] = listed ? listed[k] : 1;
  auto bits = [](double v) { long long b; std::memcpy(&b, &v, 8); return b; };
  for (int id = 0; id < n_tab; ++id) {
    MetTab& t = tab[id];
    if (id < n_key) t.listed = lst[id];
    if (t.n == 0) continue;
    t.nr0rdr = -t.r0 * t.rdr;
    t.b_lo = bits(t.rmax * t.rmax * (1.0 - 1e-12));
    t.b_hi = bits(t.rmax * t.rmax * (1.0 + 1e-12));
  }
  GB_CUDA(cudaMalloc(&d_tab, sizeof(MetTab) * n_tab));
  GB_CUDA(cudaMalloc(&d_val, sizeof(double) * val.size()));
  GB_CUDA(cudaMalloc(&d_der, sizeof(double) * der.size()));
  GB_CUDA(cudaMalloc(&d_cv, sizeof(Coef) * cv.size()));
  GB_CUDA(cudaMalloc(&d_cd, sizeof(Coef) * cd.size()));
  GB_CUDA(cudaMemcpy(d_cv, cv.data(), sizeof(Coef) * cv.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(d_cd, cd.data(), sizeof(Coef) * cd.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMalloc(&d_listed, sizeof(int) * n_key));
  GB_CUDA(cudaMalloc(&d_rho, sizeof(double) * std::max(g.mxatms, 1)));
  GB_CUDA(cudaMemcpy(d_tab, tab.data(), sizeof(MetTab) * n_tab, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(d_val, val.data(), sizeof(double) * val.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(d_der, der.data(), sizeof(double) * der.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(d_listed, lst.data(), sizeof(int) * n_key, cudaMemcpyHostToDevice));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_dens, k_metal_density, 256, 0));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_force, k_metal_forces, 256, 0));
  g.has_metal = true;
  return GB_OK;
}

// both passes; adds forces into g.fx/fy/fz and stress into stress9; returns
// engmet, virmet (pair part) and engden, virden (embedding part) in e4
void metal_forces(double* e4, double* stress9) {
  cudaStream_t st = g.stream;
  MetArgs A;
  A.tab = d_tab; A.v = d_val; A.d = d_der; A.cv = d_cv; A.cd = d_cd; A.listed = d_listed;
  A.nkey = n_key; A.ntypes = g.p.ntypes; A.ntab = n_tab; A.rcut = g.p.rcut;
  {
    const double rc2 = g.p.rcut * g.p.rcut, lo = rc2 * (1.0 - 1e-12), hi = rc2 * (1.0 + 1e-12);
    std::memcpy(&A.b_rc_lo, &lo, 8);
    std::memcpy(&A.b_rc_hi, &hi, 8);
  }
  const int T = 256;
  GB_CUDA(cudaMemsetAsync(d_rho, 0, sizeof(double) * g.mxatms, st));
  prof_begin(P_METAL_DENSITY);
  int nb = std::max(1, std::min(nblocks((long long)g.mxatms * 32, T), occ_dens * g.nsm));
  k_metal_density<<<nb, T, 0, st>>>(g.natms, g.sc, g.at_list, g.list, g.ld, g.x, g.y, g.z, g.ltype, g.ltg, g.src, A,
                                    d_rho, &g.sc->status);
  GB_LAUNCHED();
  const int nbe = nblocks(g.natms, T);
  double* blk = gb_blkacc(std::max(nbe, 1) + MACC * std::max(1, occ_force * g.nsm));
  k_metal_embed<<<nbe, T, 0, st>>>(g.natms, g.ltype, A, d_rho, blk, &g.sc->status);
  GB_LAUNCHED();
  gb_reduce_blocks(blk, nbe, 1, &g.sc->acc[A_METAL + 8]);
  k_metal_halo<<<nblocks(std::max(g.mxatms - g.natms, 1), T), T, 0, st>>>(g.natms, g.sc, g.src, d_rho);
  GB_LAUNCHED();
  prof_end(P_METAL_DENSITY);
  prof_begin(P_METAL_FORCES);
  nb = std::max(1, std::min(nblocks((long long)g.mxatms * 32, T), occ_force * g.nsm));
  double* blk2 = blk + std::max(nbe, 1);
  unsigned long long* cnt = nullptr;
  if (!g.has_coul && !g.has_vdw) {  // the pair kernel did not run: count here
    GB_CUDA(cudaMemsetAsync(&g.sc->npairs_list, 0, 2 * sizeof(unsigned long long), st));
    cnt = &g.sc->npairs_list;
  }
  k_metal_forces<<<nb, T, 0, st>>>(g.natms, g.sc, g.at_list, g.list, g.ld, g.x, g.y, g.z, g.ltype, g.ltg, g.src, A,
                                   d_rho, g.fx, g.fy, g.fz, blk2, &g.sc->status, cnt);
  GB_LAUNCHED();
  gb_reduce_blocks(blk2, nb, MACC, &g.sc->acc[A_METAL]);
  prof_end(P_METAL_FORCES);
  gb_sync_scalars();
  if (g.hsc->status & ST_METAL_DENSITY) throw (int)GB_ERR_METAL_DENSITY;
  if (g.hsc->status & ST_METAL_TABLE) throw (int)GB_ERR_METAL_TABLE;
  const double* a = &g.hsc->acc[A_METAL];
  e4[0] = a[0];
  e4[1] = a[1];
  e4[2] = a[8];
  e4[3] = 0.0;  // virden: no long-range density correction for tabulated EAM
  const double s[9] = {a[2], a[3], a[4], a[3], a[5], a[6], a[4], a[6], a[7]};
  for (int k = 0; k < 9; ++k) stress9[k] += s[k];
}

void metal_rho(double* out, int n) {
  GB_CUDA(cudaMemcpy(out, d_rho, sizeof(double) * std::min(n, g.natms), cudaMemcpyDeviceToHost));
}
