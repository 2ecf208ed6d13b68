// dlpoly_oracle.cpp -- CPU FP64 restatement of DL_POLY 5's per-timestep
// force and update path, in serial (one domain) semantics.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300
// library: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg may load it, and only for the parity tests' reference results or the timed CPU
// baseline.  It is
// never part of the product path.
//
// The reference is Fortran 2008 and cannot be compiled here (no Fortran
// toolchain), so this is a restatement, compiled with -O2 -ffp-contract=off
// -fno-fast-math so that each arithmetic expression rounds as written.  Every
// routine cites the reference file:line it follows (paths relative to the
// DL_POLY source tree).  Parity pins: source/unit_tests/test_vdw.F90:46-59
// (12-6 / LJ energies and virials) plus physics invariants; the pair sets,
// SPME, FFT and SHAKE/RATTLE have no reference golden vectors.
//
// Entry points mirror include/gb300_dlpoly.h with an orc_ prefix.

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef ORACLE_OPENMP
#include <omp.h>
#endif

#include "../include/gb300_dlpoly.h"

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kR4pie0 = 138935.4835;          // constants.F90:100
constexpr double kZeroPlus = DBL_MIN;            // constants.F90:189 Tiny(1.0_wp)
constexpr double kEpsWp = DBL_EPSILON;           // constants.F90:200
constexpr double kSmalldr = 1.0e-6;              // constants.F90:204
const double kHalfPlus = std::nextafter(0.5, 1.0);   // constants.F90:195
const double kHalfMinus = std::nextafter(0.5, 0.0);  // constants.F90:197
const double kSqrpi = std::sqrt(kPi);
const double kRsqrpi = 1.0 / std::sqrt(kPi);

// Fortran Anint: round half away from zero.
inline double anint(double x) { return std::round(x); }
// Fortran Int(real): truncation toward zero.
inline int fint(double x) { return (int)x; }
inline double sq(double x) { return x * x; }

struct Ctx {
  bool init = false;
  gb_params p{};
  double cell[9], rcell[9], celprp[10], volm;
  double rcutx;  // neigh%cutoff_extended
  int natms = 0, nlast = 0, mxatms = 0;
  // per atom, size mxatms (local then halo)
  std::vector<double> x, y, z, fx, fy, fz, chge, weight;
  std::vector<int> ltg, ltype, lfrzn, ixyz, src;
  std::vector<double> vx, vy, vz;
  std::vector<double> xbg, ybg, zbg;
  // Verlet list, list(-3:max_list, natms) column-major -> ld = max_list+4
  std::vector<int> list;
  int ld = 0;
  bool lbook = false;
  int megfrz = 0;
  std::vector<int> list_excl;  // (max_exclude+1) x natms
  // vdW
  int nkey = 0;
  std::vector<int> vdw_kind;  // per key: 0 none, 1 lj
  std::vector<double> vdw_eps, vdw_sig;
  int max_grid = 0;
  double dlrpot = 0, rdr = 0;
  std::vector<double> vtab_pot, vtab_frc;  // (max_grid+1) per key
  double elrc = 0, vlrc = 0;
  // erfc tables (table(1:nsamples), 1-based)
  int nsamples = 0;
  double erfc_rdr = 0;
  std::vector<double> erfc_tab, erfcd_tab;
  // SPME
  double ncombk[22][21];
  std::vector<double> norm2[3];
  double self_interaction = 0;
  double scaling = 0;
  bool spme_newjob = true;
  // constraints
  int ntcons = 0;
  std::vector<int> con_type, con_i, con_j;  // i,j local 0-based
  std::vector<double> prmcon;
  std::vector<double> dxx, dyy, dzz;
  std::vector<int> listot;
  std::vector<char> lstitr;
  std::vector<double> oxt, oyt, ozt;
  // neighbour list update flag
  bool update = true;
  // thermostat (thermo%ensemble and its state)
  int ens = GB_NVE;
  double temp = 0, tau_t = 0, chi = 0, sigma = 0, qmass = 0, ceng = 0, totmas = 0;
  double chi_t = 0, cint = 0, consv = 0;
  int seed[3] = {0, 0, 0};
  int nstep = 0;
  // metals, tabulated EAM (met%tab = 1): tables by Fortran index, column 1 values, column 2 derivative
  bool metal = false, metal_unsafe = false;
  bool spme_on = true;   // electrostatics present (any charge): coul_method spme
  std::vector<std::vector<double>> vmet1, vmet2, dmet1, dmet2, fmet1, fmet2;  // per key / per type
  std::vector<int> met_listed;
  std::vector<double> mrho;
  double engmet = 0, virmet = 0, engden = 0, virden = 0;
};

Ctx g;
// Host threads of the OpenMP build; kept outside Ctx so that orc_init does not reset it.
int g_nthreads = 1;

// ---------------------------------------------------------------- numerics
// dcell: source/numerics.F90:1344-1443
void dcell(const double* aaa, double* bbb) {
  bbb[0] = std::sqrt(aaa[0] * aaa[0] + aaa[1] * aaa[1] + aaa[2] * aaa[2]);
  bbb[1] = std::sqrt(aaa[3] * aaa[3] + aaa[4] * aaa[4] + aaa[5] * aaa[5]);
  bbb[2] = std::sqrt(aaa[6] * aaa[6] + aaa[7] * aaa[7] + aaa[8] * aaa[8]);
  bbb[3] = (aaa[0] * aaa[3] + aaa[1] * aaa[4] + aaa[2] * aaa[5]) / (bbb[0] * bbb[1]);
  bbb[4] = (aaa[0] * aaa[6] + aaa[1] * aaa[7] + aaa[2] * aaa[8]) / (bbb[0] * bbb[2]);
  bbb[5] = (aaa[3] * aaa[6] + aaa[4] * aaa[7] + aaa[5] * aaa[8]) / (bbb[1] * bbb[2]);
  double axb1 = aaa[1] * aaa[5] - aaa[2] * aaa[4];
  double axb2 = aaa[2] * aaa[3] - aaa[0] * aaa[5];
  double axb3 = aaa[0] * aaa[4] - aaa[1] * aaa[3];
  double bxc1 = aaa[4] * aaa[8] - aaa[5] * aaa[7];
  double bxc2 = aaa[5] * aaa[6] - aaa[3] * aaa[8];
  double bxc3 = aaa[3] * aaa[7] - aaa[4] * aaa[6];
  double cxa1 = aaa[7] * aaa[2] - aaa[8] * aaa[1];
  double cxa2 = aaa[8] * aaa[0] - aaa[6] * aaa[2];
  double cxa3 = aaa[6] * aaa[1] - aaa[7] * aaa[0];
  bbb[9] = std::fabs(aaa[0] * bxc1 + aaa[1] * bxc2 + aaa[2] * bxc3);
  double d[3];
  d[0] = bbb[9] / std::sqrt(bxc1 * bxc1 + bxc2 * bxc2 + bxc3 * bxc3);
  d[1] = bbb[9] / std::sqrt(cxa1 * cxa1 + cxa2 * cxa2 + cxa3 * cxa3);
  d[2] = bbb[9] / std::sqrt(axb1 * axb1 + axb2 * axb2 + axb3 * axb3);
  double x[3], yv[3];
  x[0] = std::fabs(aaa[0]) / bbb[0]; yv[0] = std::fabs(aaa[1]) / bbb[0];
  x[1] = std::fabs(aaa[3]) / bbb[1]; yv[1] = std::fabs(aaa[4]) / bbb[1];
  x[2] = std::fabs(aaa[6]) / bbb[2]; yv[2] = std::fabs(aaa[7]) / bbb[2];
  if (x[0] >= x[1] && x[0] >= x[2]) {
    bbb[6] = d[0];
    if (yv[1] >= yv[2]) { bbb[7] = d[1]; bbb[8] = d[2]; } else { bbb[7] = d[2]; bbb[8] = d[1]; }
  } else if (x[1] >= x[0] && x[1] >= x[2]) {
    bbb[6] = d[1];
    if (yv[0] >= yv[2]) { bbb[7] = d[0]; bbb[8] = d[2]; } else { bbb[7] = d[2]; bbb[8] = d[0]; }
  } else {
    bbb[6] = d[2];
    if (yv[0] >= yv[1]) { bbb[7] = d[0]; bbb[8] = d[1]; } else { bbb[7] = d[1]; bbb[8] = d[0]; }
  }
}

// invert: source/numerics.F90:1445-1509
void invert(const double* a, double* b, double* d) {
  b[0] = a[4] * a[8] - a[5] * a[7];
  b[1] = a[2] * a[7] - a[1] * a[8];
  b[2] = a[1] * a[5] - a[2] * a[4];
  b[3] = a[5] * a[6] - a[3] * a[8];
  b[4] = a[0] * a[8] - a[2] * a[6];
  b[5] = a[2] * a[3] - a[0] * a[5];
  b[6] = a[3] * a[7] - a[4] * a[6];
  b[7] = a[1] * a[6] - a[0] * a[7];
  b[8] = a[0] * a[4] - a[1] * a[3];
  *d = a[0] * b[0] + a[3] * b[1] + a[6] * b[2];
  double r = 0.0;
  if (std::fabs(*d) > 0.0) r = 1.0 / *d;
  for (int i = 0; i < 9; ++i) b[i] = r * b[i];
}

// images, cubic/orthorhombic branches: source/numerics.F90:1511-1540
void images1(double* xx, double* yy, double* zz) {
  const double* c = g.cell;
  bool cubic = (c[0] == c[4] && c[0] == c[8]);
  double aaa = 1.0 / c[0];
  if (cubic) {
    *xx = *xx - c[0] * anint(aaa * *xx);
    *yy = *yy - c[0] * anint(aaa * *yy);
    *zz = *zz - c[0] * anint(aaa * *zz);
  } else {
    double bbb = 1.0 / c[4], ccc = 1.0 / c[8];
    *xx = *xx - c[0] * anint(aaa * *xx);
    *yy = *yy - c[4] * anint(bbb * *yy);
    *zz = *zz - c[8] * anint(ccc * *zz);
  }
}

// pbcshift_parts, cubic branch: source/numerics.F90:1886-1907
void pbcshift() {
  const double* c = g.cell;
  if (c[0] == c[4] && c[0] == c[8]) {
    double aaa = 1.0 / c[0];
    for (int i = 0; i < g.natms; ++i) {
      double xss = aaa * g.x[i], yss = aaa * g.y[i], zss = aaa * g.z[i];
      xss = xss - anint(xss); if (xss >= kHalfMinus) xss = -xss;
      yss = yss - anint(yss); if (yss >= kHalfMinus) yss = -yss;
      zss = zss - anint(zss); if (zss >= kHalfMinus) zss = -zss;
      g.x[i] = c[0] * xss; g.y[i] = c[0] * yss; g.z[i] = c[0] * zss;
    }
  } else {  // orthorhombic branch (numerics.F90:1909-1930)
    double aaa = 1.0 / c[0], bbb = 1.0 / c[4], ccc = 1.0 / c[8];
    for (int i = 0; i < g.natms; ++i) {
      double xss = aaa * g.x[i], yss = bbb * g.y[i], zss = ccc * g.z[i];
      xss = xss - anint(xss); if (xss >= kHalfMinus) xss = -xss;
      yss = yss - anint(yss); if (yss >= kHalfMinus) yss = -yss;
      zss = zss - anint(zss); if (zss >= kHalfMinus) zss = -zss;
      g.x[i] = c[0] * xss; g.y[i] = c[4] * yss; g.z[i] = c[8] * zss;
    }
  }
}

// calc_erfc_n / calc_erfc_deriv_n: source/numerics.F90:3647-3683
double calc_erfc_n(double x) {
  const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741, a4 = -1.453152027,
               a5 = 1.061405429, pp = 0.3275911;
  double tt = 1.0 / (1.0 + pp * x);
  return tt * (a1 + tt * (a2 + tt * (a3 + tt * (a4 + tt * a5)))) * std::exp(-(x * x));
}
double calc_erfc_deriv_n(double x) { return 2.0 * std::exp(-(x * x)) * kRsqrpi; }

// three_p_interp: source/numerics.F90:250-290; tab is 1-based (tab[0] unused)
inline double three_p(const double* tab, double rdr, double point) {
  int k = fint(point * rdr);
  double diff = point * rdr - (double)k;
  double p1 = tab[k], p2 = tab[k + 1], p3 = tab[k + 2];
  if (k == 0) p1 = p1 * point;
  double t1 = p1 + (p2 - p1) * diff;
  double t2 = p2 + (p3 - p2) * (diff - 1.0);
  return t1 + (t2 - t1) * diff * 0.5;
}

// lj_energy: source/two_body_potentials.F90:260-270
void lj_energy(double eps, double sig, double r, double* e, double* gam) {
  double sor = sig / r;
  double sor6 = sor * sor * sor * sor * sor * sor;
  *e = 4.0 * eps * sor6 * (sor6 - 1.0);
  *gam = 24.0 * eps * sor6 * (2.0 * sor6 - 1.0);
}

int vdw_key(int ai, int aj) { return ai > aj ? ai * (ai - 1) / 2 + aj : aj * (aj - 1) / 2 + ai; }

// --------------------------------------------------------------- tables
// erfcgen: source/electrostatic.F90:88-127 with init_interp_table numerics.F90:215-248
void erfcgen() {
  int n = g.nsamples;
  g.erfc_tab.assign(n + 3, 0.0);
  g.erfcd_tab.assign(n + 3, 0.0);
  double spacing = g.p.rcut / (double)(n - 4);
  g.erfc_rdr = 1.0 / spacing;
  const double alpha = g.p.alpha;
  for (int i = 1; i <= n; ++i) {
    double r = (double)i * spacing;
    double ef = calc_erfc_n(alpha * r) / r;
    g.erfc_tab[i] = ef;
    double rsq = r * r;
    g.erfcd_tab[i] = (calc_erfc_n(alpha * r) / r + alpha * calc_erfc_deriv_n(alpha * r)) / rsq;
  }
}

// vdw_generate: source/vdw.F90:1397-1460 (non-tabulated potentials branch)
void vdw_generate() {
  int mg = g.max_grid;
  g.dlrpot = g.p.rvdw / (double)(mg - 4);
  g.rdr = 1.0 / g.dlrpot;
  g.vtab_pot.assign((size_t)(mg + 3) * g.nkey, 0.0);
  g.vtab_frc.assign((size_t)(mg + 3) * g.nkey, 0.0);
  for (int k = 0; k < g.nkey; ++k) {
    double* vp = &g.vtab_pot[(size_t)k * (mg + 3)];
    double* vf = &g.vtab_frc[(size_t)k * (mg + 3)];
    if (g.vdw_kind[k] != 1) continue;  // tab_potential(0,k) stays 0 -> pair skipped
    for (int i = 1; i <= mg; ++i) {
      double r = (double)i * g.dlrpot, e, gm;
      lj_energy(g.vdw_eps[k], g.vdw_sig[k], r, &e, &gm);
      vp[i] = e;
      vf[i] = gm;
    }
    vp[0] = DBL_MAX;
    vf[0] = DBL_MAX;
  }
}

// vdw_lrc, LJ branch: source/vdw.F90:617-720 (energy/virial long-range correction)
void vdw_lrc() {
  std::vector<double> numtyp(g.p.ntypes + 1, 0.0);
  for (int i = 0; i < g.natms; ++i) numtyp[g.ltype[i]] += 1.0;
  double elrc = 0, plrc = 0;
  int ivdw = 0;
  for (int i = 1; i <= g.p.ntypes; ++i)
    for (int j = 1; j <= i; ++j) {
      int k = ivdw++;
      if (g.vdw_kind[k] != 1) continue;
      double eps = g.vdw_eps[k], sig = g.vdw_sig[k], r = g.p.rvdw;
      double eadd = 4.0 * eps * (std::pow(sig, 12) / (9.0 * std::pow(r, 9)) - std::pow(sig, 6) / (3.0 * r * r * r));
      double padd = 8.0 * eps * (6.0 * std::pow(sig, 12) / (9.0 * std::pow(r, 9)) - std::pow(sig, 6) / (r * r * r));
      if (i != j) { eadd *= 2.0; padd *= 2.0; }
      double denprd = 2.0 * kPi * (numtyp[i] * numtyp[j]) / (g.volm * g.volm);
      elrc += g.volm * denprd * eadd;
      plrc += denprd * padd / 3.0;
    }
  g.elrc = elrc;
  g.vlrc = plrc * (-3.0 * g.volm);
}

// ------------------------------------------------------------ halo images
// export_atomic_data, serial form: source/deport_data.F90:1673-1900
void export_atomic_data(int mdir) {
  int kx = 0, ky = 0, kz = 0, jxyz = 0, kxyz = 0;
  double uuu = 0, vvv = 0, www = 0;
  switch (mdir) {
    case -1: kx = 1; jxyz = 1; kxyz = 3; uuu = +1.0; break;
    case 1: kx = 1; jxyz = 2; kxyz = 3; uuu = -1.0; break;
    case -2: ky = 1; jxyz = 10; kxyz = 30; vvv = +1.0; break;
    case 2: ky = 1; jxyz = 20; kxyz = 30; vvv = -1.0; break;
    case -3: kz = 1; jxyz = 100; kxyz = 300; www = +1.0; break;
    case 3: kz = 1; jxyz = 200; kxyz = 300; www = -1.0; break;
  }
  const double* c = g.cell;
  double xadd = c[0] * uuu + c[3] * vvv + c[6] * www;
  double yadd = c[1] * uuu + c[4] * vvv + c[7] * www;
  double zadd = c[2] * uuu + c[5] * vvv + c[8] * www;
  int n0 = g.nlast;
  std::vector<int> sel;
  for (int i = 0; i < n0; ++i) {
    int v = g.ixyz[i];
    if (v > 0) {
      int ix = v % 10;
      int iy = (v - ix) % 100;
      int iz = (v - (ix + iy)) % 1000;
      int j = ix * kx + iy * ky + iz * kz;
      if (j == jxyz || (j > jxyz && j % 3 == 0)) sel.push_back(i);
    }
  }
  if (g.nlast + (int)sel.size() > g.mxatms) throw GB_ERR_HALO;
  for (int i : sel) {
    int n = g.nlast++;
    g.x[n] = g.x[i] + xadd;
    g.y[n] = g.y[i] + yadd;
    g.z[n] = g.z[i] + zadd;
    g.ltg[n] = g.ltg[i];
    g.src[n] = g.src[i];
    int v = g.ixyz[i];
    int ix = v % 10, iy = (v - ix) % 100, iz = (v - (ix + iy)) % 1000;
    int j = ix * kx + iy * ky + iz * kz;
    g.ixyz[n] = v - (j == jxyz ? jxyz : kxyz);
  }
}

// export_atomic_positions (refresh, same halo set): source/deport_data.F90 +
// refresh_halo_positions halo.F90:47-114.  Halo atoms keep their source and
// shift; positions are recomputed with the same additions.
void refresh_halo_positions() {
  // Re-run the export chain over the stored ixyz of the local atoms; the halo
  // ordering and membership are unchanged, only positions move.
  int nl = g.nlast;
  std::vector<int> ixyz0(g.ixyz.begin(), g.ixyz.begin() + nl);
  g.nlast = g.natms;
  for (int i = 0; i < g.natms; ++i) g.ixyz[i] = ixyz0[i];
  for (int m : {-1, 1, -2, 2, -3, 3}) export_atomic_data(m);
  if (g.nlast != nl) throw 138;
}

// set_halo_particles: source/halo.F90:153-356 (serial: one domain)
void set_halo_particles() {
  double cut = g.rcutx + 1.0e-6;
  double cp[10];
  dcell(g.cell, cp);
  int nlx = fint(cp[6] / (cut * 1.0));
  int nly = fint(cp[7] / (cut * 1.0));
  int nlz = fint(cp[8] / (cut * 1.0));
  double xdc = (double)(nlx * 1), ydc = (double)(nly * 1), zdc = (double)(nlz * 1);
  double cwx = 1.0 / xdc, cwy = 1.0 / ydc, cwz = 1.0 / zdc;
  double ecwx = cwx, ecwy = cwy, ecwz = cwz;
  if (g.spme_on) {  // halo.F90:218-231: only with SPME electrostatics
    ecwx = std::max(cwx, (double)g.p.spline_pad / (double)g.p.kmax[0]);
    ecwy = std::max(cwy, (double)g.p.spline_pad / (double)g.p.kmax[1]);
    ecwz = std::max(cwz, (double)g.p.spline_pad / (double)g.p.kmax[2]);
  }
  ecwx = std::nextafter((-0.5 + ecwx) + 0.0 * 1.0, 2.0) + kZeroPlus;
  ecwy = std::nextafter((-0.5 + ecwy) + 0.0 * 1.0, 2.0) + kZeroPlus;
  ecwz = std::nextafter((-0.5 + ecwz) + 0.0 * 1.0, 2.0) + kZeroPlus;
  cwx = std::nextafter((-0.5 - cwx) + 1.0 * 1.0, -2.0) - kZeroPlus - (nlx == 1 ? cwx * 1.0e-10 : 0.0);
  cwy = std::nextafter((-0.5 - cwy) + 1.0 * 1.0, -2.0) - kZeroPlus - (nly == 1 ? cwy * 1.0e-10 : 0.0);
  cwz = std::nextafter((-0.5 - cwz) + 1.0 * 1.0, -2.0) - kZeroPlus - (nlz == 1 ? cwz * 1.0e-10 : 0.0);
  double rc[9], det;
  invert(g.cell, rc, &det);
  g.nlast = g.natms;
  for (int i = 0; i < g.nlast; ++i) {
    g.ixyz[i] = 0;
    double xx = rc[0] * g.x[i] + rc[3] * g.y[i] + rc[6] * g.z[i];
    double yy = rc[1] * g.x[i] + rc[4] * g.y[i] + rc[7] * g.z[i];
    double zz = rc[2] * g.x[i] + rc[5] * g.y[i] + rc[8] * g.z[i];
    if (xx <= ecwx) g.ixyz[i] += 1;
    if (xx >= cwx) g.ixyz[i] += 2;
    if (yy <= ecwy) g.ixyz[i] += 10;
    if (yy >= cwy) g.ixyz[i] += 20;
    if (zz <= ecwz) g.ixyz[i] += 100;
    if (zz >= cwz) g.ixyz[i] += 200;
  }
  for (int m : {-1, 1, -2, 2, -3, 3}) export_atomic_data(m);
  for (int i = g.natms; i < g.nlast; ++i) {
    int s = g.src[i];
    g.ltype[i] = g.ltype[s];
    g.chge[i] = g.chge[s];
    g.weight[i] = g.weight[s];
    g.lfrzn[i] = g.lfrzn[s];
  }
  // vnl_set_check: neighbours.F90:305-343
  for (int i = 0; i < g.nlast; ++i) { g.xbg[i] = g.x[i]; g.ybg[i] = g.y[i]; g.zbg[i] = g.z[i]; }
}

// ------------------------------------------------------------ Verlet list
inline int& L(int k, int i) { return g.list[(size_t)i * g.ld + (k + 3)]; }  // list(k, i+1)

bool match_sorted(int n, int top, const int* lst) {
  for (int k = 0; k < top; ++k) if (lst[k] == n) return true;
  return false;
}

// link_cell_pairs: source/neighbours.F90:356-1414 (serial, not HALF_HALO)
int link_cell_pairs() {
  double cp[10];
  dcell(g.cell, cp);
  double det = std::min(cp[6], std::min(cp[7], cp[8]));
  if (g.rcutx >= det / 2.0) return GB_ERR_CUTOFF_CELL;
  double cut = g.rcutx + kSmalldr;
  double rcsq = g.rcutx * g.rcutx;
  double dispx = 1.0 * cp[6] / cut, dispy = 1.0 * cp[7] / cut, dispz = 1.0 * cp[8] / cut;
  int nlx = fint(dispx), nly = fint(dispy), nlz = fint(dispz);
  if (nlx * nly * nlz == 0) return GB_ERR_LINK_CELLS;
  int nlp = 1;
  double nlr2 = (double)g.natms;
  det = nlr2 / (double)(nlx * nly * nlz);
  while (det > g.p.pdplnc) {
    nlp = nlp + 1;
    double rsq = (double)nlp;
    nlx = fint(dispx * rsq); nly = fint(dispy * rsq); nlz = fint(dispz * rsq);
    det = nlr2 / (double)(nlx * nly * nlz);
  }
  const int NX = nlx + 2 * nlp, NY = nly + 2 * nlp, NZ = nlz + 2 * nlp;
  const int ncells = NX * NY * NZ;
  // semi-ball offsets (neighbours.F90:490-540)
  std::vector<int> nix, niy, niz;
  std::vector<char> nir;
  {
    int nlp2 = nlp * nlp, nlp3 = (nlp - 1) * (nlp - 1);
    for (int iz = 0; iz <= nlp; ++iz) {
      int iz1 = iz > 0 ? (iz - 1) * (iz - 1) : 0;
      int jz = iz * iz;
      for (int iy = -nlp; iy <= nlp; ++iy) {
        if (iz == 0 && iy < 0) continue;
        int a = std::abs(iy);
        int iy1 = a > 0 ? (a - 1) * (a - 1) : 0;
        int ll = iz1 + iy1;
        if (ll > nlp2) continue;
        int jy = jz + iy * iy;
        for (int ix = -nlp; ix <= nlp; ++ix) {
          if (iz == 0 && iy == 0 && ix < 0) continue;
          int b = std::abs(ix);
          int ix1 = b > 0 ? (b - 1) * (b - 1) : 0;
          if (ll + ix1 > nlp2) continue;
          int jx = jy + ix * ix;
          nix.push_back(ix); niy.push_back(iy); niz.push_back(iz);
          nir.push_back(jx < nlp3);
        }
      }
    }
  }
  const int nsbcll = (int)nix.size();
  double xdc = (double)(nlx * 1), ydc = (double)(nly * 1), zdc = (double)(nlz * 1);
  int jx0 = nlp, jy0 = nlp, jz0 = nlp;
  const int nlx0s = 0, nly0s = 0, nlz0s = 0;
  const int nlx0e = nlp - 1, nly0e = nlp - 1, nlz0e = nlp - 1;
  const int nlx1s = nlx + nlp, nly1s = nly + nlp, nlz1s = nlz + nlp;
  const int nlx1e = nlx + 2 * nlp - 1, nly1e = nly + 2 * nlp - 1, nlz1e = nlz + 2 * nlp - 1;
  std::vector<int> lct_count(ncells + 2, 0), lct_start(ncells + 2, 0), which_cell(g.nlast);
  double rc[9];
  invert(g.cell, rc, &det);
  for (int i = 0; i < g.natms; ++i) {
    double xx = rc[0] * g.x[i] + rc[3] * g.y[i] + rc[6] * g.z[i];
    double yy = rc[1] * g.x[i] + rc[4] * g.y[i] + rc[7] * g.z[i];
    double zz = rc[2] * g.x[i] + rc[5] * g.y[i] + rc[8] * g.z[i];
    int ix = fint(xdc * (xx + 0.5)) + jx0;
    int iy = fint(ydc * (yy + 0.5)) + jy0;
    int iz = fint(zdc * (zz + 0.5)) + jz0;
    ix = std::max(std::min(ix, nlx1s - 1), nlx0e + 1);
    iy = std::max(std::min(iy, nly1s - 1), nly0e + 1);
    iz = std::max(std::min(iz, nlz1s - 1), nlz0e + 1);
    int icell = 1 + ix + NX * (iy + NY * iz);
    lct_count[icell]++;
    which_cell[i] = icell;
  }
  for (int i = g.natms; i < g.nlast; ++i) {
    double xx = rc[0] * g.x[i] + rc[3] * g.y[i] + rc[6] * g.z[i];
    double yy = rc[1] * g.x[i] + rc[4] * g.y[i] + rc[7] * g.z[i];
    double zz = rc[2] * g.x[i] + rc[5] * g.y[i] + rc[8] * g.z[i];
    double dx, dy, dz;
    int ix, iy, iz;
    if (xx > -kHalfPlus) { dx = xdc * (xx + 0.5); ix = fint(dx) + jx0; }
    else { dx = xdc * std::fabs(xx + 0.5); ix = -fint(dx) + jx0 - 1; }
    if (yy > -kHalfPlus) { dy = ydc * (yy + 0.5); iy = fint(dy) + jy0; }
    else { dy = ydc * std::fabs(yy + 0.5); iy = -fint(dy) + jy0 - 1; }
    if (zz > -kHalfPlus) { dz = zdc * (zz + 0.5); iz = fint(dz) + jz0; }
    else { dz = zdc * std::fabs(zz + 0.5); iz = -fint(dz) + jz0 - 1; }
    int icell;
    if (ix >= nlx0s && iy >= nly0s && iz >= nlz0s) {
      bool lx0 = ix > nlx0e, lx1 = ix < nlx1s, ly0 = iy > nly0e, ly1 = iy < nly1s, lz0 = iz > nlz0e,
           lz1 = iz < nlz1s;
      if ((lx0 && lx1) && (ly0 && ly1) && (lz0 && lz1)) {
        // put on border in the halo (neighbours.F90:705-755)
        double x0 = std::fabs(dx - (double)(nlx * 0)), x1 = std::fabs(dx - (double)(nlx * 1));
        dx = std::min(x0, x1);
        double y0 = std::fabs(dy - (double)(nly * 0)), y1 = std::fabs(dy - (double)(nly * 1));
        dy = std::min(y0, y1);
        double z0 = std::fabs(dz - (double)(nlz * 0)), z1 = std::fabs(dz - (double)(nlz * 1));
        dz = std::min(z0, z1);
        if (dx <= dy && dx <= dz) {
          ix = x0 < x1 ? nlx0e : nlx1s;
          if (std::fabs(dx - dy) < kEpsWp) iy = y0 < y1 ? nly0e : nly1s;
          if (std::fabs(dx - dz) < kEpsWp) iz = z0 < z1 ? nlz0e : nlz1s;
        } else if (dy <= dx && dy <= dz) {
          iy = y0 < y1 ? nly0e : nly1s;
          if (std::fabs(dy - dz) < kEpsWp) iz = z0 < z1 ? nlz0e : nlz1s;
        } else {
          iz = z0 < z1 ? nlz0e : nlz1s;
        }
      }
      bool out = ix < nlx0s || ix > nlx1e || iy < nly0s || iy > nly1e || iz < nlz0s || iz > nlz1e;
      icell = out ? 0 : 1 + ix + NX * (iy + NY * iz);
    } else {
      icell = 0;
    }
    lct_count[icell]++;
    which_cell[i] = icell;
  }
  // counting sort (neighbours.F90:803-823); lct_start is 1-based positions
  lct_start[0] = 1;
  for (int c = 1; c <= ncells + 1; ++c) lct_start[c] = lct_start[c - 1] + lct_count[c - 1];
  std::vector<int> lct_where(lct_start);
  std::vector<int> at_list(g.nlast + 1);
  std::vector<double> xxt(g.nlast + 1), yyt(g.nlast + 1), zzt(g.nlast + 1);
  for (int i = 0; i < g.nlast; ++i) {
    int j = lct_where[which_cell[i]];
    at_list[j] = i;  // 0-based atom index at 1-based slot j
    xxt[j] = g.x[i]; yyt[j] = g.y[i]; zzt[j] = g.z[i];
    lct_where[which_cell[i]]++;
  }
  // domain and border cells (neighbours.F90:825-857)
  std::vector<int> cell_dom, cell_bor;
  for (int iz = nlz0e + 1; iz <= nlz1s - 1; ++iz) {
    int iz1 = iz - nlz0e, iz2 = iz - nlz1s;
    for (int iy = nly0e + 1; iy <= nly1s - 1; ++iy) {
      int iy1 = iy - nly0e, iy2 = iy - nly1s;
      for (int ix = nlx0e + 1; ix <= nlx1s - 1; ++ix) {
        int ix1 = ix - nlx0e, ix2 = ix - nlx1s;
        int ic = 1 + ix + NX * (iy + NY * iz);
        cell_dom.push_back(ic);
        if ((ix1 >= 1 && ix1 <= nlp) || (ix2 <= -1 && ix2 >= -nlp) || (iy1 >= 1 && iy1 <= nlp) ||
            (iy2 <= -1 && iy2 >= -nlp) || (iz1 >= 1 && iz1 <= nlp) || (iz2 <= -1 && iz2 >= -nlp))
          cell_bor.push_back(ic);
      }
    }
  }
  const int max_list = g.p.max_list;
  for (int i = 0; i < g.natms; ++i) { L(-2, i) = 0; L(-1, i) = 0; L(0, i) = 0; L(-3, i) = 0; }
  int ibig = 0;
  bool safe = true;
  auto add = [&](int i, int j) {
    int ll = L(0, i) + 1;
    if (ll <= max_list) L(ll, i) = j + 1;
    else { ibig = std::max(ibig, ll); safe = false; }
    L(0, i) = ll;
  };
  // pass 1 (neighbours.F90:876-1027)
  for (int ic : cell_dom) {
    int ix = (ic - 1) % NX;
    int iz = (ic - 1) / (NX * NY);
    int iy = (ic - 1) / NX - NY * iz;
    for (int ii = lct_start[ic]; ii <= lct_start[ic + 1] - 1; ++ii) {
      int i = at_list[ii];
      for (int kk = 0; kk < nsbcll; ++kk) {
        int jx = ix + nix[kk], jy = iy + niy[kk], jz = iz + niz[kk];
        int jc = 1 + jx + NX * (jy + NY * jz);
        int j_start = (jc != ic) ? lct_start[jc] : ii + 1;
        if (nir[kk]) {
          for (int jj = j_start; jj <= lct_start[jc + 1] - 1; ++jj) add(i, at_list[jj]);
        } else {
          for (int jj = j_start; jj <= lct_start[jc + 1] - 1; ++jj) {
            double rsq = (xxt[jj] - g.x[i]) * (xxt[jj] - g.x[i]) + (yyt[jj] - g.y[i]) * (yyt[jj] - g.y[i]) +
                         (zzt[jj] - g.z[i]) * (zzt[jj] - g.z[i]);
            if (rsq <= rcsq) add(i, at_list[jj]);
          }
        }
      }
    }
  }
  // pass 2 (neighbours.F90:1032-1184)
  for (int ic : cell_bor) {
    int ix = (ic - 1) % NX;
    int iz = (ic - 1) / (NX * NY);
    int iy = (ic - 1) / NX - NY * iz;
    for (int ii = lct_start[ic]; ii <= lct_start[ic + 1] - 1; ++ii) {
      int i = at_list[ii];
      for (int kk = 1; kk < nsbcll; ++kk) {
        int jx = ix - nix[kk], jy = iy - niy[kk], jz = iz - niz[kk];
        if (jx <= nlx0e || jx >= nlx1s || jy <= nly0e || jy >= nly1s || jz <= nlz0e || jz >= nlz1s) {
          int jc = 1 + jx + NX * (jy + NY * jz);
          int j_start = lct_start[jc];
          if (nir[kk]) {
            for (int jj = j_start; jj <= lct_start[jc + 1] - 1; ++jj) add(i, at_list[jj]);
          } else {
            for (int jj = j_start; jj <= lct_start[jc + 1] - 1; ++jj) {
              double rsq = (xxt[jj] - g.x[i]) * (xxt[jj] - g.x[i]) + (yyt[jj] - g.y[i]) * (yyt[jj] - g.y[i]) +
                           (zzt[jj] - g.z[i]) * (zzt[jj] - g.z[i]);
              if (rsq <= rcsq) add(i, at_list[jj]);
            }
          }
        }
      }
    }
  }
  if (!safe) {
    g.p.max_list = ibig;  // report needed size through the same field
    return GB_ERR_LIST_OVERFLOW;
  }
  // frozen pairs (neighbours.F90:1198-1225)
  for (int i = 0; i < g.natms; ++i) {
    int l_end = L(0, i), m_end = l_end;
    if (g.megfrz > 1 && g.lfrzn[i] > 0) {
      for (int kk = l_end; kk >= 1; --kk) {
        int j = L(kk, i);
        if (g.lfrzn[j - 1] > 0) {
          if (kk < m_end) { L(kk, i) = L(m_end, i); L(m_end, i) = j; }
          m_end--;
        }
      }
    }
    L(-2, i) = L(0, i);
    L(0, i) = m_end;
  }
  // excluded pairs (neighbours.F90:1229-1306)
  const int ldx = g.p.max_exclude + 1;
  for (int i = 0; i < g.natms; ++i) {
    if (g.lbook) {
      int l_end = L(0, i), m_end = l_end;
      int ii = g.list_excl[(size_t)i * ldx];
      if (ii > 0) {
        const int* ex = &g.list_excl[(size_t)i * ldx + 1];
        for (int kk = l_end; kk >= 1; --kk) {
          int j = L(kk, i);
          int jj = g.ltg[j - 1];
          if (match_sorted(jj, ii, ex)) {
            if (kk < m_end) { L(kk, i) = L(m_end, i); L(m_end, i) = j; }
            m_end--;
          }
        }
      }
      L(-1, i) = L(0, i);
      L(0, i) = m_end;
      L(-3, i) = L(0, i);
    } else {
      L(-1, i) = L(0, i);
      L(-3, i) = L(0, i);
    }
  }
  return GB_OK;
}

// --------------------------------------------------------------- two-body
struct Acc {
  double engvdw = 0, virvdw = 0, engrl = 0, virrl = 0, engex = 0, virex = 0;
  double str[9] = {0};
};

// two_body_forces pair loop: source/two_body.F90:339-606 with
// vdw_forces_tab (vdw.F90:1790-2024) / vdw_forces_direct (vdw.F90:1578-1788),
// ewald_real_forces_coul (ewald_spole.F90:58-242) and ewald_excl_forces
// (ewald_spole.F90:479-679).  fxo/fyo/fzo are the force arrays to add into.
void pair_loop(int i0, int i1, double* fxo, double* fyo, double* fzo, Acc& A) {
  const int mg = g.max_grid;
  const double scaling = g.scaling;
  const double rcut = g.p.rcut, rvdw = g.p.rvdw;
  std::vector<double> xt(g.p.max_list + 1), yt(g.p.max_list + 1), zt(g.p.max_list + 1), rt(g.p.max_list + 1);
  for (int i = i0; i < i1; ++i) {
    int limit = L(0, i);
    for (int k = 1; k <= limit; ++k) {
      int j = L(k, i) - 1;
      xt[k] = g.x[i] - g.x[j];
      yt[k] = g.y[i] - g.y[j];
      zt[k] = g.z[i] - g.z[j];
      rt[k] = std::sqrt(xt[k] * xt[k] + yt[k] * yt[k] + zt[k] * zt[k]);
    }
    const int idi = g.ltg[i];
    // --- vdW
    {
      int ai = g.ltype[i];
      double fix = fxo[i], fiy = fyo[i], fiz = fzo[i];
      double s1 = 0, s2 = 0, s3 = 0, s5 = 0, s6 = 0, s9 = 0, eng = 0, vir = 0;
      for (int m = 1; m <= limit; ++m) {
        int j = L(m, i) - 1;
        int aj = g.ltype[j];
        int key = vdw_key(ai, aj) - 1;
        const double* vp = &g.vtab_pot[(size_t)key * (mg + 3)];
        const double* vf = &g.vtab_frc[(size_t)key * (mg + 3)];
        if (g.p.vdw_direct == 0 && std::fabs(vp[0]) < kZeroPlus) continue;
        double rrr = rt[m];
        if (g.vdw_kind[key] != 0 && rrr < rvdw) {
          double r_rrr = 1.0 / rrr;
          double rsq = rrr * rrr;
          double r_rsq = r_rrr * r_rrr;
          double e, gamma;
          if (g.p.vdw_direct == 0) {
            int l = fint(rrr * g.rdr);
            double ppp = rrr * g.rdr - (double)l;
            double gk = vf[l]; if (l == 0) gk = gk * rrr;
            double gk1 = vf[l + 1], gk2 = vf[l + 2];
            double t1 = gk + (gk1 - gk) * ppp;
            double t2 = gk1 + (gk2 - gk1) * (ppp - 1.0);
            gamma = (t1 + (t2 - t1) * ppp * 0.5) * r_rsq;
            double vk = vp[l], vk1 = vp[l + 1], vk2 = vp[l + 2];
            t1 = vk + (vk1 - vk) * ppp;
            t2 = vk1 + (vk2 - vk1) * (ppp - 1.0);
            e = t1 + (t2 - t1) * ppp * 0.5;
          } else {
            double eg, gg;
            lj_energy(g.vdw_eps[key], g.vdw_sig[key], rrr, &eg, &gg);
            e = eg;
            gamma = gg * r_rsq;
          }
          double fx = gamma * xt[m], fy = gamma * yt[m], fz = gamma * zt[m];
          fix += fx; fiy += fy; fiz += fz;
          if (j < g.natms) { fxo[j] -= fx; fyo[j] -= fy; fzo[j] -= fz; }
          if (j < g.natms || idi < g.ltg[j]) {
            eng += e;
            vir -= gamma * rsq;
            s1 += xt[m] * fx; s2 += xt[m] * fy; s3 += xt[m] * fz;
            s5 += yt[m] * fy; s6 += yt[m] * fz; s9 += zt[m] * fz;
          }
        }
      }
      fxo[i] = fix; fyo[i] = fiy; fzo[i] = fiz;
      A.engvdw += eng; A.virvdw += vir;
      A.str[0] += s1; A.str[1] += s2; A.str[2] += s3; A.str[3] += s2; A.str[4] += s5;
      A.str[5] += s6; A.str[6] += s3; A.str[7] += s6; A.str[8] += s9;
    }
    // --- real-space Ewald
    {
      double atom_coeffs_i = g.chge[i] * scaling;
      if (!(std::fabs(atom_coeffs_i) < kZeroPlus)) {
        double f0 = 0, f1 = 0, f2 = 0, eng = 0, vir = 0;
        double st[6] = {0, 0, 0, 0, 0, 0};
        for (int m = 1; m <= limit; ++m) {
          int j = L(m, i) - 1;
          double rr = rt[m];
          double prefac = g.chge[j];
          if (std::fabs(prefac) > kZeroPlus && rr < rcut) {
            prefac = atom_coeffs_i * prefac;
            double erf_gamma = prefac * three_p(g.erfcd_tab.data(), g.erfc_rdr, rr);
            double fc0 = erf_gamma * xt[m], fc1 = erf_gamma * yt[m], fc2 = erf_gamma * zt[m];
            f0 += fc0; f1 += fc1; f2 += fc2;
            double e_comp = 0;
            if (j < g.natms || idi < g.ltg[j]) {
              if (j < g.natms) { fxo[j] -= fc0; fyo[j] -= fc1; fzo[j] -= fc2; }
              e_comp = prefac * three_p(g.erfc_tab.data(), g.erfc_rdr, rr);
              eng += e_comp;
              vir -= erf_gamma * rr * rr;
              st[0] += xt[m] * fc0; st[1] += xt[m] * fc1; st[2] += xt[m] * fc2;
              st[3] += yt[m] * fc1; st[4] += yt[m] * fc2; st[5] += zt[m] * fc2;
            }
          }
        }
        fxo[i] += f0; fyo[i] += f1; fzo[i] += f2;
        A.engrl += eng; A.virrl += vir;
        A.str[0] += st[0]; A.str[1] += st[1]; A.str[2] += st[2]; A.str[3] += st[1]; A.str[4] += st[3];
        A.str[5] += st[4]; A.str[6] += st[2]; A.str[7] += st[4]; A.str[8] += st[5];
      }
    }
  }
  // --- exclusion corrections (two_body.F90:552-606; ewald_spole.F90:479-679)
  if (g.lbook) {
    const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741, a4 = -1.453152027,
                 a5 = 1.061405429, pp = 0.3275911, r10 = 0.1, r216 = 1.0 / 216.0, r42 = 1.0 / 42.0,
                 rr3 = 1.0 / 3.0;
    const double alpha = g.p.alpha;
    for (int i = i0; i < i1; ++i) {
      int limit = L(-1, i) - L(0, i);
      if (limit <= 0) continue;
      double chgea = g.chge[i];
      if (!(std::fabs(chgea) > kZeroPlus)) continue;
      chgea = chgea * scaling;
      const int idi = g.ltg[i];
      double fix = fxo[i], fiy = fyo[i], fiz = fzo[i];
      double s1 = 0, s2 = 0, s3 = 0, s5 = 0, s6 = 0, s9 = 0;
      for (int m = 1; m <= limit; ++m) {
        int j = L(L(0, i) + m, i) - 1;
        double xx = g.x[i] - g.x[j], yy = g.y[i] - g.y[j], zz = g.z[i] - g.z[j];
        double rrr = std::sqrt(xx * xx + yy * yy + zz * zz);
        double chgprd = g.chge[j];
        if (std::fabs(chgprd) > kZeroPlus && rrr < rcut) {
          chgprd = chgprd * chgea;
          double rsq = rrr * rrr;
          double alpr = rrr * alpha;
          double alpr2 = alpr * alpr;
          double erfr, egamma;
          if (alpr < 1.0e-2) {
            erfr = 2.0 * chgprd * (alpha / kSqrpi) *
                   (1.0 + alpr2 * (-rr3 + alpr2 * (r10 + alpr2 * (-r42 + alpr2 * r216))));
            egamma = -4.0 * chgprd * (alpha * alpha * alpha / kSqrpi) *
                     (rr3 + alpr2 * (-2.0 * r10 + alpr2 * (3.0 * r42 - 4.0 * alpr2 * r216)));
          } else {
            double exp1 = std::exp(-(alpha * rrr) * (alpha * rrr));
            double tt = 1.0 / (1.0 + pp * alpha * rrr);
            erfr = chgprd * (1.0 - tt * (a1 + tt * (a2 + tt * (a3 + tt * (a4 + tt * a5)))) * exp1) / rrr;
            egamma = -(erfr - 2.0 * chgprd * (alpha / kSqrpi) * exp1) / rsq;
          }
          double fx = egamma * xx, fy = egamma * yy, fz = egamma * zz;
          fix += fx; fiy += fy; fiz += fz;
          if (j < g.natms) { fxo[j] -= fx; fyo[j] -= fy; fzo[j] -= fz; }
          if (j < g.natms || idi < g.ltg[j]) {
            A.engex -= erfr;
            A.virex -= egamma * rsq;
            s1 += xx * fx; s2 += xx * fy; s3 += xx * fz; s5 += yy * fy; s6 += yy * fz; s9 += zz * fz;
          }
        }
      }
      fxo[i] = fix; fyo[i] = fiy; fzo[i] = fiz;
      A.str[0] += s1; A.str[1] += s2; A.str[2] += s3; A.str[3] += s2; A.str[4] += s5;
      A.str[5] += s6; A.str[6] += s3; A.str[7] += s6; A.str[8] += s9;
    }
  }
}

// Pair loop over all local atoms; with OpenMP each thread accumulates into a
// private force array (the sum order changes, the arithmetic per pair does not).
void two_body_real(Acc& A) {
  const int nl = g.nlast;
#ifdef ORACLE_OPENMP
  int nt = g_nthreads;
  if (nt > 1) {
    std::vector<std::vector<double>> F(nt, std::vector<double>((size_t)3 * nl, 0.0));
    std::vector<Acc> As(nt);
#pragma omp parallel num_threads(nt)
    {
      int t = omp_get_thread_num();
      double* fx = F[t].data();
      int chunk = 64;
#pragma omp for schedule(dynamic, 1)
      for (int b = 0; b < (g.natms + chunk - 1) / chunk; ++b)
        pair_loop(b * chunk, std::min(g.natms, (b + 1) * chunk), fx, fx + nl, fx + 2 * nl, As[t]);
    }
    for (int t = 0; t < nt; ++t) {
      for (int i = 0; i < g.natms; ++i) {
        g.fx[i] += F[t][i]; g.fy[i] += F[t][nl + i]; g.fz[i] += F[t][2 * nl + i];
      }
      A.engvdw += As[t].engvdw; A.virvdw += As[t].virvdw; A.engrl += As[t].engrl;
      A.virrl += As[t].virrl; A.engex += As[t].engex; A.virex += As[t].virex;
      for (int k = 0; k < 9; ++k) A.str[k] += As[t].str[k];
    }
    return;
  }
#endif
  pair_loop(0, g.natms, g.fx.data(), g.fy.data(), g.fz.data(), A);
}

// ------------------------------------------------------------------- SPME
// bspline_coeffs_gen: source/bspline.F90:73-190 (+ spl_cexp :308-353)
void bspline_coeffs_gen() {
  const int s = g.p.nsplines;
  for (int n = 0; n < 22; ++n) for (int k = 0; k < 21; ++k) g.ncombk[n][k] = 0.0;
  for (int n = 1; n <= s; ++n)
    for (int k = 0; k <= n; ++k) {
      double a = 1.0, b = 1.0;
      for (int i = n - k + 1; i <= n; ++i) a *= (double)i;
      for (int i = 1; i <= std::max(1, k); ++i) b *= 1.0 / (double)i;
      g.ncombk[k][n] = a * b;
    }
  std::vector<double> cspline(s + 1, 0.0);
  cspline[2] = 1.0;
  for (int k = 3; k <= s; ++k)
    for (int j = k; j >= 2; --j)
      cspline[j] = ((double)(j - 1) * cspline[j] + (double)(k - j + 1) * cspline[j - 1]) * (1.0 / (double)(k - 1));
  for (int d = 0; d < 3; ++d) {
    int K = g.p.kmax[d];
    std::vector<std::complex<double>> ww(K);
    ww[0] = {1.0, 0.0};
    for (int i = 1; i <= K / 2; ++i) {
      double arg = (2.0 * kPi / (double)K) * (double)i;
      ww[i] = {std::cos(arg), std::sin(arg)};
      ww[K - i] = std::conj(ww[i]);
    }
    g.norm2[d].assign(K, 0.0);
    for (int i = 0; i < K; ++i) {
      std::complex<double> t(0.0, 0.0);
      for (int k = 0; k <= s - 2; ++k) t += cspline[k + 2] * ww[(size_t)(((long)i * k) % K)];
      std::complex<double> c = ww[(size_t)(((long)i * (s - 1)) % K)] / t;
      g.norm2[d][i] = (c * std::conj(c)).real();
    }
  }
}

// bspline_splines_gen for one atom and one dimension: source/bspline.F90:192-306.
// d[0..2][1..s]: derivative order 0..2 at spline points 1..s.
void splines_1d(double u, double d[3][21]) {
  const int s = g.p.nsplines;
  const int nd = 2;
  double zd[22], fd[22];
  for (int j = 0; j <= s + 1; ++j) zd[j] = 0.0;
  zd[s] = u - std::trunc(u);
  zd[s - 1] = 1.0 - zd[s];
  double centre = zd[s];
  for (int k = s - 2; k >= nd + 1; --k) {
    double k_r = (double)(s - k + 1);
    double km1_rr = 1.0 / (double)(s - k);
    for (int j = k; j <= s - 1; ++j) {
      double pt = centre + (double)(s - j);
      zd[j] = (pt * zd[j] + (k_r - pt) * zd[j + 1]) * km1_rr;
    }
    zd[s] = zd[s] * centre * km1_rr;
  }
  for (int l = nd; l >= 1; --l) {
    double k_r = (double)(s - l + 1);
    double km1_rr = 1.0 / (double)(s - l);
    for (int j = 0; j <= s + 1; ++j) fd[j] = 0.0;
    for (int j = 1; j <= s - 1; ++j) {
      for (int n = 0; n <= std::min(l, s - j); n += 2) {
        fd[j] = fd[j] + g.ncombk[n][l] * zd[j + n];
        fd[j] = fd[j] - g.ncombk[n + 1][l] * zd[j + n + 1];
      }
      double pt = centre + (double)(s - j);
      zd[j] = (pt * zd[j] + (k_r - pt) * zd[j + 1]) * km1_rr;
    }
    for (int j = 1; j <= s - 1; ++j) d[l][j] = fd[j];
    d[l][s] = zd[s];
    zd[s] = zd[s] * centre * km1_rr;
  }
  for (int j = 1; j <= s; ++j) d[0][j] = zd[j];
}

// In-place unnormalised complex DFT of length n along a strided line:
// x(j) = sum_k c(k) exp(isign*2*pi*i*j*k/n)  (gpfa235.F90:39-132 definition).
// Recursive mixed-radix Cooley-Tukey; the rounding differs from GPFA by O(1e-16).
// The twiddle w(m) = exp(isign*2*pi*i*m/n) is tabulated per (n, isign) with the
// angle formed as isign*2*pi*m/n, so every factor is the value the butterfly
// would compute for the exponent (q*kk) mod n.
const std::complex<double>* twiddles(int n, int isign) {
  thread_local std::vector<std::vector<std::complex<double>>> tab[2];
  auto& t = tab[isign > 0 ? 1 : 0];
  if ((int)t.size() <= n) t.resize(n + 1);
  auto& w = t[n];
  if (w.empty()) {
    w.resize(n);
    for (int m = 0; m < n; ++m) {
      double ang = (double)isign * 2.0 * kPi * (double)m / (double)n;
      w[m] = std::complex<double>(std::cos(ang), std::sin(ang));
    }
  }
  return w.data();
}

// work holds at least 2n values: this level's reordered copy, then the deeper levels'.
void fft1d(std::complex<double>* a, int n, int isign, std::complex<double>* work) {
  if (n == 1) return;
  int r = (n % 2 == 0) ? 2 : (n % 3 == 0) ? 3 : (n % 5 == 0) ? 5 : n;
  int m = n / r;
  std::complex<double>* sub = work;
  for (int q = 0; q < r; ++q)
    for (int k = 0; k < m; ++k) sub[(size_t)q * m + k] = a[(size_t)k * r + q];
  for (int q = 0; q < r; ++q) fft1d(&sub[(size_t)q * m], m, isign, work + n);
  const std::complex<double>* w = twiddles(n, isign);
  for (int k = 0; k < m; ++k)
    for (int t = 0; t < r; ++t) {
      std::complex<double> acc(0.0, 0.0);
      int kk = k + t * m;
      for (int q = 0, e = 0; q < r; ++q) {  // e = (q * kk) mod n
        acc += sub[(size_t)q * m + k] * w[e];
        e += kk;
        if (e >= n) e -= n;
      }
      a[kk] = acc;
    }
}

void fft3d(std::vector<std::complex<double>>& G, int isign) {
  const int K1 = g.p.kmax[0], K2 = g.p.kmax[1], K3 = g.p.kmax[2];
  const int Kmax = std::max(K1, std::max(K2, K3));
  int nt = g_nthreads;
  (void)nt;
#pragma omp parallel num_threads(nt) if (nt > 1)
  {
    std::vector<std::complex<double>> line(Kmax), work(2 * (size_t)Kmax);
#pragma omp for collapse(2)
    for (int l = 0; l < K3; ++l)
      for (int k = 0; k < K2; ++k) fft1d(&G[((size_t)l * K2 + k) * K1], K1, isign, work.data());
#pragma omp for collapse(2)
    for (int l = 0; l < K3; ++l)
      for (int j = 0; j < K1; ++j) {
        for (int k = 0; k < K2; ++k) line[k] = G[((size_t)l * K2 + k) * K1 + j];
        fft1d(line.data(), K2, isign, work.data());
        for (int k = 0; k < K2; ++k) G[((size_t)l * K2 + k) * K1 + j] = line[k];
      }
#pragma omp for collapse(2)
    for (int k = 0; k < K2; ++k)
      for (int j = 0; j < K1; ++j) {
        for (int l = 0; l < K3; ++l) line[l] = G[((size_t)l * K2 + k) * K1 + j];
        fft1d(line.data(), K3, isign, work.data());
        for (int l = 0; l < K3; ++l) G[((size_t)l * K2 + k) * K1 + j] = line[l];
      }
  }
}

// ewald_spme_forces_coul: source/ewald_spole.F90:244-477, with
// spme_construct_charge_array (ewald_general.F90:517-576),
// spme_construct_potential_grid_coul (ewald_spole.F90:1257-1386) and
// spme_calc_force_energy (ewald_general.F90:717-869).  Forces are added into
// fxo/fyo/fzo for the local atoms.
void spme(double* eng_rc, double* vir_rc, double* stress9, double* fxo, double* fyo, double* fzo) {
  const int s = g.p.nsplines;
  const int K1 = g.p.kmax[0], K2 = g.p.kmax[1], K3 = g.p.kmax[2];
  const double Kr[3] = {(double)K1, (double)K2, (double)K3};
  if (g.spme_newjob) { bspline_coeffs_gen(); g.spme_newjob = false; }
  double rvolm = 1.0 / g.volm;
  double scale = kPi * kSqrpi * std::pow(g.p.alpha, 1 - 3) * (0.5 * rvolm) * g.scaling;
  double rc[9], det;
  invert(g.cell, rc, &det);
  const int nl = g.nlast;
  std::vector<double> u((size_t)3 * nl);
  std::vector<int> to_calc;
  std::vector<int> rind((size_t)3 * nl);
  for (int i = 0; i < nl; ++i) {
    for (int d = 0; d < 3; ++d)
      u[3 * i + d] = Kr[d] * (rc[d] * g.x[i] + rc[d + 3] * g.y[i] + rc[d + 6] * g.z[i] + 0.5);
    if (u[3 * i] >= -kZeroPlus && u[3 * i + 1] >= -kZeroPlus && u[3 * i + 2] >= -kZeroPlus &&
        std::fabs(g.chge[i]) > kZeroPlus)
      to_calc.push_back(i);
    for (int d = 0; d < 3; ++d) rind[3 * i + d] = fint(u[3 * i + d]);
  }
  // charge spreading with clamping to the grid block (serial block = whole grid).
  // The OpenMP build gives each thread a range of z planes; every grid point still
  // receives its terms in atom order, so the grid equals the serial one bit for bit.
  std::vector<double> Q((size_t)K1 * K2 * K3, 0.0);
  const int ncalc = (int)to_calc.size();
  std::vector<double> sp0((size_t)ncalc * 3 * s);  // order-0 splines of the spread atoms
  {
    int nt = g_nthreads;
    (void)nt;
#pragma omp parallel for num_threads(nt) if (nt > 1)
    for (int a = 0; a < ncalc; ++a) {
      const int i = to_calc[a];
      double spl[3][21];
      for (int d = 0; d < 3; ++d) {
        double dd[3][21];
        splines_1d(u[3 * i + d], dd);
        for (int t = 1; t <= s; ++t) sp0[((size_t)a * 3 + d) * s + (t - 1)] = dd[0][t];
      }
      (void)spl;
    }
#pragma omp parallel num_threads(nt) if (nt > 1)
    {
      int tid = 0, ntt = 1;
#ifdef ORACLE_OPENMP
      tid = omp_get_thread_num();
      ntt = omp_get_num_threads();
#endif
      const int pl0 = 1 + (int)((long)K3 * tid / ntt), pl1 = (int)((long)K3 * (tid + 1) / ntt);
      for (int a = 0; a < ncalc; ++a) {
        const int i = to_calc[a];
        const double* sx = &sp0[((size_t)a * 3 + 0) * s];
        const double* sy = &sp0[((size_t)a * 3 + 1) * s];
        const double* sz = &sp0[((size_t)a * 3 + 2) * s];
        const int n1 = rind[3 * i], n2 = rind[3 * i + 1], n3 = rind[3 * i + 2];
        int j_lo = std::max(1, n1 - 1 - s + 3), k_lo = std::max(1, n2 - 1 - s + 3), l_lo = std::max(1, n3 - 1 - s + 3);
        int j_hi = std::min(K1, n1 + 1) - 1 + 1, k_hi = std::min(K2, n2 + 1) - 1 + 1, l_hi = std::min(K3, n3 + 1) - 1 + 1;
        if (j_hi - j_lo < 0 || k_hi - k_lo < 0 || l_hi - l_lo < 0) continue;
        int t1 = n1 - s - 1 + 2, t2 = n2 - s - 1 + 2, t3 = n3 - s - 1 + 2;
        double q = g.chge[i];
        for (int l = std::max(l_lo, pl0); l <= std::min(l_hi, pl1); ++l) {
          double f1 = q * sz[l - t3 - 1];
          for (int k = k_lo; k <= k_hi; ++k) {
            double f2 = f1 * sy[k - t2 - 1];
            double* row = &Q[((size_t)(l - 1) * K2 + (k - 1)) * K1];
            for (int j = j_lo; j <= j_hi; ++j) row[j - 1] = row[j - 1] + f2 * sx[j - t1 - 1];
          }
        }
      }
    }
  }
  // potential grid: FFT(+1), influence function, stress, FFT(-1)
  std::vector<std::complex<double>> G(Q.size());
  for (size_t n = 0; n < Q.size(); ++n) G[n] = {Q[n], 0.0};
  fft3d(G, 1);
  double recip_conv_fac = kPi / g.p.alpha;
  double test_fac = (1.0e-6 / recip_conv_fac) * (1.0e-6 / recip_conv_fac);
  double rcp[10];
  dcell(rc, rcp);
  double cut_off = 0.5 * 1.05 * std::min(Kr[0] * rcp[6], std::min(Kr[1] * rcp[7], Kr[2] * rcp[8]));
  double cut_off_2 = cut_off * cut_off;
  double st[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  // one z plane of the influence-function multiply; its stress terms go to sp
  auto influence_plane = [&](int l, double (&sp)[3][3]) {
    int ll = l - 1; if (2 * ll > K3) ll -= K3;
    double rp3[3] = {(double)ll * rc[2], (double)ll * rc[5], (double)ll * rc[8]};
    double bb3 = g.norm2[2][l - 1];
    for (int k = 1; k <= K2; ++k) {
      int kk = k - 1; if (2 * kk > K2) kk -= K2;
      double rp2[3] = {rp3[0] + (double)kk * rc[1], rp3[1] + (double)kk * rc[4], rp3[2] + (double)kk * rc[7]};
      double bb2 = bb3 * g.norm2[1][k - 1];
      for (int j = 1; j <= K1; ++j) {
        int jj = j - 1; if (2 * jj > K1) jj -= K1;
        double rp1[3] = {rp2[0] + (double)jj * rc[0], rp2[1] + (double)jj * rc[3], rp2[2] + (double)jj * rc[6]};
        double bb1 = bb2 * g.norm2[0][j - 1];
        double k2 = rp1[0] * rp1[0] + rp1[1] * rp1[1] + rp1[2] * rp1[2];
        std::complex<double>& cell = G[((size_t)(l - 1) * K2 + (k - 1)) * K1 + (j - 1)];
        if (k2 <= cut_off_2 && k2 > test_fac) {
          double fpf = std::sqrt(k2) * recip_conv_fac;
          std::complex<double> pc = bb1 * cell * std::exp(-(fpf * fpf)) / (kSqrpi * fpf * fpf);
          double pv = (pc * (-2.0 * ((1.0 + fpf * fpf) / k2)) * std::conj(cell)).real();
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) sp[a][b] += rp1[a] * rp1[b] * pv;
          cell = pc;
        } else {
          cell = {0.0, 0.0};
        }
      }
    }
    };
#ifdef ORACLE_OPENMP
  if (g_nthreads > 1) {
    std::vector<double> part((size_t)g_nthreads * 9, 0.0);
#pragma omp parallel num_threads(g_nthreads)
    {
      double sp[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma omp for schedule(static)
      for (int l = 1; l <= K3; ++l) influence_plane(l, sp);
      const int t = omp_get_thread_num();
      for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) part[(size_t)t * 9 + 3 * a + b] = sp[a][b];
    }
    for (int t = 0; t < g_nthreads; ++t)
      for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) st[a][b] += part[(size_t)t * 9 + 3 * a + b];
  } else
#endif
  {
    for (int l = 1; l <= K3; ++l) influence_plane(l, st);
  }
  fft3d(G, -1);
  // gather over local atoms with the periodic extended grid (real part)
  double rkmax[3];
  for (int a = 0; a < 3; ++a) rkmax[a] = rc[a] * Kr[0] + rc[a + 3] * Kr[1] + rc[a + 6] * Kr[2];
  std::vector<double> F((size_t)3 * g.natms, 0.0);
  double energy0 = 0.0, ftot[3] = {0, 0, 0};
  auto phi = [&](int jj, int kk, int ll) {
    int a = ((jj % K1) + K1) % K1, b = ((kk % K2) + K2) % K2, c = ((ll % K3) + K3) % K3;
    return G[((size_t)c * K2 + b) * K1 + a].real();
  };
  // one atom's gather: its energy term et and force sums cf; the net-force terms go to ft
  auto gather_atom = [&](int i, double& et, double (&cf)[3], double (&ft)[3]) {
    double spl[3][3][21];
    for (int d = 0; d < 3; ++d) splines_1d(u[3 * i + d], spl[d]);
    double q = g.chge[i];
    for (int l = 1; l <= s; ++l) {
      int ll = rind[3 * i + 2] + 1 - s + l - 1;  // 0-based
      double e2 = q * spl[2][0][l];
      double ft13 = q * spl[2][0][l], ft23 = q * spl[2][0][l], ft33 = q * spl[2][1][l];
      for (int k = 1; k <= s; ++k) {
        int kk = rind[3 * i + 1] + 1 - s + k - 1;
        double e1 = e2 * spl[1][0][k];
        double ft12 = ft13 * spl[1][0][k], ft22 = ft23 * spl[1][1][k], ft32 = ft33 * spl[1][0][k];
        for (int j = 1; j <= s; ++j) {
          int jj = rind[3 * i] + 1 - s + j - 1;
          double ph = phi(jj, kk, ll);
          double a0 = ft12 * spl[0][1][j] * ph * rkmax[0];
          double a1 = ft22 * spl[0][0][j] * ph * rkmax[1];
          double a2 = ft32 * spl[0][0][j] * ph * rkmax[2];
          ft[0] -= a0; ft[1] -= a1; ft[2] -= a2;
          cf[0] += a0; cf[1] += a1; cf[2] += a2;
          et += e1 * spl[0][0][j] * ph;
        }
      }
    }
  };
#ifdef ORACLE_OPENMP
  if (g_nthreads > 1) {
    std::vector<double> part((size_t)g_nthreads * 4, 0.0);
#pragma omp parallel num_threads(g_nthreads)
    {
      double e = 0.0, ft[3] = {0, 0, 0};
#pragma omp for schedule(static)
      for (int i = 0; i < g.natms; ++i) {
        if (std::fabs(g.chge[i]) <= kZeroPlus) continue;
        double et = 0.0, cf[3] = {0, 0, 0};
        gather_atom(i, et, cf, ft);
        e += et;
        F[3 * i] -= cf[0]; F[3 * i + 1] -= cf[1]; F[3 * i + 2] -= cf[2];
      }
      const int t = omp_get_thread_num();
      part[4 * t] = e; part[4 * t + 1] = ft[0]; part[4 * t + 2] = ft[1]; part[4 * t + 3] = ft[2];
    }
    for (int t = 0; t < g_nthreads; ++t) {
      energy0 += part[4 * t];
      for (int a = 0; a < 3; ++a) ftot[a] += part[4 * t + 1 + a];
    }
  } else
#endif
  {
    for (int i = 0; i < g.natms; ++i) {
      if (std::fabs(g.chge[i]) <= kZeroPlus) continue;
      double et = 0.0, cf[3] = {0, 0, 0};
      gather_atom(i, et, cf, ftot);
      energy0 += et;
      F[3 * i] -= cf[0]; F[3 * i + 1] -= cf[1]; F[3 * i + 2] -= cf[2];
    }
  }
  for (int a = 0; a < 3; ++a) ftot[a] /= (double)g.natms;  // megatm
  for (int i = 0; i < g.natms; ++i)
    for (int a = 0; a < 3; ++a) F[3 * i + a] = F[3 * i + a] - ftot[a];
  double q0 = energy0 * scale;
  for (int i = 0; i < g.natms; ++i) {
    fxo[i] += F[3 * i] * scale * 2.0;
    fyo[i] += F[3 * i + 1] * scale * 2.0;
    fzo[i] += F[3 * i + 2] * scale * 2.0;
  }
  double s9[9];
  for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) s9[a * 3 + b] = st[a][b] * scale;  // reshape: (beta,alpha) col-major
  double stt[9];
  // stress_contrib = Reshape(stress_temp(beta,alpha)) column-major: index = beta + 3*alpha
  for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) stt[b + 3 * a] = st[a][b] * scale;
  (void)s9;
  double eng = q0;
  *eng_rc = eng + g.self_interaction;
  stt[0] += eng; stt[4] += eng; stt[8] += eng;
  for (int k = 0; k < 9; ++k) stress9[k] += stt[k];
  *vir_rc = -(stt[0] + stt[4] + stt[8]);
}

// ------------------------------------------------------- constraints / VV
// constraints_tags: source/constraints.F90:438-586 (serial: all local)
void constraints_tags() {
  g.listot.assign(g.natms, 0);
  g.dxx.assign(g.ntcons, 0.0); g.dyy.assign(g.ntcons, 0.0); g.dzz.assign(g.ntcons, 0.0);
  for (int k = 0; k < g.ntcons; ++k) {
    int i = g.con_i[k], j = g.con_j[k];
    g.dxx[k] = g.x[i] - g.x[j];
    g.dyy[k] = g.y[i] - g.y[j];
    g.dzz[k] = g.z[i] - g.z[j];
    g.listot[i]++;
    g.listot[j]++;
    images1(&g.dxx[k], &g.dyy[k], &g.dzz[k]);
  }
  g.lstitr.assign(g.natms, 0);
  for (int k = 0; k < g.natms; ++k) g.lstitr[k] = (g.listot[k] > 0 && g.lfrzn[k] == 0);
}

// constraints_shake_vv: source/constraints.F90:777-1030
int constraints_shake(double tstep, double* str, double* vir, int* iters) {
  for (int k = 0; k < 9; ++k) str[k] = 0.0;
  double tstep2 = tstep * tstep;
  bool safe = false;
  int icyc = 0;
  std::vector<double> dxt(g.ntcons), dyt(g.ntcons), dzt(g.ntcons), dt2(g.ntcons), esig(g.ntcons);
  std::vector<double> xxt(g.natms), yyt(g.natms), zzt(g.natms);
  while (!safe && icyc < g.p.shake_maxit) {
    icyc++;
    for (int k = 0; k < g.ntcons; ++k) {
      int i = g.con_i[k], j = g.con_j[k];
      dxt[k] = g.x[i] - g.x[j]; dyt[k] = g.y[i] - g.y[j]; dzt[k] = g.z[i] - g.z[j];
      images1(&dxt[k], &dyt[k], &dzt[k]);
    }
    safe = true;
    for (int k = 0; k < g.ntcons; ++k) {
      double d0 = g.prmcon[g.con_type[k]];
      dt2[k] = dxt[k] * dxt[k] + dyt[k] * dyt[k] + dzt[k] * dzt[k] - d0 * d0;
      esig[k] = 0.5 * std::fabs(dt2[k]);
      safe = safe && (esig[k] < g.p.shake_tol * d0);
    }
    if (!safe) {
      std::fill(xxt.begin(), xxt.end(), 0.0);
      std::fill(yyt.begin(), yyt.end(), 0.0);
      std::fill(zzt.begin(), zzt.end(), 0.0);
      for (int k = 0; k < g.ntcons; ++k) {
        int i = g.con_i[k], j = g.con_j[k];
        double amti = tstep2 / g.weight[i], amtj = tstep2 / g.weight[j];
        if (g.lfrzn[i] != 0) amti = 0.0;
        if (g.lfrzn[j] != 0) amtj = 0.0;
        double gamma = dt2[k] / ((amti + amtj) * (g.dxx[k] * dxt[k] + g.dyy[k] * dyt[k] + g.dzz[k] * dzt[k]));
        str[0] -= gamma * g.dxx[k] * g.dxx[k];
        str[1] -= gamma * g.dxx[k] * g.dyy[k];
        str[2] -= gamma * g.dxx[k] * g.dzz[k];
        str[4] -= gamma * g.dyy[k] * g.dyy[k];
        str[5] -= gamma * g.dyy[k] * g.dzz[k];
        str[8] -= gamma * g.dzz[k] * g.dzz[k];
        if (g.lfrzn[i] == 0) {
          double gammi = -0.5 * gamma * amti;
          xxt[i] += g.dxx[k] * gammi; yyt[i] += g.dyy[k] * gammi; zzt[i] += g.dzz[k] * gammi;
        }
        if (g.lfrzn[j] == 0) {
          double gammj = 0.5 * gamma * amtj;
          xxt[j] += g.dxx[k] * gammj; yyt[j] += g.dyy[k] * gammj; zzt[j] += g.dzz[k] * gammj;
        }
      }
      for (int k = 0; k < g.ntcons; ++k) {
        int i = g.con_i[k], j = g.con_j[k];
        if (g.lfrzn[i] == 0) {
          double dli = 1.0 / (double)g.listot[i];
          g.x[i] += xxt[i] * dli; g.y[i] += yyt[i] * dli; g.z[i] += zzt[i] * dli;
        }
        if (g.lfrzn[j] == 0) {
          double dlj = 1.0 / (double)g.listot[j];
          g.x[j] += xxt[j] * dlj; g.y[j] += yyt[j] * dlj; g.z[j] += zzt[j] * dlj;
        }
      }
    }
  }
  *iters = icyc;
  if (!safe) return GB_ERR_SHAKE;
  str[3] = str[1]; str[6] = str[2]; str[7] = str[5];
  *vir = -(str[0] + str[4] + str[8]);
  return GB_OK;
}

// constraints_rattle: source/constraints.F90:587-775 (kit = 1, lfst = .true.)
int constraints_rattle(double tstep, int* iters) {
  for (int k = 0; k < g.ntcons; ++k) {
    double dis = 1.0 / std::sqrt(g.dxx[k] * g.dxx[k] + g.dyy[k] * g.dyy[k] + g.dzz[k] * g.dzz[k]);
    g.dxx[k] *= dis; g.dyy[k] *= dis; g.dzz[k] *= dis;
  }
  bool safe = false;
  int icyc = 0;
  std::vector<double> vxt(g.natms), vyt(g.natms), vzt(g.natms);
  while (!safe && icyc < g.p.shake_maxit) {
    icyc++;
    std::fill(vxt.begin(), vxt.end(), 0.0);
    std::fill(vyt.begin(), vyt.end(), 0.0);
    std::fill(vzt.begin(), vzt.end(), 0.0);
    double esig = 0.0;
    for (int k = 0; k < g.ntcons; ++k) {
      int i = g.con_i[k], j = g.con_j[k];
      double amti = tstep / g.weight[i], amtj = tstep / g.weight[j];
      if (g.lfrzn[i] != 0) amti = 0.0;
      if (g.lfrzn[j] != 0) amtj = 0.0;
      double gamma = g.dxx[k] * (g.vx[i] - g.vx[j]) + g.dyy[k] * (g.vy[i] - g.vy[j]) + g.dzz[k] * (g.vz[i] - g.vz[j]);
      esig = std::max(esig, 0.5 * tstep * std::fabs(gamma));
      gamma = gamma / (amti + amtj);
      if (g.lfrzn[i] == 0) {
        double gammi = -gamma * amti;
        vxt[i] += g.dxx[k] * gammi; vyt[i] += g.dyy[k] * gammi; vzt[i] += g.dzz[k] * gammi;
      }
      if (g.lfrzn[j] == 0) {
        double gammj = gamma * amtj;
        vxt[j] += g.dxx[k] * gammj; vyt[j] += g.dyy[k] * gammj; vzt[j] += g.dzz[k] * gammj;
      }
    }
    safe = (esig < g.p.shake_tol);
    if (!safe) {
      for (int k = 0; k < g.ntcons; ++k) {
        int i = g.con_i[k], j = g.con_j[k];
        if (g.lfrzn[i] == 0) {
          double dli = 1.0 / (double)g.listot[i];
          g.vx[i] += vxt[i] * dli; g.vy[i] += vyt[i] * dli; g.vz[i] += vzt[i] * dli;
        }
        if (g.lfrzn[j] == 0) {
          double dlj = 1.0 / (double)g.listot[j];
          g.vx[j] += vxt[j] * dlj; g.vy[j] += vyt[j] * dlj; g.vz[j] += vzt[j] * dlj;
        }
      }
    }
  }
  *iters = icyc;
  return safe ? GB_OK : GB_ERR_RATTLE;
}

// kinstress: source/kinetics.F90:218-262
void kinstress(double* s) {
  for (int k = 0; k < 9; ++k) s[k] = 0.0;
  for (int i = 0; i < g.natms; ++i) {
    if (g.lfrzn[i] != 0) continue;
    double w = g.weight[i];
    s[0] += w * g.vx[i] * g.vx[i]; s[1] += w * g.vx[i] * g.vy[i]; s[2] += w * g.vx[i] * g.vz[i];
    s[4] += w * g.vy[i] * g.vy[i]; s[5] += w * g.vy[i] * g.vz[i]; s[8] += w * g.vz[i] * g.vz[i];
  }
  s[3] = s[1]; s[6] = s[2]; s[7] = s[5];
}

// ------------------------------------------------------------------ thermostats
// sarurnd (numerics.F90:458-635): the SARU generator as the reference evaluates it,
// in 64-bit integers (Ishft is a logical shift) with the products formed in double
// precision and reduced with Mod(., 2^32).
static inline int64_t lshl(int64_t x, int n) { return (int64_t)((uint64_t)x << n); }
static inline int64_t lshr(int64_t x, int n) { return (int64_t)((uint64_t)x >> n); }
static inline int64_t int32of(int64_t x) { return (int64_t)(int32_t)(uint32_t)(uint64_t)x; }
static inline int64_t prodmod(double a, double b) { return (int64_t)std::fmod(a * b, 4294967296.0); }

double sarurnd(int64_t seeda, int64_t seedb, int64_t seedc) {
  const int64_t two32 = 4294967296LL;
  int64_t seed1 = seeda % two32; if (seed1 < 0) seed1 += two32;
  int64_t seed2 = seedb % two32; if (seed2 < 0) seed2 += two32;
  int64_t seed3 = seedc % two32; if (seed3 < 0) seed3 += two32;
  int64_t itmp;
  seed3 = (seed3 ^ (lshl(seed1, 7) ^ lshr(seed2, 6))) % two32;
  itmp = lshr(seed1, 4) ^ lshr(seed3, 15);
  seed2 = (seed2 + itmp) % two32;
  seed1 = (seed1 ^ (lshl(seed2, 9) + lshl(seed3, 8))) % two32;
  itmp = lshr(seed2, 11) ^ lshl(seed1, 1);
  itmp = prodmod(2771807053.0, (double)itmp);
  seed3 = (seed3 ^ itmp) % two32;
  itmp = lshl(seed1, 4) ^ lshr(seed3, 16);
  itmp = prodmod(1925059961.0, (double)itmp);
  seed2 = (seed2 + itmp) % two32;
  itmp = lshr(seed3, 5) ^ lshr(int32of(seed2), 22);
  itmp = prodmod(1060677357.0, (double)itmp);
  if (itmp < 0) itmp += two32;
  seed1 = (seed1 ^ itmp) % two32;
  itmp = prodmod((double)seed1, (double)seed3);
  seed2 = (seed2 + itmp) % two32;
  seed1 = (seed1 + (seed3 ^ lshr(seed2, 2))) % two32;
  seed2 = seed2 ^ lshr(int32of(seed2), 17);
  if (seed2 < 0) seed2 += two32;
  itmp = seed1 ^ lshr(int32of(seed1), 14);
  int64_t state = prodmod(2044649123.0, (double)itmp);
  if (state < 0) state += two32;
  int64_t wstate = ((state + seed2) ^ lshr(int32of(state), 8)) % two32;
  if (wstate < 0) wstate += two32;
  itmp = wstate ^ 3722418165LL;
  itmp = prodmod((double)wstate, (double)itmp);
  state = (state + itmp) % two32;
  wstate = (2882246391LL + lshr(wstate, 1)) % two32;
  itmp = prodmod(1273716057.0, (double)state);
  state = (itmp + 637592055LL) % two32;
  wstate = (wstate + 2148127051LL + (lshr(int32of(wstate), 31) & 3666320093LL)) % two32;
  int64_t v = ((state ^ lshr(state, 26)) + wstate) % two32;
  itmp = v ^ lshr(v, 20);
  int64_t u32 = prodmod((double)itmp, 1767372199.0);
  const double rtwo32 = 1.0 / 4294967296.0;
  double p1 = (double)int32of(u32) * rtwo32 + (0.5 + 0.5 * rtwo32);
  double p2 = (double)state * (rtwo32 * rtwo32);
  return p1 + p2;
}

// box_mueller_saru3 (numerics.F90:745-803), counter starting at k0; seed shifts added
int box_mueller_saru3(int64_t i, int64_t j, int64_t k0, double* g1, double* g2, double* g3) {
  const int64_t a = i + g.seed[0], b = j + g.seed[1];
  int64_t k = k0 + g.seed[2];
  double ran0 = 1.0, ran1 = 0.0, ran2 = 0.0;
  int guard = 0;
  while (ran0 <= DBL_MIN || ran0 >= 1.0) {
    ran1 = 2.0 * sarurnd(a, b, k) - 1.0;
    ran2 = 2.0 * sarurnd(a, b, k + 1) - 1.0;
    ran0 = ran1 * ran1 + ran2 * ran2;
    k += 2;
    if (++guard > 64) return GB_ERR_RNG;
  }
  ran0 = std::sqrt(-2.0 * std::log(ran0) / ran0);
  *g1 = ran0 * ran1;
  *g2 = ran0 * ran2;
  ran0 = 1.0;
  guard = 0;
  while (ran0 <= DBL_MIN || ran0 >= 1.0) {
    ran1 = 2.0 * sarurnd(a, b, k) - 1.0;
    ran2 = 2.0 * sarurnd(a, b, k + 1) - 1.0;
    ran0 = ran1 * ran1 + ran2 * ran2;
    k += 2;
    if (++guard > 64) return GB_ERR_RNG;
  }
  ran0 = std::sqrt(-2.0 * std::log(ran0) / ran0);
  *g3 = ran0 * ran1;
  return GB_OK;
}

// langevin_forces, setforces branch (langevin.F90:57-194; global id = i + 1)
int langevin_forces(int nstep, double tstep, std::vector<double>& fx, std::vector<double>& fy,
                    std::vector<double>& fz) {
  const double scale = std::sqrt(2.0 * g.chi * 0.831451115 * g.temp / tstep);
  fx.assign(g.natms, 0.0); fy.assign(g.natms, 0.0); fz.assign(g.natms, 0.0);
  for (int i = 0; i < g.natms; ++i) {
    if (g.lfrzn[i] == 0 && g.weight[i] > 1.0e-6) {
      int st = box_mueller_saru3(i + 1, nstep, 0, &fx[i], &fy[i], &fz[i]);
      if (st) return st;
      double tmp = scale * std::sqrt(g.weight[i]);
      fx[i] = fx[i] * tmp; fy[i] = fy[i] * tmp; fz[i] = fz[i] * tmp;
    }
  }
  return GB_OK;
}

// langevin_scalers (nvt_langevin.F90:1552-1621)
void langevin_scalers(double chi, double tstep, double* t0, double* t1, double* scr, double* scv, double* scl) {
  const double stol = 1.0e-3;
  *t0 = std::exp(-chi * tstep);
  if (chi <= DBL_MIN) { *t1 = tstep; *scr = 0.0; *scl = 0.0; *scv = 0.0; return; }
  *t1 = (1.0 - *t0) / chi;
  double alpha = 0.5 * chi * tstep;
  if (alpha < stol) {
    *scr = (alpha - alpha * alpha + 0.5 * (alpha * alpha * alpha) - (alpha * alpha * alpha * alpha) / 6.0 +
            0.075 * (alpha * alpha * alpha * alpha * alpha)) / chi;
    *scl = (alpha - 0.2 * (alpha * alpha * alpha) + (32.0 * (alpha * alpha * alpha * alpha * alpha)) / 525.0) /
           (chi * std::sqrt(3.0));
    *scv = 1.0 - alpha + 5.0 * (alpha * alpha) / 6.0 - 0.5 * (alpha * alpha * alpha);
  } else {
    *scr = (1.0 - *t0) * (1.0 - *t0) / (std::sqrt(alpha * (1.0 - *t0 * *t0)) * 2.0 * chi);
    *scl = std::sqrt(1.0 - std::tanh(alpha) / alpha) / chi;
    *scv = std::sqrt((1.0 - *t0 * *t0) / (4.0 * alpha));
  }
}

// getkin (kinetics.F90): 0.5 sum over non-frozen atoms of m v^2
double getkin() {
  double e = 0.0;
  for (int i = 0; i < g.natms; ++i)
    if (g.lfrzn[i] == 0) e += g.weight[i] * (g.vx[i] * g.vx[i] + g.vy[i] * g.vy[i] + g.vz[i] * g.vz[i]);
  return 0.5 * e;
}

// getvom (kinetics.F90:365-419) and its subtraction from the free atoms
void remove_vom() {
  double vom[3] = {0, 0, 0};
  for (int i = 0; i < g.natms; ++i)
    if (g.lfrzn[i] == 0) {
      vom[0] += g.weight[i] * g.vx[i]; vom[1] += g.weight[i] * g.vy[i]; vom[2] += g.weight[i] * g.vz[i];
    }
  if (g.totmas >= DBL_MIN) for (int k = 0; k < 3; ++k) vom[k] = vom[k] / g.totmas;
  for (int i = 0; i < g.natms; ++i)
    if (g.lfrzn[i] == 0 && g.weight[i] > 1.0e-6) { g.vx[i] -= vom[0]; g.vy[i] -= vom[1]; g.vz[i] -= vom[2]; }
}

// nvt_b0_scl (nvt_berendsen.F90:907-962); stage 1 scales, stage 0 only measures
void nvt_b0_scl(int stage, double tstep, double* strkin, double* engke) {
  kinstress(strkin);
  *engke = 0.5 * (strkin[0] + strkin[4] + strkin[8]);
  g.chi_t = std::sqrt(1.0 + tstep / g.tau_t * (g.sigma / *engke - 1.0));
  if (stage == 0) return;
  for (int i = 0; i < g.natms; ++i) { g.vx[i] *= g.chi_t; g.vy[i] *= g.chi_t; g.vz[i] *= g.chi_t; }
  double tmp = g.chi_t * g.chi_t;
  for (int k = 0; k < 9; ++k) strkin[k] *= tmp;
  *engke *= tmp;
}

// nvt_h0_scl (nvt_nose_hoover.F90) with pmass = chip = 0
void nvt_h0_scl(double tstep, double* engke) {
  double hstep = 0.5 * tstep, qstep = 0.5 * hstep;
  g.cint = g.cint + qstep * g.chi_t;
  *engke = getkin();
  g.chi_t = g.chi_t + hstep * (2.0 * *engke + 0.0 - g.ceng) / g.qmass;
  g.cint = g.cint + hstep * g.chi_t;
  double scale = std::exp(-tstep * g.chi_t);
  for (int i = 0; i < g.natms; ++i) { g.vx[i] *= scale; g.vy[i] *= scale; g.vz[i] *= scale; }
  *engke = *engke * (scale * scale);
  g.chi_t = g.chi_t + hstep * (2.0 * *engke + 0.0 - g.ceng) / g.qmass;
  g.cint = g.cint + qstep * g.chi_t;
}

int set_ensemble(int kind, double temp, double tau_t, double chi, const int32_t* seed, double degfre) {
  g.ens = kind; g.temp = temp; g.tau_t = tau_t; g.chi = chi;
  for (int k = 0; k < 3; ++k) g.seed[k] = seed ? seed[k] : 0;
  if (degfre <= 0.0) degfre = 3.0 * (double)(g.natms - g.megfrz) - 3.0 - (double)g.ntcons;
  g.sigma = 0.5 * degfre * 0.831451115 * temp;   // temperature.F90:178
  g.qmass = 2.0 * g.sigma * tau_t * tau_t;
  g.ceng = 2.0 * g.sigma;
  g.totmas = 0.0;
  for (int i = 0; i < g.natms; ++i) if (g.lfrzn[i] == 0) g.totmas += g.weight[i];
  g.chi_t = 0.0; g.cint = 0.0; g.consv = 0.0;
  return GB_OK;
}

// nve_0_vv: source/nve.F90:38-235 (lvar = .false.); with an NVT ensemble the
// stages of nvt_b0_vv (nvt_berendsen.F90:39-258), nvt_h0_vv (nvt_nose_hoover.F90)
// or nvt_l0_vv (nvt_langevin.F90)
int nve_vv(int stage, double* strkin, double* engke, int* iters, double* vircon, double* strcon) {
  const double tstep = g.p.tstep, hstep = 0.5 * tstep, rstep = 1.0 / tstep;
  if (g.ntcons > 0) constraints_tags();
  *iters = 0;
  if (stage == 1) {
    if (g.ens == GB_NVT_LANGEVIN) {
      std::vector<double> fxr, fyr, fzr, fxl, fyl, fzl;
      int st = langevin_forces(g.nstep, tstep, fxr, fyr, fzr);
      if (st) return st;
      st = langevin_forces(-g.nstep, tstep, fxl, fyl, fzl);
      if (st) return st;
      double t0, t1, scr1, scv1, scl1;
      langevin_scalers(g.chi, tstep, &t0, &t1, &scr1, &scv1, &scl1);
      for (int i = 0; i < g.natms; ++i) {
        if (g.weight[i] > 1.0e-6) {
          double tmp = hstep / g.weight[i];
          g.vx[i] = g.vx[i] + tmp * g.fx[i];
          g.vy[i] = g.vy[i] + tmp * g.fy[i];
          g.vz[i] = g.vz[i] + tmp * g.fz[i];
          tmp = tstep / g.weight[i];
          g.x[i] = g.x[i] + g.vx[i] * t1 + tmp * (fxr[i] * scr1 + fxl[i] * scl1);
          g.y[i] = g.y[i] + g.vy[i] * t1 + tmp * (fyr[i] * scr1 + fyl[i] * scl1);
          g.z[i] = g.z[i] + g.vz[i] * t1 + tmp * (fzr[i] * scr1 + fzl[i] * scl1);
          g.vx[i] = g.vx[i] * t0 + tmp * fxr[i] * scv1;
          g.vy[i] = g.vy[i] * t0 + tmp * fyr[i] * scv1;
          g.vz[i] = g.vz[i] * t0 + tmp * fzr[i] * scv1;
        }
      }
    } else {
      if (g.ens == GB_NVT_NOSE_HOOVER) {
        double ek;
        nvt_h0_scl(hstep, &ek);
      }
      for (int i = 0; i < g.natms; ++i) {
        if (g.weight[i] > 1.0e-6) {
          double tmp = hstep / g.weight[i];
          g.vx[i] = g.vx[i] + tmp * g.fx[i];
          g.vy[i] = g.vy[i] + tmp * g.fy[i];
          g.vz[i] = g.vz[i] + tmp * g.fz[i];
          g.x[i] = g.x[i] + tstep * g.vx[i];
          g.y[i] = g.y[i] + tstep * g.vy[i];
          g.z[i] = g.z[i] + tstep * g.vz[i];
        }
      }
    }
    if (g.ntcons > 0) {
      // apply_shake: constraints.F90:1071-1200
      g.oxt.assign(g.natms, 0.0); g.oyt.assign(g.natms, 0.0); g.ozt.assign(g.natms, 0.0);
      for (int i = 0; i < g.natms; ++i)
        if (g.lstitr[i]) { g.oxt[i] = g.x[i]; g.oyt[i] = g.y[i]; g.ozt[i] = g.z[i]; }
      double str[9], vir;
      int st = constraints_shake(tstep, str, &vir, iters);
      if (st) return st;
      if (vircon) *vircon = vir;
      if (strcon) for (int k = 0; k < 9; ++k) strcon[k] = str[k];
      for (int i = 0; i < g.natms; ++i) {
        if (!g.lstitr[i]) continue;
        double xt = (g.x[i] - g.oxt[i]) * rstep, yt = (g.y[i] - g.oyt[i]) * rstep, zt = (g.z[i] - g.ozt[i]) * rstep;
        g.vx[i] += xt; g.vy[i] += yt; g.vz[i] += zt;
        double tmp = g.weight[i] / hstep;
        g.fx[i] += xt * tmp; g.fy[i] += yt * tmp; g.fz[i] += zt * tmp;
      }
    }
  } else {
    for (int i = 0; i < g.natms; ++i) {
      if (g.weight[i] > 1.0e-6) {
        double tmp = hstep / g.weight[i];
        g.vx[i] = g.vx[i] + tmp * g.fx[i];
        g.vy[i] = g.vy[i] + tmp * g.fy[i];
        g.vz[i] = g.vz[i] + tmp * g.fz[i];
      }
    }
    if (g.ntcons > 0) {
      int st = constraints_rattle(tstep, iters);
      if (st) return st;
    }
    double sk[9], ek;
    if (g.ens == GB_NVT_BERENDSEN) {
      nvt_b0_scl(1, tstep, sk, &ek);
      remove_vom();
      nvt_b0_scl(0, tstep, sk, &ek);
    } else if (g.ens == GB_NVT_NOSE_HOOVER) {
      nvt_h0_scl(hstep, &ek);
      g.consv = 0.5 * g.qmass * g.chi_t * g.chi_t + g.ceng * g.cint;
      kinstress(sk);
    } else {
      if (g.ens == GB_NVT_LANGEVIN) remove_vom();
      kinstress(sk);
      ek = 0.5 * (sk[0] + sk[4] + sk[8]);
    }
    if (strkin) for (int k = 0; k < 9; ++k) strkin[k] = sk[k];
    if (engke) *engke = ek;
  }
  return GB_OK;
}

// vnl_check: source/neighbours.F90:123-296 (padding stays fixed: the
// no-strict auto-push never raises it for the configurations served here)
bool vnl_check() {
  double tol = 0.0;
  for (int i = 0; i < g.natms; ++i) {
    double xx = g.x[i] - g.xbg[i], yy = g.y[i] - g.ybg[i], zz = g.z[i] - g.zbg[i];
    images1(&xx, &yy, &zz);
    double r = std::sqrt(xx * xx + yy * yy + zz * zz);
    tol = std::max(tol, r);
  }
  return tol >= kHalfMinus * g.p.rpad;
}

// ------------------------------------------------------------------- metals (tabulated EAM)
// metal_table_derivatives: source/metal.F90:2807-2897
void metal_table_derivatives(const std::vector<double>& buffer, std::vector<double>& vvv) {
  vvv[1] = buffer[1]; vvv[2] = buffer[2]; vvv[3] = buffer[3]; vvv[4] = buffer[4];
  double delmet = buffer[4];
  int v_end = (int)std::lround(buffer[1]);
  int i_start = 5 + 2, i_end = v_end - 2;
  for (int i = i_start; i <= i_end; ++i) {
    double aa0 = buffer[i], f0, f1, f2, f3, f4;
    if (std::fabs(aa0) <= kZeroPlus) {
      f0 = 0.0; f1 = 0.0; f2 = 0.0; f3 = 0.0; f4 = 0.0;
    } else {
      f0 = buffer[i - 2] / aa0; f1 = buffer[i - 1] / aa0; f2 = 1.0;
      f3 = buffer[i + 1] / aa0; f4 = buffer[i + 2] / aa0;
    }
    double d1y = (f1 - f0);
    double d2y = (f2 - f1) - (f1 - f0);
    double d3y = (f3 - f0) + 3.0 * (f1 - f2);
    double d4y = (f4 - f3) + 3.0 * (f2 - f3) + 3.0 * (f2 - f1) + (f0 - f1);
    aa0 = aa0 / delmet;
    double aa4 = d4y / 24.0;
    double aa3 = (d3y + 12.0 * aa4) / 6.0;
    double aa2 = (d2y + 6.0 * aa3 - 14.0 * aa4) / 2.0;
    double aa1 = d1y + 3.0 * aa2 - 7.0 * aa3 + 15.0 * aa4;
    vvv[i] = aa1 * aa0;
    if (i == i_start) {
      vvv[i_start - 2] = (aa1 - 4.0 * aa2 + 12.0 * aa3 - 32.0 * aa4) * aa0;
      vvv[i_start - 1] = (aa1 - 2.0 * aa2 + 3.0 * aa3 - 4.0 * aa4) * aa0;
    } else if (i == i_end) {
      vvv[i_end + 1] = (aa1 + 2.0 * aa2 + 3.0 * aa3 + 4.0 * aa4) * aa0;
      vvv[i_end + 2] = (aa1 + 4.0 * aa2 + 12.0 * aa3 + 32.0 * aa4) * aa0;
    }
  }
}

// metal_table_read, tab = 1 (source/metal.F90:1489-1925), energies already in internal units
int metal_tables(int ntab, const int32_t* kind, const int32_t* t1, const int32_t* t2, const int32_t* ngrid,
                 const double* start, const double* finish, const double* values, const int32_t* listed) {
  const int nt = g.p.ntypes, nkey = nt * (nt + 1) / 2;
  int maxgrid = 8;
  for (int k = 0; k < ntab; ++k) maxgrid = std::max(maxgrid, ngrid[k] + 4);
  const size_t len = (size_t)maxgrid + 2;
  g.vmet1.assign(nkey, std::vector<double>(len, 0.0)); g.vmet2 = g.vmet1;
  g.dmet1.assign(nt, std::vector<double>(len, 0.0)); g.dmet2 = g.dmet1;
  g.fmet1 = g.dmet1; g.fmet2 = g.dmet1;
  size_t pos = 0;
  for (int k = 0; k < ntab; ++k) {
    int ng = ngrid[k];
    if (ng < 5 || kind[k] < 1 || kind[k] > 3 || t1[k] < 1 || t1[k] > nt) return GB_ERR_ARG;
    std::vector<double> buffer(len, 0.0);
    buffer[1] = (double)(ng + 4);
    buffer[4] = (finish[k] - start[k]) / (double)(ng - 1);
    buffer[2] = start[k] - 5.0 * buffer[4];
    buffer[3] = finish[k];
    for (int i = 0; i < ng; ++i) buffer[5 + i] = values[pos + i];
    pos += ng;
    std::vector<double>*c1, *c2;
    if (kind[k] == 1) {
      if (t2[k] < 1 || t2[k] > nt) return GB_ERR_ARG;
      int a = std::max(t1[k], t2[k]), b = std::min(t1[k], t2[k]);
      int k0 = a * (a - 1) / 2 + b - 1;
      c1 = &g.vmet1[k0]; c2 = &g.vmet2[k0];
    } else if (kind[k] == 2) {
      c1 = &g.dmet1[t1[k] - 1]; c2 = &g.dmet2[t1[k] - 1];
    } else {
      c1 = &g.fmet1[t1[k] - 1]; c2 = &g.fmet2[t1[k] - 1];
    }
    for (int i = 1; i <= 4; ++i) (*c1)[i] = buffer[i];
    for (int i = 5; i < (int)len; ++i) (*c1)[i] = (i - 4 > ng) ? 0.0 : buffer[i];
    metal_table_derivatives(buffer, *c2);
    if (kind[k] == 2) for (int i = 1; i <= 4; ++i) (*c2)[i] = 0.0;
    if (kind[k] != 3)
      for (int i = 5; i <= ng + 4; ++i) (*c2)[i] = -((double)i * buffer[4] + buffer[2]) * (*c2)[i];
  }
  g.met_listed.assign(nkey, 1);
  if (listed) for (int k = 0; k < nkey; ++k) g.met_listed[k] = listed[k];
  g.metal = ntab > 0;
  return GB_OK;
}

// three-point table interpolation of metal_ld_compute / metal_forces
static bool met_index(const std::vector<double>& t, double r, int* l, double* ppp) {
  double rdr = 1.0 / t[4];
  double rr1 = r - t[2];
  int k = std::min((int)std::lround(rr1 * rdr), (int)std::lround(t[1]) - 1);
  bool ok = true;
  if (k < 5) { ok = false; k = 6; }
  *l = k;
  *ppp = rr1 * rdr - (double)k;
  return ok;
}

static double met_interp(const std::vector<double>& v, int l, double ppp, int density) {
  double vk0 = v[l - 1], vk1 = v[l], vk2 = v[l + 1];
  double t1 = vk1 + ppp * (vk1 - vk0);
  double t2 = vk1 + ppp * (vk2 - vk1);
  if (ppp < 0.0) {
    double d = t1 + 0.5 * (t2 - t1) * (ppp + 1.0);
    if (density && d < 0.0) d = t1;
    return d;
  } else if (l == 5) {
    return t2;
  }
  double d = t2 + 0.5 * (t2 - t1) * (ppp - 1.0);
  if (density && d < 0.0) d = t2;
  return d;
}

// metal_ld_compute (metal.F90:897-1257) with metal_ld_collect_eam (:2207-2516) and
// metal_ld_set_halo (:3146): rho becomes F'(rho) on local atoms and halo images
int metal_ld_compute(double* stress) {
  g.mrho.assign(g.nlast, 0.0);
  bool safe = true;
  g.engden = 0.0;
  g.virden = 0.0;
  std::vector<double> rrt(g.p.max_list + 1);
  for (int i = 0; i < g.natms; ++i) {
    int limit = L(0, i);
    for (int k = 1; k <= limit; ++k) {
      int j = L(k, i) - 1;
      double xx = g.x[i] - g.x[j], yy = g.y[i] - g.y[j], zz = g.z[i] - g.z[j];
      rrt[k] = std::sqrt(xx * xx + yy * yy + zz * zz);
    }
    int ai = g.ltype[i];
    for (int m = 1; m <= limit; ++m) {
      int j = L(m, i) - 1;
      int aj = g.ltype[j];
      int ki = ai, kj = aj;
      double rrr = rrt[m];
      const std::vector<double>& dj = g.dmet1[kj - 1];
      if (std::fabs(dj[1]) > kZeroPlus && std::lround(dj[1]) > 5) {
        if (rrr <= dj[3]) {
          int l; double ppp;
          if (!met_index(dj, rrr, &l, &ppp)) safe = false;
          double density = met_interp(dj, l, ppp, 1);
          g.mrho[i] += density;
          if (ki == kj && j < g.natms) g.mrho[j] += density;
        }
      }
      const std::vector<double>& di = g.dmet1[ki - 1];
      if (std::fabs(di[1]) > kZeroPlus && std::lround(di[1]) > 5) {
        if (ki != kj && j < g.natms) {
          if (rrr <= di[3]) {
            int l; double ppp;
            if (!met_index(di, rrr, &l, &ppp)) safe = false;
            g.mrho[j] += met_interp(di, l, ppp, 1);
          }
        }
      }
    }
  }
  if (!safe) return GB_ERR_METAL_TABLE;
  for (int i = 0; i < g.natms; ++i) {
    const std::vector<double>& f1 = g.fmet1[g.ltype[i] - 1];
    const std::vector<double>& f2 = g.fmet2[g.ltype[i] - 1];
    if (std::fabs(f1[1]) > kZeroPlus) {
      double rhosqr = g.mrho[i];
      if (rhosqr >= f1[2] + 5.0 * f1[4]) {
        if (rhosqr <= f1[3]) {
          int l; double ppp;
          if (!met_index(f1, rhosqr, &l, &ppp)) safe = false;
          g.engden += met_interp(f1, l, ppp, 0);
          g.mrho[i] = met_interp(f2, l, ppp, 0);
        } else {
          int l = (int)std::lround(f1[1]);
          g.engden += f1[l];
          g.mrho[i] = 0.0;
        }
      } else {
        safe = false;
      }
    }
  }
  if (!safe) return GB_ERR_METAL_DENSITY;
  stress[0] -= g.virden / 3.0; stress[4] -= g.virden / 3.0; stress[8] -= g.virden / 3.0;
  for (int k = g.natms; k < g.nlast; ++k) g.mrho[k] = g.mrho[g.src[k]];
  return GB_OK;
}

// metal_forces, tabulated EAM branch (metal.F90:193-895), serial without HALF_HALO
void metal_forces(double* stress) {
  g.engmet = 0.0;
  g.virmet = 0.0;
  std::vector<double> xxt(g.p.max_list + 1), yyt(g.p.max_list + 1), zzt(g.p.max_list + 1), rrt(g.p.max_list + 1);
  const int nt = g.p.ntypes;
  (void)nt;
  for (int i = 0; i < g.natms; ++i) {
    int limit = L(0, i);
    for (int k = 1; k <= limit; ++k) {
      int j = L(k, i) - 1;
      xxt[k] = g.x[i] - g.x[j]; yyt[k] = g.y[i] - g.y[j]; zzt[k] = g.z[i] - g.z[j];
      rrt[k] = std::sqrt(xxt[k] * xxt[k] + yyt[k] * yyt[k] + zzt[k] * zzt[k]);
    }
    int idi = g.ltg[i], ai = g.ltype[i];
    double fix = g.fx[i], fiy = g.fy[i], fiz = g.fz[i];
    double s1 = 0, s2 = 0, s3 = 0, s5 = 0, s6 = 0, s9 = 0;
    for (int m = 1; m <= limit; ++m) {
      int j = L(m, i) - 1;
      int aj = g.ltype[j];
      int ki = ai, kj = aj;
      int key = (ai > aj ? ai * (ai - 1) / 2 + aj : aj * (aj - 1) / 2 + ai) - 1;
      double rrr = rrt[m];
      if (!(g.met_listed[key] && rrr <= g.p.rcut)) continue;  // keypot >= 0 .and. rrr <= met%rcut
      double rsq = rrr * rrr;
      double eng = 0.0, gamma1 = 0.0, gamma2 = 0.0, gamma3 = 0.0;
      const bool count = j < g.natms || idi < g.ltg[j];
      const std::vector<double>& v1 = g.vmet1[key];
      int l = 0; double ppp = 0.0;
      if (std::fabs(v1[1]) > kZeroPlus) {
        if (rrr <= v1[3]) {
          if (!met_index(v1, rrr, &l, &ppp)) g.metal_unsafe = true;
          gamma1 = met_interp(g.vmet2[key], l, ppp, 0);
          if (count) eng = met_interp(v1, l, ppp, 0);
        }
      }
      const std::vector<double>& dj = g.dmet1[kj - 1];
      const std::vector<double>& di = g.dmet1[ki - 1];
      if (std::fabs(dj[1]) > kZeroPlus && std::lround(di[1]) > 5) {
        if (rrr <= dj[3]) {
          int ld; double ppd;
          if (!met_index(dj, rrr, &ld, &ppd)) g.metal_unsafe = true;
          gamma2 = met_interp(g.dmet2[kj - 1], ld, ppd, 0);
        }
      }
      if (ki == kj) {
        gamma3 = gamma2;
      } else if (std::fabs(di[1]) > kZeroPlus && std::lround(di[1]) > 5) {
        if (rrr <= di[3]) {
          int ld; double ppd;
          if (!met_index(di, rrr, &ld, &ppd)) g.metal_unsafe = true;
          gamma3 = met_interp(g.dmet2[ki - 1], ld, ppd, 0);
        }
      }
      double gamma = (gamma1 + (gamma2 * g.mrho[i] + gamma3 * g.mrho[j])) / rsq;
      double fx = gamma * xxt[m], fy = gamma * yyt[m], fz = gamma * zzt[m];
      fix += fx; fiy += fy; fiz += fz;
      if (j < g.natms) { g.fx[j] -= fx; g.fy[j] -= fy; g.fz[j] -= fz; }
      if (count) {
        g.engmet += eng;
        g.virmet -= gamma * rsq;
        s1 += xxt[m] * fx; s2 += xxt[m] * fy; s3 += xxt[m] * fz;
        s5 += yyt[m] * fy; s6 += yyt[m] * fz; s9 += zzt[m] * fz;
      }
    }
    g.fx[i] = fix; g.fy[i] = fiy; g.fz[i] = fiz;
    stress[0] += s1; stress[1] += s2; stress[2] += s3; stress[3] += s2; stress[4] += s5;
    stress[5] += s6; stress[6] += s3; stress[7] += s6; stress[8] += s9;
  }
}

int calculate_forces(double* eng8, double* stress9) {
  for (int i = 0; i < g.nlast; ++i) { g.fx[i] = 0.0; g.fy[i] = 0.0; g.fz[i] = 0.0; }
  double st[9] = {0};
  double erc = 0, vrc = 0;
  g.engmet = g.virmet = g.engden = g.virden = 0.0;
  if (g.metal) {  // metal_ld_compute precedes the Ewald sums (two_body.F90:281-291)
    int e = metal_ld_compute(st);
    if (e) return e;
  }
  spme(&erc, &vrc, st, g.fx.data(), g.fy.data(), g.fz.data());
  Acc A;
  two_body_real(A);
  for (int k = 0; k < 9; ++k) st[k] += A.str[k];
  if (g.metal) {  // metal_forces inside the pair loop (two_body.F90:367-372)
    g.metal_unsafe = false;
    metal_forces(st);
    if (g.metal_unsafe) return GB_ERR_METAL_TABLE;
  }
  if (eng8) {
    eng8[0] = erc; eng8[1] = vrc; eng8[2] = A.engrl; eng8[3] = A.virrl;
    eng8[4] = A.engex; eng8[5] = A.virex; eng8[6] = A.engvdw; eng8[7] = A.virvdw;
  }
  if (stress9) for (int k = 0; k < 9; ++k) stress9[k] = st[k];
  return GB_OK;
}

}  // namespace

// ============================================================ C interface
extern "C" {

int orc_init(const gb_params* prm, int natms, const int32_t* ltype, const double* chge,
             const double* weight, const int32_t* lfrzn, const double* vdw_prm, int ntcons,
             const int32_t* listcon, const double* prmcon, const int32_t* list_excl) {
  g = Ctx();
  g.p = *prm;
  std::memcpy(g.cell, prm->cell, sizeof(g.cell));
  double det;
  invert(g.cell, g.rcell, &det);
  dcell(g.cell, g.celprp);
  g.volm = g.celprp[9];
  g.rcutx = prm->rcut + prm->rpad;
  g.natms = natms;
  g.mxatms = prm->mxatms;
  int mx = g.mxatms;
  g.x.assign(mx, 0); g.y.assign(mx, 0); g.z.assign(mx, 0);
  g.fx.assign(mx, 0); g.fy.assign(mx, 0); g.fz.assign(mx, 0);
  g.chge.assign(mx, 0); g.weight.assign(mx, 0);
  g.ltg.assign(mx, 0); g.ltype.assign(mx, 0); g.lfrzn.assign(mx, 0); g.ixyz.assign(mx, 0); g.src.assign(mx, 0);
  g.xbg.assign(mx, 0); g.ybg.assign(mx, 0); g.zbg.assign(mx, 0);
  g.vx.assign(natms, 0); g.vy.assign(natms, 0); g.vz.assign(natms, 0);
  g.megfrz = 0;
  for (int i = 0; i < natms; ++i) {
    g.ltype[i] = ltype[i]; g.chge[i] = chge[i]; g.weight[i] = weight[i]; g.lfrzn[i] = lfrzn[i];
    g.ltg[i] = i + 1; g.src[i] = i;
    if (lfrzn[i]) g.megfrz++;
  }
  g.spme_on = false;
  for (int i = 0; i < natms; ++i) g.spme_on = g.spme_on || chge[i] != 0.0;
  g.ld = prm->max_list + 4;
  g.list.assign((size_t)g.ld * natms, 0);
  int ldx = prm->max_exclude + 1;
  g.list_excl.assign((size_t)ldx * natms, 0);
  g.lbook = false;
  if (list_excl) {
    std::memcpy(g.list_excl.data(), list_excl, sizeof(int32_t) * ldx * natms);
    for (int i = 0; i < natms; ++i) if (g.list_excl[(size_t)i * ldx] > 0) g.lbook = true;
  }
  g.nkey = prm->ntypes * (prm->ntypes + 1) / 2;
  g.vdw_kind.assign(g.nkey, 0); g.vdw_eps.assign(g.nkey, 0); g.vdw_sig.assign(g.nkey, 0);
  for (int k = 0; k < g.nkey; ++k) {
    g.vdw_kind[k] = (int)vdw_prm[3 * k];
    g.vdw_eps[k] = vdw_prm[3 * k + 1];
    g.vdw_sig[k] = vdw_prm[3 * k + 2];
  }
  g.nsamples = std::max(1004, (int)std::lround(prm->rcut / 0.01) + 4);
  g.max_grid = std::max(1004, (int)std::lround(prm->rvdw / 0.01) + 4);
  erfcgen();
  vdw_generate();
  vdw_lrc();
  g.scaling = kR4pie0 / prm->epsq;
  double sq2 = 0;
  for (int i = 0; i < natms; ++i) sq2 += chge[i] * chge[i];
  g.self_interaction = -sq2 * (g.scaling * prm->alpha * (1.0 / 1.7724538509055161040) / 1.0);
  g.ntcons = ntcons;
  g.con_type.resize(ntcons); g.con_i.resize(ntcons); g.con_j.resize(ntcons);
  int nct = 0;
  for (int k = 0; k < ntcons; ++k) {
    g.con_type[k] = listcon[3 * k] - 1;
    g.con_i[k] = listcon[3 * k + 1] - 1;
    g.con_j[k] = listcon[3 * k + 2] - 1;
    nct = std::max(nct, listcon[3 * k]);
  }
  g.prmcon.assign(prmcon ? prmcon : nullptr, prmcon ? prmcon + nct : nullptr);
  g.spme_newjob = true;
  g.update = true;
  g.nstep = 0;
  set_ensemble(GB_NVE, 0.0, 0.0, 0.0, nullptr, 0.0);
  g.init = true;
  return GB_OK;
}

int orc_set_threads(int n) { g_nthreads = n < 1 ? 1 : n; return GB_OK; }

int orc_upload_state(const double* x, const double* y, const double* z, const double* vx, const double* vy,
                     const double* vz) {
  if (!g.init) return GB_ERR_NOT_INIT;
  for (int i = 0; i < g.natms; ++i) {
    g.x[i] = x[i]; g.y[i] = y[i]; g.z[i] = z[i];
    if (vx) { g.vx[i] = vx[i]; g.vy[i] = vy[i]; g.vz[i] = vz[i]; }
  }
  return GB_OK;
}

int orc_download_state(double* x, double* y, double* z, double* vx, double* vy, double* vz, double* fx,
                       double* fy, double* fz) {
  if (!g.init) return GB_ERR_NOT_INIT;
  for (int i = 0; i < g.natms; ++i) {
    if (x) { x[i] = g.x[i]; y[i] = g.y[i]; z[i] = g.z[i]; }
    if (vx) { vx[i] = g.vx[i]; vy[i] = g.vy[i]; vz[i] = g.vz[i]; }
    if (fx) { fx[i] = g.fx[i]; fy[i] = g.fy[i]; fz[i] = g.fz[i]; }
  }
  return GB_OK;
}

int orc_relocate(void) {
  if (!g.init) return GB_ERR_NOT_INIT;
  pbcshift();
  try { set_halo_particles(); } catch (int e) { return e; }
  return GB_OK;
}

int orc_list_build(int32_t* list_out, int ldlist, int32_t* max_list_io) {
  if (!g.init) return GB_ERR_NOT_INIT;
  int want = g.p.max_list;
  int st = link_cell_pairs();
  if (st == GB_ERR_LIST_OVERFLOW) {
    if (max_list_io) *max_list_io = g.p.max_list;
    g.p.max_list = want;
    return st;
  }
  if (st) return st;
  if (list_out) {
    if (ldlist != g.ld) return GB_ERR_ARG;
    std::memcpy(list_out, g.list.data(), sizeof(int32_t) * g.list.size());
  }
  return GB_OK;
}

// halo: nlast and per-halo-atom source (0-based local index) and positions
int orc_halo(int32_t* nlast, int32_t* src, double* hx, double* hy, double* hz) {
  if (!g.init) return GB_ERR_NOT_INIT;
  *nlast = g.nlast;
  for (int i = g.natms; i < g.nlast; ++i) {
    if (src) src[i - g.natms] = g.src[i];
    if (hx) { hx[i - g.natms] = g.x[i]; hy[i - g.natms] = g.y[i]; hz[i - g.natms] = g.z[i]; }
  }
  return GB_OK;
}

int orc_vnl_check(int32_t* update) {
  if (!g.init) return GB_ERR_NOT_INIT;
  *update = vnl_check() ? 1 : 0;
  return GB_OK;
}

int orc_refresh(int32_t* update) {
  if (!g.init) return GB_ERR_NOT_INIT;
  bool upd = vnl_check();
  *update = upd ? 1 : 0;
  try {
    if (upd) { pbcshift(); set_halo_particles(); }
    else refresh_halo_positions();
  } catch (int e) { return e; }
  return GB_OK;
}

int orc_forces(double* eng_out, double* stress_out) {
  if (!g.init) return GB_ERR_NOT_INIT;
  return calculate_forces(eng_out, stress_out);
}

int orc_spme(double* eng_rc, double* vir_rc, double* stress_out) {
  if (!g.init) return GB_ERR_NOT_INIT;
  for (int i = 0; i < g.nlast; ++i) { g.fx[i] = 0.0; g.fy[i] = 0.0; g.fz[i] = 0.0; }
  double st[9] = {0};
  spme(eng_rc, vir_rc, st, g.fx.data(), g.fy.data(), g.fz.data());
  if (stress_out) for (int k = 0; k < 9; ++k) stress_out[k] = st[k];
  return GB_OK;
}

int orc_real(double* eng_out, double* stress_out) {
  if (!g.init) return GB_ERR_NOT_INIT;
  for (int i = 0; i < g.nlast; ++i) { g.fx[i] = 0.0; g.fy[i] = 0.0; g.fz[i] = 0.0; }
  Acc A;
  two_body_real(A);
  if (eng_out) {
    eng_out[0] = A.engrl; eng_out[1] = A.virrl; eng_out[2] = A.engex; eng_out[3] = A.virex;
    eng_out[4] = A.engvdw; eng_out[5] = A.virvdw;
  }
  if (stress_out) for (int k = 0; k < 9; ++k) stress_out[k] = A.str[k];
  return GB_OK;
}

int orc_set_metal_eam(int ntab, const int32_t* kind, const int32_t* t1, const int32_t* t2, const int32_t* ngrid,
                      const double* start, const double* finish, const double* values, const int32_t* listed) {
  if (!g.init) return GB_ERR_NOT_INIT;
  if (ntab < 0) return GB_ERR_ARG;
  if (ntab == 0) { g.metal = false; return GB_OK; }
  return metal_tables(ntab, kind, t1, t2, ngrid, start, finish, values, listed);
}

int orc_metal_energies(double* out4) {
  if (!g.init) return GB_ERR_NOT_INIT;
  out4[0] = g.engmet; out4[1] = g.virmet; out4[2] = g.engden; out4[3] = g.virden;
  return GB_OK;
}

int orc_metal_rho(double* out) {
  if (!g.init) return GB_ERR_NOT_INIT;
  if (!g.metal || (int)g.mrho.size() < g.natms) return GB_ERR_ARG;
  for (int i = 0; i < g.natms; ++i) out[i] = g.mrho[i];
  return GB_OK;
}

int orc_set_ensemble(int kind, double temp, double tau_t, double chi, const int32_t* seed, double degfre) {
  if (!g.init) return GB_ERR_NOT_INIT;
  if (kind < GB_NVE || kind > GB_NVT_LANGEVIN) return GB_ERR_ARG;
  if (kind != GB_NVE && !(temp > 0.0)) return GB_ERR_ARG;
  if ((kind == GB_NVT_BERENDSEN || kind == GB_NVT_NOSE_HOOVER) && !(tau_t > 0.0)) return GB_ERR_ARG;
  if (kind == GB_NVT_LANGEVIN && !(chi >= 0.0)) return GB_ERR_ARG;
  return set_ensemble(kind, temp, tau_t, chi, seed, degfre);
}

int orc_set_step(int32_t nstep) {
  if (!g.init) return GB_ERR_NOT_INIT;
  g.nstep = nstep;
  return GB_OK;
}

int orc_thermostat_state(double* chi_t, double* cint, double* consv) {
  if (!g.init) return GB_ERR_NOT_INIT;
  if (chi_t) *chi_t = g.chi_t;
  if (cint) *cint = g.cint;
  if (consv) *consv = g.ens == GB_NVT_NOSE_HOOVER ? g.consv : 0.0;
  return GB_OK;
}

int orc_set_thermostat_state(double chi_t, double cint) {
  if (!g.init) return GB_ERR_NOT_INIT;
  g.chi_t = chi_t;
  g.cint = cint;
  return GB_OK;
}

// sarurnd / box_mueller_saru3 on arrays (no seed shifts); needs no gb_init
int orc_rng_eval(int mode, int n, const int64_t* a, const int64_t* b, const int64_t* c, double* out) {
  if ((mode != 0 && mode != 1) || n < 0) return GB_ERR_ARG;
  int keep[3] = {g.seed[0], g.seed[1], g.seed[2]};
  g.seed[0] = g.seed[1] = g.seed[2] = 0;
  int st = GB_OK;
  for (int i = 0; i < n && st == GB_OK; ++i) {
    if (mode == 0) out[i] = sarurnd(a[i], b[i], c[i]);
    else st = box_mueller_saru3(a[i], b[i], c[i], &out[3 * i], &out[3 * i + 1], &out[3 * i + 2]);
  }
  for (int k = 0; k < 3; ++k) g.seed[k] = keep[k];
  return st;
}

int orc_vv(int stage, double* strkin, double* engke, int32_t* iters, double* vircon, double* strcon) {
  if (!g.init) return GB_ERR_NOT_INIT;
  int it = 0;
  int st = nve_vv(stage, strkin, engke, &it, vircon, strcon);
  if (iters) *iters = it;
  return st;
}

// md_vv loop (drivers.F90:2059-2288) for nsteps, starting from a state whose
// forces are current (orc_forces called after the initial list build).
int orc_md_run(int nsteps, gb_step_stats* stats) {
  if (!g.init) return GB_ERR_NOT_INIT;
  for (int s = 0; s < nsteps; ++s) {
    gb_step_stats S;
    std::memset(&S, 0, sizeof(S));
    int it = 0;
    ++g.nstep;
    int st = nve_vv(1, nullptr, nullptr, &it, &S.vircon, S.strcon);
    if (st) return st;
    S.shake_iters = it;
    int32_t upd = 0;
    st = orc_refresh(&upd);
    if (st) return st;
    S.list_rebuilt = upd;
    if (upd) {
      st = link_cell_pairs();
      if (st) return st;
    }
    double e8[8], st9[9];
    st = calculate_forces(e8, st9);
    if (st) return st;
    S.engcpe_rc = e8[0]; S.vircpe_rc = e8[1]; S.engcpe_rl = e8[2]; S.vircpe_rl = e8[3];
    S.engcpe_ex = e8[4]; S.vircpe_ex = e8[5]; S.engvdw = e8[6]; S.virvdw = e8[7];
    for (int k = 0; k < 9; ++k) S.stress[k] = st9[k];
    st = nve_vv(2, S.strkin, &S.engke, &it, nullptr, nullptr);
    if (st) return st;
    S.rattle_iters = it;
    S.mts_full = 1;
    S.consv = g.ens == GB_NVT_NOSE_HOOVER ? g.consv : 0.0;
    S.engmet = g.engmet + g.engden;
    S.virmet = g.virmet + g.virden;
    if (stats) stats[s] = S;
  }
  return GB_OK;
}

// Known-answer helper: lj_energy at one distance (two_body_potentials.F90:260).
int orc_lj_kat(double eps, double sig, double r, double* e, double* gamma) {
  lj_energy(eps, sig, r, e, gamma);
  return GB_OK;
}

// B-spline values for one coordinate (d[3*s]: derivative 0,1,2 at points 1..s)
int orc_splines(double u, int order, double* out) {
  g.p.nsplines = order;
  for (int n = 0; n < 22; ++n) for (int k = 0; k < 21; ++k) g.ncombk[n][k] = 0.0;
  for (int n = 1; n <= order; ++n)
    for (int k = 0; k <= n; ++k) {
      double a = 1.0, b = 1.0;
      for (int i = n - k + 1; i <= n; ++i) a *= (double)i;
      for (int i = 1; i <= std::max(1, k); ++i) b *= 1.0 / (double)i;
      g.ncombk[k][n] = a * b;
    }
  double d[3][21];
  splines_1d(u, d);
  for (int l = 0; l < 3; ++l) for (int j = 1; j <= order; ++j) out[l * order + (j - 1)] = d[l][j];
  return GB_OK;
}

// Energies that two_body_forces adds outside the pair loop (two_body.F90:766-790).
int orc_constants(double* self_interaction, double* elrc, double* vlrc) {
  if (!g.init) return GB_ERR_NOT_INIT;
  if (self_interaction) *self_interaction = g.self_interaction;
  if (elrc) *elrc = g.elrc;
  if (vlrc) *vlrc = g.vlrc;
  return GB_OK;
}

void orc_finalize(void) { g = Ctx(); }

}  // extern "C"
