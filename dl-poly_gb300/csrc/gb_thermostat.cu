// gb_thermostat.cu - NVT thermostats of the velocity Verlet stages on the device.
//
// Follows:
//   nvt_b0_vv, nvt_b0_scl    source/nvt_berendsen.F90:39-258, :907-962
//   nvt_h0_vv, nvt_h0_scl    source/nvt_nose_hoover.F90 (nvt_h0_vv; nvt_h0_scl)
//   nvt_l0_vv                source/nvt_langevin.F90 (nvt_l0_vv), langevin_scalers :1552-1621
//   langevin_forces          source/langevin.F90:57-194 (setforces branch)
//   sarurnd, box_mueller_saru3  source/numerics.F90:458-635, :745-803
//   getvom, getkin, kinstress   source/kinetics.F90
//   dispatch on thermo%ensemble source/drivers.F90:1132-1175
//
// The thermostat scalars (chi_t, cint, the scale factor, the centre-of-mass
// velocity) live in device memory: a block reduction gives the kinetic stress
// and momentum, one thread advances the thermostat, and the velocity kernels
// read the result, so a stage needs no host round trip until its end.  The
// Langevin random forces are generated inside the position update from the
// counter-based generator keyed on (global atom id, step): nothing is stored.
#include <cfloat>
#include <cmath>

#include "gb_common.cuh"

namespace {

inline int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

constexpr double kBoltz = 0.831451115;  // constants.F90:104

// ---------------------------------------------------------------- random numbers
// The uniform deviate of sarurnd: the SARU generator (Afshar et al., Comput. Phys.
// Commun. 184 (2013) 1119) as the reference evaluates it, in 64-bit integers with
// logical shifts and with the 32x32-bit products formed in double precision and
// reduced modulo 2^32.  Those products round above 2^53, so the stream differs from
// the 32-bit original; this follows the reference's arithmetic step for step so
// that the same (atom, step) gives the same deviate.
__device__ __forceinline__ long long lsl(long long x, int n) { return (long long)((unsigned long long)x << n); }
__device__ __forceinline__ long long lsr(long long x, int n) { return (long long)((unsigned long long)x >> n); }
__device__ __forceinline__ long long sext32(long long x) { return (long long)(int)(unsigned)(unsigned long long)x; }
__device__ __forceinline__ long long mod32(long long x) { return x % 4294967296LL; }
__device__ __forceinline__ long long dmulmod(double c, long long x) {
  return (long long)fmod(__dmul_rn(c, (double)x), 4294967296.0);
}

__device__ double saru_uniform(long long a, long long b, long long c) {
  const long long T32 = 4294967296LL;
  long long s1 = mod32(a), s2 = mod32(b), s3 = mod32(c), t;
  if (s1 < 0) s1 += T32;
  if (s2 < 0) s2 += T32;
  if (s3 < 0) s3 += T32;
  s3 = mod32(s3 ^ (lsl(s1, 7) ^ lsr(s2, 6)));
  s2 = mod32(s2 + (lsr(s1, 4) ^ lsr(s3, 15)));
  s1 = mod32(s1 ^ (lsl(s2, 9) + lsl(s3, 8)));
  s3 = mod32(s3 ^ dmulmod(2771807053.0, lsr(s2, 11) ^ lsl(s1, 1)));
  s2 = mod32(s2 + dmulmod(1925059961.0, lsl(s1, 4) ^ lsr(s3, 16)));
  t = dmulmod(1060677357.0, lsr(s3, 5) ^ lsr(sext32(s2), 22));
  if (t < 0) t += T32;
  s1 = mod32(s1 ^ t);
  s2 = mod32(s2 + (long long)fmod(__dmul_rn((double)s1, (double)s3), 4294967296.0));
  s1 = mod32(s1 + (s3 ^ lsr(s2, 2)));
  s2 = s2 ^ lsr(sext32(s2), 17);
  if (s2 < 0) s2 += T32;
  long long state = dmulmod(2044649123.0, s1 ^ lsr(sext32(s1), 14));
  if (state < 0) state += T32;
  long long wstate = mod32((state + s2) ^ lsr(sext32(state), 8));
  if (wstate < 0) wstate += T32;
  state = mod32(state + (long long)fmod(__dmul_rn((double)wstate, (double)(wstate ^ 3722418165LL)), 4294967296.0));
  wstate = mod32(2882246391LL + lsr(wstate, 1));
  state = mod32(dmulmod(1273716057.0, state) + 637592055LL);
  wstate = mod32(wstate + 2148127051LL + (lsr(sext32(wstate), 31) & 3666320093LL));
  long long v = mod32((state ^ lsr(state, 26)) + wstate);
  long long u32 = dmulmod(1767372199.0, v ^ lsr(v, 20));
  const double r32 = 2.3283064365386963e-10;  // 2^-32
  double p1 = __dadd_rn(__dmul_rn((double)sext32(u32), r32), 0.5 + 0.5 * r32);
  double p2 = __dmul_rn((double)state, r32 * r32);
  return __dadd_rn(p1, p2);
}

// Three unit Gaussians by the polar Box-Muller method on consecutive counters
// (box_mueller_saru3).  The rejection loops are capped; a cap hit sets *bad.
__device__ void gauss3(long long i, long long j, const int* seed, double g[3], int* bad) {
  const long long a = i + seed[0], b = j + seed[1];
  long long k = seed[2];
  double r0 = 1.0, r1 = 0.0, r2 = 0.0;
  int guard = 0;
  while (r0 <= DBL_MIN || r0 >= 1.0) {
    r1 = 2.0 * saru_uniform(a, b, k) - 1.0;
    r2 = 2.0 * saru_uniform(a, b, k + 1) - 1.0;
    r0 = __dadd_rn(__dmul_rn(r1, r1), __dmul_rn(r2, r2));
    k += 2;
    if (++guard > 64) { *bad = 1; r0 = 0.5; break; }
  }
  r0 = sqrt(-2.0 * log(r0) / r0);
  g[0] = r0 * r1;
  g[1] = r0 * r2;
  r0 = 1.0;
  guard = 0;
  while (r0 <= DBL_MIN || r0 >= 1.0) {
    r1 = 2.0 * saru_uniform(a, b, k) - 1.0;
    r2 = 2.0 * saru_uniform(a, b, k + 1) - 1.0;
    r0 = __dadd_rn(__dmul_rn(r1, r1), __dmul_rn(r2, r2));
    k += 2;
    if (++guard > 64) { *bad = 1; r0 = 0.5; break; }
  }
  r0 = sqrt(-2.0 * log(r0) / r0);
  g[2] = r0 * r1;
}

__global__ void k_rng_eval(int mode, int n, const long long* a, const long long* b, const long long* c,
                           double* out, int* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (mode == 0) {
    out[i] = saru_uniform(a[i], b[i], c[i]);
  } else {
    const int seed[3] = {0, 0, (int)c[i]};
    double gg[3];
    int bad = 0;
    gauss3(a[i], b[i], seed, gg, &bad);
    out[3 * i] = gg[0]; out[3 * i + 1] = gg[1]; out[3 * i + 2] = gg[2];
    if (bad) atomicOr(status, ST_RNG);
  }
}

// ---------------------------------------------------------------- velocity kernels
// kinetic stress (6) and momentum (3) of the non-frozen atoms, per block
__global__ void k_kin_mom(int n, const double* w, const int* lfrzn, const double* vx, const double* vy,
                          const double* vz, double* blk) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (i < n && lfrzn[i] == 0) {
    const double m = w[i];
    a[0] = m * vx[i] * vx[i]; a[1] = m * vx[i] * vy[i]; a[2] = m * vx[i] * vz[i];
    a[3] = m * vy[i] * vy[i]; a[4] = m * vy[i] * vz[i]; a[5] = m * vz[i] * vz[i];
    a[6] = m * vx[i]; a[7] = m * vy[i]; a[8] = m * vz[i];
  }
  block_reduce_store<9>(a, blk);
}

// v <- scale * v (every atom), then subtract the centre-of-mass velocity from
// the non-frozen atoms with mass (when sub_vom), then the kinetic stress of the
// result per block
__global__ void k_scale_kin(int n, const double* th, int sub_vom, const double* w, const int* lfrzn, double* vx,
                            double* vy, double* vz, double* blk) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a[6] = {0, 0, 0, 0, 0, 0};
  if (i < n) {
    const double s = th[2];
    double x = vx[i] * s, y = vy[i] * s, z = vz[i] * s;
    if (sub_vom && lfrzn[i] == 0 && w[i] > 1.0e-6) { x -= th[3]; y -= th[4]; z -= th[5]; }
    vx[i] = x; vy[i] = y; vz[i] = z;
    if (lfrzn[i] == 0) {
      const double m = w[i];
      a[0] = m * x * x; a[1] = m * x * y; a[2] = m * x * z; a[3] = m * y * y; a[4] = m * y * z; a[5] = m * z * z;
    }
  }
  block_reduce_store<6>(a, blk);
}

// Nose-Hoover stage 1: v <- scale*v (nvt_h0_scl), then the VV half kick and drift
__global__ void k_vv1_scaled(int n, double hstep, double tstep, const double* th, const double* w, const double* fx,
                             const double* fy, const double* fz, double* vx, double* vy, double* vz, double* x,
                             double* y, double* z) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = th[2];
  double ux = s * vx[i], uy = s * vy[i], uz = s * vz[i];
  if (w[i] > 1.0e-6) {
    const double tmp = hstep / w[i];
    ux = ux + tmp * fx[i];
    uy = uy + tmp * fy[i];
    uz = uz + tmp * fz[i];
    x[i] = x[i] + tstep * ux;
    y[i] = y[i] + tstep * uy;
    z[i] = z[i] + tstep * uz;
  }
  vx[i] = ux; vy[i] = uy; vz[i] = uz;
}

struct LangevinArgs {
  double hstep, tstep, rscale, t0, t1, scr, scl, scv;
  int nstep;
  int seed[3];
};

// Langevin stage 1 (nvt_l0_vv): the random impulses of steps +nstep and -nstep
// (langevin_forces), drawn here per atom, enter the drift and the velocity
__global__ void k_vv1_langevin(int n, LangevinArgs L, const double* w, const int* lfrzn, const int* ltg,
                               const double* fx, const double* fy, const double* fz, double* vx, double* vy,
                               double* vz, double* x, double* y, double* z, int* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !(w[i] > 1.0e-6)) return;
  double fr[3] = {0, 0, 0}, fl[3] = {0, 0, 0};
  if (lfrzn[i] == 0) {
    int bad = 0;
    gauss3(ltg[i], L.nstep, L.seed, fr, &bad);
    gauss3(ltg[i], -L.nstep, L.seed, fl, &bad);
    if (bad) atomicOr(status, ST_RNG);
    const double tmp = L.rscale * sqrt(w[i]);
#pragma unroll
    for (int k = 0; k < 3; ++k) { fr[k] *= tmp; fl[k] *= tmp; }
  }
  double tmp = L.hstep / w[i];
  double ux = vx[i] + tmp * fx[i], uy = vy[i] + tmp * fy[i], uz = vz[i] + tmp * fz[i];
  tmp = L.tstep / w[i];
  x[i] = x[i] + ux * L.t1 + tmp * (fr[0] * L.scr + fl[0] * L.scl);
  y[i] = y[i] + uy * L.t1 + tmp * (fr[1] * L.scr + fl[1] * L.scl);
  z[i] = z[i] + uz * L.t1 + tmp * (fr[2] * L.scr + fl[2] * L.scl);
  vx[i] = ux * L.t0 + tmp * fr[0] * L.scv;
  vy[i] = uy * L.t0 + tmp * fr[1] * L.scv;
  vz[i] = uz * L.t0 + tmp * fr[2] * L.scv;
}

// ---------------------------------------------------------------- thermostat scalars (one thread)
// Nose-Hoover half step of the thermostat (nvt_h0_scl with tstep = ts, pmass = 0):
// kinetic energy from the reduced kinetic stress
__global__ void k_nh_scalars(DevScalars* sc, double ts, double qmass, double ceng) {
  double* th = sc->th;
  const double* k = &sc->acc[A_KINMOM];
  const double hs = 0.5 * ts, qs = 0.5 * hs;
  th[1] = th[1] + qs * th[0];
  double engke = 0.5 * (k[0] + k[3] + k[5]);
  th[0] = th[0] + hs * (2.0 * engke - ceng) / qmass;
  th[1] = th[1] + hs * th[0];
  const double scale = exp(-ts * th[0]);
  th[2] = scale;
  engke = engke * (scale * scale);
  th[6] = engke;
  th[0] = th[0] + hs * (2.0 * engke - ceng) / qmass;
  th[1] = th[1] + qs * th[0];
  th[7] = 0.5 * qmass * th[0] * th[0] + ceng * th[1];
  th[3] = th[4] = th[5] = 0.0;
}

// Berendsen scale (nvt_b0_scl) and, with it or alone (Langevin), the centre-of-mass
// velocity after scaling (getvom)
__global__ void k_scale_vom_scalars(DevScalars* sc, int berendsen, double tstep, double tau_t, double sigma,
                                    double totmas) {
  double* th = sc->th;
  const double* k = &sc->acc[A_KINMOM];
  double chi = 1.0;
  if (berendsen) {
    const double engke = 0.5 * (k[0] + k[3] + k[5]);
    chi = sqrt(1.0 + tstep / tau_t * (sigma / engke - 1.0));
  }
  th[2] = chi;
  const double inv = totmas >= DBL_MIN ? 1.0 / totmas : 0.0;
  th[3] = chi * k[6] * inv;
  th[4] = chi * k[7] * inv;
  th[5] = chi * k[8] * inv;
}

// Berendsen: chi_t recomputed from the final kinetic energy (the second nvt_b0_scl call)
__global__ void k_berendsen_final(DevScalars* sc, double tstep, double tau_t, double sigma) {
  const double* s = &sc->acc[A_STRKIN];
  const double engke = 0.5 * (s[0] + s[3] + s[5]);
  sc->th[0] = sqrt(1.0 + tstep / tau_t * (sigma / engke - 1.0));
}

}  // namespace

// ---------------------------------------------------------------- host side
// langevin_scalers (nvt_langevin.F90:1552-1621)
static void langevin_scalers(double chi, double tstep, double* t0, double* t1, double* scr, double* scv,
                             double* scl) {
  const double stol = 1.0e-3;
  *t0 = std::exp(-chi * tstep);
  if (chi <= DBL_MIN) {
    *t1 = tstep;
    *scr = 0.0; *scl = 0.0; *scv = 0.0;
    return;
  }
  *t1 = (1.0 - *t0) / chi;
  const double al = 0.5 * chi * tstep;
  if (al < stol) {
    *scr = (al - al * al + 0.5 * (al * al * al) - (al * al * al * al) / 6.0 + 0.075 * (al * al * al * al * al)) / chi;
    *scl = (al - 0.2 * (al * al * al) + (32.0 * (al * al * al * al * al)) / 525.0) / (chi * std::sqrt(3.0));
    *scv = 1.0 - al + 5.0 * (al * al) / 6.0 - 0.5 * (al * al * al);
  } else {
    *scr = (1.0 - *t0) * (1.0 - *t0) / (std::sqrt(al * (1.0 - *t0 * *t0)) * 2.0 * chi);
    *scl = std::sqrt(1.0 - std::tanh(al) / al) / chi;
    *scv = std::sqrt((1.0 - *t0 * *t0) / (4.0 * al));
  }
}

void thermo_setup(int kind, double temp, double tau_t, double chi, const int32_t* seed, double degfre) {
  g.ens = kind;
  g.temp = temp;
  g.tau_t = tau_t;
  g.chi_fric = chi;
  for (int k = 0; k < 3; ++k) g.seed[k] = seed ? seed[k] : 0;
  if (degfre <= 0.0) {  // temperature.F90:109-143: 3 per free atom, less the centre of mass and constraints
    degfre = 3.0 * (double)(g.natms - g.megfrz) - 3.0 - (double)g.ntcons;
  }
  g.degfre = degfre;
  g.sigma = 0.5 * degfre * kBoltz * temp;       // temperature.F90:178
  g.qmass = 2.0 * g.sigma * tau_t * tau_t;      // nvt_h0_vv first call
  g.ceng = 2.0 * g.sigma;
  std::vector<double> w(g.natms);
  std::vector<int> fz(g.natms);
  GB_CUDA(cudaMemcpy(w.data(), g.weight, sizeof(double) * g.natms, cudaMemcpyDeviceToHost));
  GB_CUDA(cudaMemcpy(fz.data(), g.lfrzn, sizeof(int) * g.natms, cudaMemcpyDeviceToHost));
  double tm = 0.0;
  for (int i = 0; i < g.natms; ++i)
    if (fz[i] == 0) tm += w[i];
  g.totmas = tm;
  langevin_scalers(chi, g.p.tstep, &g.lang_t0, &g.lang_t1, &g.lang_scr, &g.lang_scv, &g.lang_scl);
  thermo_set_state(0.0, 0.0);
}

void thermo_set_state(double chi_t, double cint) {
  double th[8] = {chi_t, cint, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  GB_CUDA(cudaMemcpyAsync(g.sc->th, th, sizeof(th), cudaMemcpyHostToDevice, g.stream));
  GB_CUDA(cudaStreamSynchronize(g.stream));
}

void thermo_state(double* chi_t, double* cint, double* consv) {
  gb_sync_scalars();
  if (chi_t) *chi_t = g.hsc->th[0];
  if (cint) *cint = g.hsc->th[1];
  if (consv) *consv = g.ens == GB_NVT_NOSE_HOOVER ? g.hsc->th[7] : 0.0;
}

static void reduce_kin_mom() {
  const int nb = nblocks(g.natms, 256);
  double* blk = gb_blkacc(nb * 9);
  k_kin_mom<<<nb, 256, 0, g.stream>>>(g.natms, g.weight, g.lfrzn, g.vx, g.vy, g.vz, blk);
  GB_LAUNCHED();
  gb_reduce_blocks(blk, nb, 9, &g.sc->acc[A_KINMOM]);
}

bool thermo_vv1(double hstep, double tstep) {
  const int n = g.natms, nb = nblocks(n, 256);
  if (g.ens == GB_NVT_NOSE_HOOVER) {
    reduce_kin_mom();
    k_nh_scalars<<<1, 1, 0, g.stream>>>(g.sc, hstep, g.qmass, g.ceng);
    GB_LAUNCHED();
    k_vv1_scaled<<<nb, 256, 0, g.stream>>>(n, hstep, tstep, g.sc->th, g.weight, g.fx, g.fy, g.fz, g.vx, g.vy, g.vz,
                                           g.x, g.y, g.z);
    GB_LAUNCHED();
    return true;
  }
  if (g.ens == GB_NVT_LANGEVIN) {
    LangevinArgs L;
    L.hstep = hstep; L.tstep = tstep;
    L.rscale = std::sqrt(2.0 * g.chi_fric * kBoltz * g.temp / tstep);
    L.t0 = g.lang_t0; L.t1 = g.lang_t1; L.scr = g.lang_scr; L.scl = g.lang_scl; L.scv = g.lang_scv;
    L.nstep = g.nstep;
    for (int k = 0; k < 3; ++k) L.seed[k] = g.seed[k];
    k_vv1_langevin<<<nb, 256, 0, g.stream>>>(n, L, g.weight, g.lfrzn, g.ltg, g.fx, g.fy, g.fz, g.vx, g.vy, g.vz,
                                             g.x, g.y, g.z, &g.sc->status);
    GB_LAUNCHED();
    return true;
  }
  return false;
}

bool thermo_vv2_finish(double* strkin, double* engke) {
  if (g.ens == GB_NVE) return false;
  const int n = g.natms, nb = nblocks(n, 256);
  reduce_kin_mom();
  int sub_vom = 1;
  if (g.ens == GB_NVT_NOSE_HOOVER) {
    k_nh_scalars<<<1, 1, 0, g.stream>>>(g.sc, 0.5 * g.p.tstep, g.qmass, g.ceng);
    sub_vom = 0;
  } else {
    k_scale_vom_scalars<<<1, 1, 0, g.stream>>>(g.sc, g.ens == GB_NVT_BERENDSEN ? 1 : 0, g.p.tstep, g.tau_t,
                                               g.sigma, g.totmas);
  }
  GB_LAUNCHED();
  double* blk = gb_blkacc(nb * 6);
  k_scale_kin<<<nb, 256, 0, g.stream>>>(n, g.sc->th, sub_vom, g.weight, g.lfrzn, g.vx, g.vy, g.vz, blk);
  GB_LAUNCHED();
  gb_reduce_blocks(blk, nb, 6, &g.sc->acc[A_STRKIN]);
  if (g.ens == GB_NVT_BERENDSEN) {
    k_berendsen_final<<<1, 1, 0, g.stream>>>(g.sc, g.p.tstep, g.tau_t, g.sigma);
    GB_LAUNCHED();
  }
  gb_sync_scalars();
  const double* s = &g.hsc->acc[A_STRKIN];
  double sk[9] = {s[0], s[1], s[2], s[1], s[3], s[4], s[2], s[4], s[5]};
  if (strkin) for (int k = 0; k < 9; ++k) strkin[k] = sk[k];
  if (engke) *engke = g.ens == GB_NVT_NOSE_HOOVER ? g.hsc->th[6] : 0.5 * (sk[0] + sk[4] + sk[8]);
  return true;
}

void rng_eval(int mode, int n, const int64_t* a, const int64_t* b, const int64_t* c, double* out) {
  if (n <= 0) return;
  const int nv = mode == 0 ? 1 : 3;
  long long* d = nullptr;
  double* o = nullptr;
  GB_CUDA(cudaMalloc(&d, sizeof(long long) * 3 * (size_t)n));
  GB_CUDA(cudaMalloc(&o, sizeof(double) * nv * (size_t)n));
  GB_CUDA(cudaMemcpy(d, a, sizeof(long long) * n, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(d + n, b, sizeof(long long) * n, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(d + 2 * (size_t)n, c, sizeof(long long) * n, cudaMemcpyHostToDevice));
  k_rng_eval<<<nblocks(n, 256), 256, 0, g.stream>>>(mode, n, d, d + n, d + 2 * (size_t)n, o, &g.sc->status);
  GB_LAUNCHED();
  GB_CUDA(cudaMemcpyAsync(out, o, sizeof(double) * nv * (size_t)n, cudaMemcpyDeviceToHost, g.stream));
  GB_CUDA(cudaStreamSynchronize(g.stream));
  cudaFree(d);
  cudaFree(o);
}
