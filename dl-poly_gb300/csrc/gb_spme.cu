// gb_spme.cu - SPME reciprocal space on the device.
//
// Follows ewald_spme_forces_coul (source/ewald_spole.F90:244-477):
//   fractional coordinates u = K (rcell . r + 1/2)            (:364-370)
//   B-splines of order p            bspline_splines_gen (bspline.F90:192-306)
//   charge spreading                spme_construct_charge_array (ewald_general.F90:517-576)
//   FFT, influence function, stress spme_construct_potential_grid_coul (ewald_spole.F90:1257-1386)
//   force / energy gather, net-force removal spme_calc_force_energy (ewald_general.F90:717-869)
//
// The reference spreads local atoms and their positive halo images with the
// grid clamped to [0,K); that is the periodic spread of every atom with
// floor-based splines, which is what the brick kernel computes (no halo
// needed).  The gather uses the reference's own truncation convention
// (n = Int(u), w = u - Aint(u)) and periodic grid reads, so atoms that drifted
// out of the cell between relocations get the same spline values.
//
// Spreading is atomic free: atoms are sorted by grid brick (B >= p-1 points
// per side); one CTA owns a brick and gathers from the 2x2x2 source bricks
// whose atoms can reach it, one thread per grid row along x.
//
// The 3-D FFT is an in-shared-memory Stockham transform (radix 4, 3, 5, 2)
// along x, y and z; the z pass applies the influence function theta(m)
// (precomputed in FP64 on the host: |b(m)|^2 exp(-pi^2 m^2/a^2)/(sqrt(pi) f^2)
// inside the spherical cut) and accumulates the reciprocal stress, then runs
// the inverse z transform on the same tile before writing it back.
#include <cfloat>
#include <climits>
#include <cmath>

#include "gb_common.cuh"
#include "gb_dfr.cuh"
#include "gb_fft.cuh"

namespace {

constexpr int PMAX = 12;

// ------------------------------------------------------------ spline prep
// Cardinal B-spline values M_p(w + p - 1 - t), t = 0..p-1, by the order
// recursion of bspline_splines_gen (bspline.F90:227-245), valid as the
// polynomial pieces for any w (the reference also feeds w outside [0,1)).
// P > 0 fixes the order at compile time: the recursion unrolls into registers
// and 1/(n-1) folds to the same correctly rounded constant the division gives.
template <typename T, int P = 0>
__device__ __forceinline__ void bspline_vals(T w, int p_rt, T* m /*p*/, T* dm /*p or null*/) {
  const int p = P ? P : p_rt;
  // z[j], j = 1..p as in the reference (z[p] <-> M(w), z[1] <-> M(w+p-1))
  T z[PMAX + 2];
#pragma unroll
  for (int j = 0; j < PMAX + 2; ++j) z[j] = (T)0;
  z[p] = w;
  z[p - 1] = (T)1 - w;
  // raise from order 2 to order p-1
#pragma unroll
  for (int n = 3; n <= p - 1; ++n) {
    const T rn = T(1.0 / (double)(n - 1));
#pragma unroll
    for (int j = p - n + 1; j <= p - 1; ++j) {
      const T pt = w + (T)(p - j);
      z[j] = (pt * z[j] + ((T)n - pt) * z[j + 1]) * rn;
    }
    z[p] = z[p] * w * rn;
  }
  if (dm) {
    // derivative of order p from order p-1 values: M_{p-1}(x) - M_{p-1}(x-1)
#pragma unroll
    for (int j = 1; j <= p; ++j) dm[j - 1] = z[j] - z[j + 1];
  }
  {
    const int n = p;
    const T rn = T(1.0 / (double)(n - 1));
#pragma unroll
    for (int j = 1; j <= p - 1; ++j) {
      const T pt = w + (T)(p - j);
      z[j] = (pt * z[j] + ((T)n - pt) * z[j + 1]) * rn;
    }
    z[p] = z[p] * w * rn;
  }
  // output in grid order t = 0..p-1  <->  reference spline index s = t+1
#pragma unroll
  for (int t = 0; t < p; ++t) m[t] = z[t + 1];
}

// Splines and brick binning: a CTA takes PREP_AT atoms with one thread per atom and
// dimension (threads d * PREP_AT + a), so that each thread builds one spline; the
// dimension-0 threads then combine the three brick coordinates through shared memory.
constexpr int PREP_AT = 64;
template <typename T, int P>
__global__ void __launch_bounds__(3 * PREP_AT, std::is_same<T, dfr>::value ? 5 : 0) k_spme_prep(int natms, const double* __restrict__ x,
                                                           const double* __restrict__ y, const double* __restrict__ z,
                                                           const double* __restrict__ q, SpmeGeom sg, T* spl,
                                                           int* nidx, int* brick_of, int* brick_count, int* gidx,
                                                           float* gw, float2* gq, T* gsp) {
  __shared__ int bsh[3][PREP_AT];
  const int d = threadIdx.x / PREP_AT, a = threadIdx.x - d * PREP_AT;
  const int i = blockIdx.x * PREP_AT + a;
  const int p = P ? P : sg.p;
  if (i < natms) {
    const double u = sg.Kr[d] * (((sg.rc[d] * x[i] + sg.rc[d + 3] * y[i]) + sg.rc[d + 6] * z[i]) + 0.5);
    const double fl = floor(u);
    const int n = (int)fl;
    const T w = (T)(u - fl);
    double tr = fl;
    if (gidx) {
      // the gather's own convention: Int(u), u - Aint(u) (ewald_spole.F90:387, bspline.F90:216)
      tr = trunc(u);
      int g0 = ((int)tr - p + 1) % sg.K[d];
      if (g0 < 0) g0 += sg.K[d];
      gidx[3 * i + d] = g0;
      if (gw) gw[3 * i + d] = (float)(u - tr);
    }
    T m[PMAX], dm[PMAX];
    bspline_vals<T, P>(w, p, m, gsp ? dm : nullptr);
    // the z splines carry the charge: the spreads weight a point by Mx (My (Mz q))
    const T qT = d == 2 ? (T)q[i] : T(1);
#pragma unroll
    for (int t = 0; t < p; ++t) spl[((size_t)i * 3 + d) * p + t] = d == 2 ? m[t] * qT : m[t];
    if (gsp) {
      // the double-float gather's splines, values then derivatives, z ones times the
      // charge, component-major ([value, derivative][x, y, z][point][atom]: coalesced
      // here and in the gather's copy).  u - Aint(u) differs from u - floor(u) only for
      // u < 0 (an atom just below the cell's lower face)
      if (tr != fl) bspline_vals<T, P>((T)(u - tr), p, m, dm);
      T* o = gsp + (size_t)d * p * natms + i;
      const size_t dstep = (size_t)3 * p * natms;
#pragma unroll
      for (int t = 0; t < p; ++t) {
        o[(size_t)t * natms] = d == 2 ? m[t] * qT : m[t];
        o[dstep + (size_t)t * natms] = d == 2 ? dm[t] * qT : dm[t];
      }
    }
    int nw = n % sg.K[d];
    if (nw < 0) nw += sg.K[d];
    nidx[3 * i + d] = nw;
    bsh[d][a] = nw / sg.B[d];
  }
  __syncthreads();
  if (d != 0 || i >= natms) return;
  int b = bsh[0][a] + sg.nb[0] * (bsh[1][a] + sg.nb[1] * bsh[2][a]);
  if (fabs(q[i]) <= DBL_MIN) b = -1;
  if (gq) {  // double-float gather: the charge, zero for atoms that take no part
    float h = 0.f, l = 0.f;
    if (b >= 0) df_split(q[i], &h, &l);
    gq[i] = make_float2(h, l);
  }
  brick_of[i] = b;
  // the lanes of a warp that share a brick add their count with one atomic (atoms of
  // nearby index are near each other in the lattice start); counts are order-independent
  const unsigned grp = __match_any_sync(__activemask(), b);
  if (b >= 0 && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&brick_count[b], __popc(grp));
}

// atoms into their bricks' ranges; the lanes of a warp that share a brick take
// consecutive slots with one atomic
__global__ void k_brick_scatter(int natms, const int* brick_of, const int* start, int* fill, int* tmp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natms) return;
  const int b = brick_of[i];
  const int lane = threadIdx.x & 31;
  const unsigned grp = __match_any_sync(__activemask(), b);
  const int leader = __ffs(grp) - 1;
  int base = 0;
  if (b >= 0 && lane == leader) base = atomicAdd(&fill[b], __popc(grp));
  base = __shfl_sync(grp, base, leader);
  if (b < 0) return;
  tmp[start[b] + base + __popc(grp & ((1u << lane) - 1u))] = i;
}

__global__ void k_brick_sort(int nbricks, const int* start, const int* tmp, int* out) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nbricks) return;
  int s = start[warp], n = start[warp + 1] - s;
  for (int a = lane; a < n; a += 32) {
    int v = tmp[s + a], r = 0;
    for (int b = 0; b < n; ++b) r += tmp[s + b] < v;
    out[s + r] = v;
  }
}

// ------------------------------------------------------------- spreading
constexpr int SPREAD_CH = 32;
constexpr int SPREAD_NT = 512;             // threads of a tile-spread CTA
constexpr int SPREAD_NW = SPREAD_NT / 32;  // its warps (a power of two: plane owner = z & (NW - 1))
constexpr int BMAX = 16;

// tile point += a * b.  Double-float tiles hold unnormalised compensated pairs: the exact
// product's high part enters a two-sum with the point's sum, its rounding error and cross
// terms the correction (12 FP32 operations; the halo reduction renormalises)
template <typename T>
__device__ __forceinline__ T tile_upd(T v, T a, T b) { return fma(a, b, v); }
template <>
__device__ __forceinline__ dfr tile_upd<dfr>(dfr v, dfr a, dfr b) {
  dacc c;
  c.s = v.hi;
  c.c = v.lo;
  dacc_add_prod(c, to_df(a), to_df(b));
  return dfr(c.s, c.c);
}
template <typename T>
__device__ __forceinline__ void tile_acc(T* dst, T a, T b) { *dst = tile_upd(*dst, a, b); }

// Tile scatter: CTA = one brick and the atoms whose floor(u) lies in it.  The
// CTA owns a (B+p-1)^3 shared-memory tile covering the brick plus the p-1
// points below it that its atoms reach; atoms are scattered one after another
// (one FMA per grid point, no atomics; each warp owns every nw-th z plane of the
// tile, so a chunk of atoms needs one barrier; launched with SPREAD_NT threads),
// then the tile is written to its own slot of `ext` for the halo reduction below.
// Per chunk atom the set-up stores Mx, the p x p products My (Mz q) and the atom's
// tile offset with its z and y offsets (one 16-byte read per atom in the scatter).
// NT = 256 (order 8): warp w owns the tile planes z = w (mod 8) and takes the whole plane
// of each atom, two points per lane (rows k and k + 4), two independent updates.
template <typename T, int P, int NT = SPREAD_NT>
__global__ void k_spme_spread_tile(SpmeGeom sg, const int* __restrict__ bstart, const int* __restrict__ batoms,
                                   const T* __restrict__ spl, const int* __restrict__ nidx,
                                   const double* __restrict__ q, T* __restrict__ ext) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int p = P ? P : sg.p;
  const int b = blockIdx.x;
  const int bx = b % sg.nb[0], by = (b / sg.nb[0]) % sg.nb[1], bz = b / (sg.nb[0] * sg.nb[1]);
  const int g0x = bx * sg.B[0], g0y = by * sg.B[1], g0z = bz * sg.B[2];
  const int TXd = sg.B[0] + p - 1, TYd = sg.B[1] + p - 1, TZd = sg.B[2] + p - 1;
  const int PL = TXd * TYd;
  const int tsize = PL * TZd;
  int4* info = reinterpret_cast<int4*>(smem_raw);  // [SPREAD_CH] tile offset, z offset, y offset, x offset
  T* Pkl = reinterpret_cast<T*>(info + SPREAD_CH);  // [SPREAD_CH][p*p] My(k) * q Mz(l)
  T* Mx = Pkl + SPREAD_CH * p * p;                   // [SPREAD_CH][p]
  T* tile = Mx + SPREAD_CH * p;
  for (int e = threadIdx.x; e < tsize; e += blockDim.x) tile[e] = (T)0;
  const int s0 = bstart[b], s1 = bstart[b + 1];
  const int p2 = p * p;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = s0; c < s1; c += SPREAD_CH) {
    const int nc = min(SPREAD_CH, s1 - c);
    __syncthreads();
    for (int e = threadIdx.x; e < nc * p; e += blockDim.x) {
      const int a = e / p, t = e - a * p;
      const int i = batoms[c + a];
      Mx[a * p + t] = spl[((size_t)i * 3 + 0) * p + t];
      if (t == 0) {
        const int ox = nidx[3 * i + 0] - g0x, oy = nidx[3 * i + 1] - g0y, oz = nidx[3 * i + 2] - g0z;
        info[a] = make_int4(oz * PL + oy * TXd + ox, oz, oy, ox);
      }
    }
    for (int e = threadIdx.x; e < nc * p2; e += blockDim.x) {
      const int a = e / p2, kl = e - a * p2, k = kl % p, l = kl / p;
      const int i = batoms[c + a];
      Pkl[a * p2 + kl] = spl[((size_t)i * 3 + 1) * p + k] * spl[((size_t)i * 3 + 2) * p + l];  // My (Mz q)
    }
    __syncthreads();
    // every tile point is only ever written by one warp, in atom order, so the warps run
    // through the chunk without a barrier per atom.  Orders up to 8: the points of tile
    // plane z and row y belong to warp (z mod 8) + 8 (y mod 2), so every warp takes one
    // plane and every other row of each atom (for p = 8 one point per lane); higher orders:
    // plane z belongs to warp z mod NW.
    constexpr int NW = NT / 32;
    if constexpr (NT == 256) {
      static_assert(P == 8, "eight warps: one plane of an order-8 atom each");
      const int j = lane & 7, m = lane >> 3;  // column, first row
      const T* mxj = Mx + j;
      T* tj = tile + j;
      for (int a = 0; a < nc; ++a) {
        const int4 f = info[a];
        const int l = (wid - f.y) & 7;
        T* d0 = tj + (f.x + l * PL + m * TXd);
        T* d1 = d0 + 4 * TXd;
        const T mx = mxj[a * 8];
        const T* pk = Pkl + a * 64 + l * 8;
        const T v0 = *d0, v1 = *d1;
        *d0 = tile_upd(v0, mx, pk[m]);
        *d1 = tile_upd(v1, mx, pk[m + 4]);
      }
      __syncwarp();
    } else if (p <= 8) {
      static_assert(NW == 16, "the split below gives warps w and w + 8 the even and odd rows");
      const int grp = wid & 7, half = wid >> 3;
      const int m = lane / p, j = lane - m * p;  // this lane's row pair and column
      const T* mxj = Mx + j;
      T* tj = tile + j;
      for (int a = 0; a < nc; ++a) {
        const int4 f = info[a];
        const int l = (grp - f.y) & 7;
        const int k = ((half - f.z) & 1) + 2 * m;
        if (l < p && k < p) tile_acc(tj + (f.x + l * PL + k * TXd), mxj[a * p], Pkl[a * p2 + l * p + k]);
      }
      __syncwarp();
    } else {
      for (int a = 0; a < nc; ++a) {
        const int4 f = info[a];
        for (int l = (wid - f.y) & (NW - 1); l < p; l += NW) {
          T* plane = tile + f.x + l * PL;
          for (int kj = lane; kj < p2; kj += 32) {
            const int j = kj % p, k = kj / p;
            tile_acc(plane + (k * TXd + j), Mx[a * p + j], Pkl[a * p2 + l * p + k]);
          }
        }
        __syncwarp();
      }
    }
  }
  __syncthreads();
  T* out = ext + (size_t)b * tsize;
  for (int e = threadIdx.x; e < tsize; e += blockDim.x) out[e] = tile[e];
}

// Mixed form: the same tile decomposition, but warps scatter different atoms
// concurrently with 64-bit integer shared-memory atomics on a 2^-40 fixed-point
// tile (no barrier per atom; integer sums are order independent, so the grid
// is bit-reproducible).  The tile goes to `ext` as int64.
template <int P>  // spline order known at compile time (0: taken from sg.p)
__global__ void k_spme_spread_fix(SpmeGeom sg, const int* __restrict__ bstart, const int* __restrict__ batoms,
                                  const float* __restrict__ spl, const int* __restrict__ nidx,
                                  const double* __restrict__ q, long long* __restrict__ ext) {
  extern __shared__ unsigned char smem_raw[];
  const int p = P ? P : sg.p;
  const int b = blockIdx.x;
  const int bx = b % sg.nb[0], by = (b / sg.nb[0]) % sg.nb[1], bz = b / (sg.nb[0] * sg.nb[1]);
  const int g0x = bx * sg.B[0], g0y = by * sg.B[1], g0z = bz * sg.B[2];
  const int TXd = sg.B[0] + p - 1, TYd = sg.B[1] + p - 1, TZd = sg.B[2] + p - 1;
  const int tsize = TXd * TYd * TZd;
  long long* tile = reinterpret_cast<long long*>(smem_raw);
  for (int e = threadIdx.x; e < tsize; e += blockDim.x) tile[e] = 0;
  __syncthreads();
  const int s0 = bstart[b], s1 = bstart[b + 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int p2 = p * p, p3 = p2 * p;
  for (int a = s0 + wid; a < s1; a += nw) {
    const int i = batoms[a];
    const float* sx = spl + ((size_t)i * 3 + 0) * p;
    const float* sy = sx + p;
    const float* sz = sy + p;
    const int ox = nidx[3 * i] - g0x, oy = nidx[3 * i + 1] - g0y, oz = nidx[3 * i + 2] - g0z;
    for (int e = lane; e < p3; e += 32) {
      const int j = e % p, kl = e / p, k = kl % p, l = kl / p;
      const float w = sx[j] * (sy[k] * sz[l]);  // sz carries q
      atomicAdd((unsigned long long*)&tile[((oz + l) * TYd + (oy + k)) * TXd + (ox + j)],
                (unsigned long long)fix40(w));
    }
    (void)p2;
  }
  __syncthreads();
  long long* out = ext + (size_t)b * tsize;
  for (int e = threadIdx.x; e < tsize; e += blockDim.x) out[e] = tile[e];
}
// The tiles that cover grid index g along one dimension: its own brick b0 (tile
// coordinate g - b0 B + p - 1) and, when g lies in the lower halo of the next
// brick, that brick too (periodic).
struct TileCover {
  int b[2], t[2], n;
};
__device__ __forceinline__ TileCover tile_cover(int g, int B, int p, int nb) {
  TileCover c;
  const int b0 = g / B;
  c.b[0] = b0;
  c.t[0] = g - b0 * B + p - 1;
  c.b[1] = b0 + 1 == nb ? 0 : b0 + 1;
  c.t[1] = c.t[0] - B;
  c.n = c.t[1] >= 0 ? 2 : 1;
  return c;
}

// Halo reduction: every grid point sums, in a fixed order (z, then y, then x
// covering tile), the tile entries of the (at most 2 per dimension) bricks
// whose tiles cover it.  Launched on a (x blocks, K1, K2) grid: y and z come
// from the block index, so the per-point index arithmetic is one division.
template <typename T, typename S>
__device__ __forceinline__ S tile_sum(const SpmeGeom& sg, const T* __restrict__ ext, int gx, int gy, int gz) {
  const int p = sg.p;
  const int TXd = sg.B[0] + p - 1, TYd = sg.B[1] + p - 1, TZd = sg.B[2] + p - 1;
  const size_t tsize = (size_t)TXd * TYd * TZd;
  const TileCover cx = tile_cover(gx, sg.B[0], p, sg.nb[0]);
  const TileCover cy = tile_cover(gy, sg.B[1], p, sg.nb[1]);
  const TileCover cz = tile_cover(gz, sg.B[2], p, sg.nb[2]);
  // all (up to 8) covering entries are loaded before the sum; absent ones are zero,
  // and adding an exact zero leaves the sum unchanged, so the order of the others holds
  T v[8];
#pragma unroll
  for (int iz = 0; iz < 2; ++iz)
#pragma unroll
    for (int iy = 0; iy < 2; ++iy)
#pragma unroll
      for (int ix = 0; ix < 2; ++ix) {
        T e = (T)0;
        if (iz < cz.n && iy < cy.n && ix < cx.n) {
          const int b = cx.b[ix] + sg.nb[0] * (cy.b[iy] + sg.nb[1] * cz.b[iz]);
          e = ext[(size_t)b * tsize + ((size_t)cz.t[iz] * TYd + cy.t[iy]) * TXd + cx.t[ix]];
        }
        v[(iz * 2 + iy) * 2 + ix] = e;
      }
  S s = (S)0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += v[k];
  return s;
}

// fixed-point halo reduction for the mixed form (int64 sums, one conversion per point)
__global__ void k_spme_tile_reduce_fix(SpmeGeom sg, const long long* __restrict__ ext, float* __restrict__ Q) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x, gy = blockIdx.y, gz = blockIdx.z;
  if (gx >= sg.K[0]) return;
  const long long s = tile_sum<long long, long long>(sg, ext, gx, gy, gz);
  Q[((size_t)gz * sg.K[1] + gy) * sg.K[0] + gx] = (float)s * 9.094947017729282e-13f;  // 2^-40
}

template <typename T>
__global__ void k_spme_tile_reduce(SpmeGeom sg, const T* __restrict__ ext, T* __restrict__ Q) {
  const int gx = blockIdx.x * blockDim.x + threadIdx.x, gy = blockIdx.y, gz = blockIdx.z;
  if (gx >= sg.K[0]) return;
  Q[((size_t)gz * sg.K[1] + gy) * sg.K[0] + gx] = tile_sum<T, T>(sg, ext, gx, gy, gz);
}

inline size_t spread_smem(int B0, int B1, int B2, int p, size_t esz) {
  const size_t tsize = (size_t)(B0 + p - 1) * (B1 + p - 1) * (B2 + p - 1);
  return esz * (tsize + (size_t)SPREAD_CH * p * p + (size_t)SPREAD_CH * p) + sizeof(int4) * SPREAD_CH;
}

// --------------------------------------------------------------- gather
// per atom: trunc-based splines (Int(u), u - Aint(u)), p^3 periodic grid
// reads of the real potential, separable sums.  Writes the unscaled force
// -(K.rcell) q sum dM M M phi and accumulates energy and net force.
template <typename T, int P>
__global__ void k_spme_gather(int natms, const double* __restrict__ x, const double* __restrict__ y,
                              const double* __restrict__ z, const double* __restrict__ q, SpmeGeom sg,
                              const T* __restrict__ phi, double rk0, double rk1, double rk2, double* fout,
                              double* blk) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[4] = {0, 0, 0, 0};
  if (i < natms && fabs(q[i]) > DBL_MIN) {
    const int p = P ? P : sg.p;
    T m[3][PMAX], dm[3][PMAX];
    int n0[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double u = sg.Kr[d] * (((sg.rc[d] * x[i] + sg.rc[d + 3] * y[i]) + sg.rc[d + 6] * z[i]) + 0.5);
      double tr = trunc(u);
      int n = (int)tr;
      bspline_vals<T, P>((T)(u - tr), p, m[d], dm[d]);
      n0[d] = n - p + 1;
    }
    const int K0 = sg.K[0], K1 = sg.K[1], K2 = sg.K[2];
    int ix[PMAX];
#pragma unroll
    for (int t = 0; t < p; ++t) { int v = (n0[0] + t) % K0; if (v < 0) v += K0; ix[t] = v; }
    const T qi = (T)q[i];
    // separable sums: rows along x first, then y within a z plane, then z
    T e = 0, fxs = 0, fys = 0, fzs = 0;
#pragma unroll
    for (int l = 0; l < p; ++l) {
      int zz = (n0[2] + l) % K2; if (zz < 0) zz += K2;
      T a0 = 0, a1 = 0, a2 = 0;
#pragma unroll
      for (int k = 0; k < p; ++k) {
        int yy = (n0[1] + k) % K1; if (yy < 0) yy += K1;
        const T* row = phi + ((size_t)zz * K1 + yy) * K0;
        T s0 = 0, s1 = 0;
#pragma unroll
        for (int t = 0; t < PMAX; ++t) {
          if (t < p) {
            const T ph = row[ix[t]];
            s0 = fma(m[0][t], ph, s0);
            s1 = fma(dm[0][t], ph, s1);
          }
        }
        a0 = fma(m[1][k], s0, a0);   // sum My Mx phi
        a1 = fma(m[1][k], s1, a1);   // sum My dMx phi
        a2 = fma(dm[1][k], s0, a2);  // sum dMy Mx phi
      }
      e = fma(m[2][l], a0, e);
      fxs = fma(m[2][l], a1, fxs);
      fys = fma(m[2][l], a2, fys);
      fzs = fma(dm[2][l], a0, fzs);
    }
    const double fx_ = -(double)qi * (double)fxs * rk0, fy_ = -(double)qi * (double)fys * rk1,
                 fz_ = -(double)qi * (double)fzs * rk2;
    fout[3 * i] = fx_; fout[3 * i + 1] = fy_; fout[3 * i + 2] = fz_;
    acc[0] = (double)qi * (double)e;
    acc[1] = fx_; acc[2] = fy_; acc[3] = fz_;
  } else if (i < natms) {
    fout[3 * i] = 0; fout[3 * i + 1] = 0; fout[3 * i + 2] = 0;
  }
  block_reduce_store<4>(acc, blk);
}

// FP32 gather, one warp per atom: lane pr = (j, k) of the p x p (x, y) rows sums its z
// column (x fastest, so groups of p lanes read contiguous grid points).  A warp takes
// GATHER_AB atoms at a time: 3 x GATHER_AB lanes build their splines in parallel, and
// the four per-atom sums are combined by a reduce-scatter that leaves the energy sum in
// lane 0 and the x, y, z force sums in lanes 8, 16, 24.
constexpr int GATHER_AB = 8;  // atoms per warp batch
template <int P>
__global__ void __launch_bounds__(256, 4) k_spme_gather_f32(int natms, const float* __restrict__ q4, SpmeGeom sg,
                                                         const int* __restrict__ gidx, const float* __restrict__ gw,
                                                         const float* __restrict__ phi, float rk0, float rk1,
                                                         float rk2, float* __restrict__ fout, double* blk) {
  __shared__ float sp[8][GATHER_AB][2][3][P];  // per warp and atom: value/derivative, dimension, point
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int K0 = sg.K[0], K1 = sg.K[1], K2 = sg.K[2];
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * GATHER_AB; base < natms;
       base += nwarps * GATHER_AB) {
    if (lane < 3 * GATHER_AB) {
      const int a = lane / 3, d = lane - 3 * a, i = base + a;
      if (i < natms) {
        float m[PMAX], dm[PMAX];
        bspline_vals<float, P>(gw[3 * i + d], P, m, dm);
#pragma unroll
        for (int t = 0; t < P; ++t) { sp[wid][a][0][d][t] = m[t]; sp[wid][a][1][d][t] = dm[t]; }
      }
    }
    __syncwarp();
    const int na = min(GATHER_AB, natms - base);
    for (int a = 0; a < na; ++a) {
      const int i = base + a;
      const float qi = q4[4 * i + 3];
      const int gx = gidx[3 * i], gy = gidx[3 * i + 1], gz = gidx[3 * i + 2];
      float v[4] = {0.f, 0.f, 0.f, 0.f};  // energy, x, y, z sums
      int zo[P];  // z-plane offsets of this atom
#pragma unroll
      for (int l = 0; l < P; ++l) {
        int zz = gz + l; if (zz >= K2) zz -= K2;
        zo[l] = zz * K1 * K0;
      }
#pragma unroll
      for (int pr = lane; pr < P * P; pr += 32) {
        const int j = pr % P, k = pr / P;
        int xx = gx + j; if (xx >= K0) xx -= K0;
        int yy = gy + k; if (yy >= K1) yy -= K1;
        const float mx = sp[wid][a][0][0][j], dmx = sp[wid][a][1][0][j];
        const float my = sp[wid][a][0][1][k], dmy = sp[wid][a][1][1][k];
        const float* col = phi + (yy * K0 + xx);
        // the z column against Mz and dMz (separable: 2 products per grid point), then the
        // column's x/y spline products
        float za = 0.f, zc = 0.f;
#pragma unroll
        for (int l = 0; l < P; ++l) {
          const float pa = col[zo[l]];
          za = fmaf(sp[wid][a][0][2][l], pa, za);
          zc = fmaf(sp[wid][a][1][2][l], pa, zc);
        }
        const float p0 = mx * my;
        v[0] = fmaf(p0, za, v[0]);
        v[1] = fmaf(dmx * my, za, v[1]);
        v[2] = fmaf(mx * dmy, za, v[2]);
        v[3] = fmaf(p0, zc, v[3]);
      }
      // reduce-scatter: level 16 keeps (v0, v1) in the lower half-warp, (v2, v3) in the upper
      const bool up16 = lane & 16, up8 = lane & 8;
      float k0 = up16 ? v[2] : v[0], k1 = up16 ? v[3] : v[1];
      const float s0 = up16 ? v[0] : v[2], s1 = up16 ? v[1] : v[3];
      k0 += __shfl_xor_sync(0xffffffffu, s0, 16);
      k1 += __shfl_xor_sync(0xffffffffu, s1, 16);
      float r = up8 ? k1 : k0;
      r += __shfl_xor_sync(0xffffffffu, up8 ? k0 : k1, 8);
#pragma unroll
      for (int o = 4; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
      if ((lane & 7) == 0) {
        const int comp = lane >> 3;
        if (comp == 0) {
          acc[0] += qi * r;
        } else {
          const float f = -qi * r * (comp == 1 ? rk0 : (comp == 2 ? rk1 : rk2));
          fout[3 * i + comp - 1] = f;
          acc[comp] += f;
        }
      }
    }
    __syncwarp();  // the batch's splines are read before the next batch writes them
  }
  block_reduce_store<4>(acc, blk);
}

// a * b as an unnormalised compensated pair: the exact product's high part and, in the
// correction, its rounding error and the cross terms
__device__ __forceinline__ dacc dacc_prod(df x, df y) {
  const df p = two_prod(x.hi, y.hi);
  dacc r;
  r.s = p.hi;
  r.c = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo));
  return r;
}

// a + b of two compensated pairs
__device__ __forceinline__ dacc dacc_sum(dacc a, dacc b) {
  const df u = two_sum(a.s, b.s);
  dacc r;
  r.s = u.hi;
  r.c = __fadd_rn(__fadd_rn(a.c, b.c), u.lo);
  return r;
}

__device__ __forceinline__ dacc shfl_xor_dacc(dacc v, int o) {
  dacc r;
  r.s = __shfl_xor_sync(0xffffffffu, v.s, o);
  r.c = __shfl_xor_sync(0xffffffffu, v.c, o);
  return r;
}

__device__ __forceinline__ df ld_df(const dfr* p) {
  const float2 v = *reinterpret_cast<const float2*>(p);
  return df_make(v.x, v.y);
}

// FP64 form, the same warp-per-atom layout in double-float.  The splines come from the
// preparation kernel (values and derivatives in the gather's truncation convention, the z
// ones times the charge, component-major); a warp copies those of 8 atoms at a time into
// shared memory (64 contiguous bytes per component) and gathers the atoms one after
// another.  Lane (j, k) of the p x p
// (x, y) rows sums its z columns against Mz q and dMz q as compensated dot products (each
// exact product's high part enters a two-sum, its error and cross terms the correction;
// 2 products per grid point, the z-plane offsets computed once per atom).  For p = 8 a
// lane holds the columns (j, k) and (j, k + 4), which it contracts with My and dMy, then
// with Mx and dMx; otherwise each column is weighted with its x/y spline products.  The
// four per-atom sums (energy, x, y, z) stay unnormalised compensated pairs through a
// reduce-scatter over the warp (two values after the first butterfly level, one after
// the second) that leaves them in lanes 0, 8, 16, 24.  No FP64 instruction: forces leave
// as double-floats.
template <int P>
__global__ void __launch_bounds__(256, 6) k_spme_gather_wdf(int natms, SpmeGeom sg, const int* __restrict__ gidx,
                                                         const dfr* __restrict__ gsp,
                                                         const float2* __restrict__ gq, const dfr* __restrict__ phi,
                                                         float2 rk0, float2 rk1, float2 rk2,
                                                         float2* __restrict__ fout, double* blk) {
  constexpr int NS = 6 * P;  // spline components per atom: [value, derivative][x, y, z][point]
  static_assert(GATHER_AB == 8, "8 atoms per batch");
  __shared__ __align__(16) dfr sp[8][NS][GATHER_AB];  // per warp: component, atom
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int K0 = sg.K[0], K1 = sg.K[1], K2 = sg.K[2];
  const int K01 = K0 * K1;
  dacc acc[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) { acc[c].s = 0.f; acc[c].c = 0.f; }
  for (int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * GATHER_AB; base < natms;
       base += nwarps * GATHER_AB) {
    const int na = min(GATHER_AB, natms - base);
#pragma unroll
    for (int e = lane; e < NS * GATHER_AB; e += 32) {
      const int c = e >> 3, a = e & 7;
      if (a < na)
        reinterpret_cast<float2*>(&sp[wid][c][a])[0] =
            reinterpret_cast<const float2*>(gsp + (size_t)c * natms + base + a)[0];
    }
    __syncwarp();
    for (int a = 0; a < na; ++a) {
      const int i = base + a;
      if (gq[i].x == 0.f) {  // uniform over the warp
        if (lane < 3) fout[3 * i + lane] = make_float2(0.f, 0.f);
        continue;
      }
      const int gx = gidx[3 * i], gy = gidx[3 * i + 1], gz = gidx[3 * i + 2];
      // spline component (value or derivative, dimension, point) of this atom
      auto spv = [&](int part, int d, int t) { return ld_df(&sp[wid][(part * 3 + d) * P + t][a]); };
      int zo[P];
#pragma unroll
      for (int l = 0; l < P; ++l) {
        int zz = gz + l;
        if (zz >= K2) zz -= K2;
        zo[l] = zz * K01;
      }
      dacc v[4];  // energy, x, y, z sums of this lane
      if constexpr (P == 8) {
        const int j = lane & 7, k = lane >> 3;
        int xx = gx + j; if (xx >= K0) xx -= K0;
        int y0 = gy + k; if (y0 >= K1) y0 -= K1;
        int y1 = gy + k + 4; if (y1 >= K1) y1 -= K1;
        const dfr* c0 = phi + (y0 * K0 + xx);
        const dfr* c1 = phi + (y1 * K0 + xx);
        dacc a0, b0, a1, b1;
        a0.s = a0.c = b0.s = b0.c = a1.s = a1.c = b1.s = b1.c = 0.f;
#pragma unroll
        for (int l = 0; l < P; ++l) {
          const df mz = spv(0, 2, l), dmz = spv(1, 2, l);
          const df p0 = ld_df(c0 + zo[l]), p1 = ld_df(c1 + zo[l]);
          dacc_add_prod(a0, mz, p0);
          dacc_add_prod(b0, dmz, p0);
          dacc_add_prod(a1, mz, p1);
          dacc_add_prod(b1, dmz, p1);
        }
        // y: My and dMy against the two columns' sums
        const df my0 = spv(0, 1, k), dmy0 = spv(1, 1, k);
        const df my1 = spv(0, 1, k + 4), dmy1 = spv(1, 1, k + 4);
        const df ca0 = df_make(a0.s, a0.c), cc0 = df_make(b0.s, b0.c);
        const df ca1 = df_make(a1.s, a1.c), cc1 = df_make(b1.s, b1.c);
        dacc A = dacc_prod(my0, ca0), B = dacc_prod(dmy0, ca0), C = dacc_prod(my0, cc0);
        dacc_add_prod(A, my1, ca1);
        dacc_add_prod(B, dmy1, ca1);
        dacc_add_prod(C, my1, cc1);
        // x: Mx and dMx
        const df mx = spv(0, 0, j), dmx = spv(1, 0, j);
        const df Ad = df_make(A.s, A.c);
        v[0] = dacc_prod(mx, Ad);
        v[1] = dacc_prod(dmx, Ad);
        v[2] = dacc_prod(mx, df_make(B.s, B.c));
        v[3] = dacc_prod(mx, df_make(C.s, C.c));
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) { v[c].s = 0.f; v[c].c = 0.f; }
#pragma unroll
        for (int pr = lane; pr < P * P; pr += 32) {
          const int j = pr % P, k = pr / P;
          int xx = gx + j; if (xx >= K0) xx -= K0;
          int yy = gy + k; if (yy >= K1) yy -= K1;
          const dfr* col = phi + (yy * K0 + xx);
          dacc za, zc;
          za.s = za.c = zc.s = zc.c = 0.f;
#pragma unroll
          for (int l = 0; l < P; ++l) {
            const df ph = ld_df(col + zo[l]);
            dacc_add_prod(za, spv(0, 2, l), ph);
            dacc_add_prod(zc, spv(1, 2, l), ph);
          }
          const df ca = df_make(za.s, za.c), cc = df_make(zc.s, zc.c);
          const df mx = spv(0, 0, j), dmx = spv(1, 0, j);
          const df my = spv(0, 1, k), dmy = spv(1, 1, k);
          const df w0 = df_mul(mx, my);
          dacc_add_prod(v[0], w0, ca);
          dacc_add_prod(v[1], df_mul(dmx, my), ca);
          dacc_add_prod(v[2], df_mul(mx, dmy), ca);
          dacc_add_prod(v[3], w0, cc);
        }
      }
      // reduce-scatter: level 16 keeps (v0, v1) in the lower half-warp, (v2, v3) in the upper
      const bool up16 = lane & 16, up8 = lane & 8;
      dacc k0 = up16 ? v[2] : v[0], k1 = up16 ? v[3] : v[1];
      const dacc s0 = up16 ? v[0] : v[2], s1 = up16 ? v[1] : v[3];
      k0 = dacc_sum(k0, shfl_xor_dacc(s0, 16));
      k1 = dacc_sum(k1, shfl_xor_dacc(s1, 16));
      dacc r = up8 ? k1 : k0;
      r = dacc_sum(r, shfl_xor_dacc(up8 ? k0 : k1, 8));
#pragma unroll
      for (int o = 4; o > 0; o >>= 1) r = dacc_sum(r, shfl_xor_dacc(r, o));
      // lane 0: energy; lanes 8, 16, 24: x, y, z (the charge is in the z splines)
      if ((lane & 7) == 0) {
        const int comp = lane >> 3;
        const df qr = two_sum(r.s, r.c);
        if (comp == 0) {
          dacc_add(acc[0], qr);
        } else {
          const float2 rk = comp == 1 ? rk0 : (comp == 2 ? rk1 : rk2);
          const df f = df_neg(df_mul(qr, df_make(rk.x, rk.y)));
          fout[3 * i + comp - 1] = make_float2(f.hi, f.lo);
          dacc_add(acc[comp], f);
        }
      }
    }
    __syncwarp();  // the batch's splines are read before the next batch writes them
  }
  dfr out[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) out[c] = to_dfr(two_sum(acc[c].s, acc[c].c));
  block_reduce_store<4>(out, blk);
}

// FP64 form with the double-float gather: forces += (F - Fnet/N) * 2 * scale
__global__ void k_spme_apply_df(int natms, const float2* __restrict__ f, const double* __restrict__ sums,
                                double scale2, double rn, double* fx, double* fy, double* fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natms) return;
  const double m0 = sums[1] * rn, m1 = sums[2] * rn, m2 = sums[3] * rn;
  const float2 a = f[3 * i], b = f[3 * i + 1], c = f[3 * i + 2];
  fx[i] += (((double)a.x + (double)a.y) - m0) * scale2;
  fy[i] += (((double)b.x + (double)b.y) - m1) * scale2;
  fz[i] += (((double)c.x + (double)c.y) - m2) * scale2;
}

// mixed form: forces += (F - Fnet/N) * 2 * scale as 2^40 fixed point (FP32 math)
__global__ void k_spme_apply_fix_f32(int natms, const float* __restrict__ f, const double* __restrict__ sums,
                                     float scale2, float rn, unsigned long long* fixp, float* rec) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natms) return;
  // the three net-force means are read as FP64 and converted once per thread
  const float m0 = (float)sums[1] * rn, m1 = (float)sums[2] * rn, m2 = (float)sums[3] * rn;
  const float v0 = (f[3 * i] - m0) * scale2, v1 = (f[3 * i + 1] - m1) * scale2, v2 = (f[3 * i + 2] - m2) * scale2;
  if (fixp) {
    atomicAdd(&fixp[3 * i + 0], (unsigned long long)fix40(v0));
    atomicAdd(&fixp[3 * i + 1], (unsigned long long)fix40(v1));
    atomicAdd(&fixp[3 * i + 2], (unsigned long long)fix40(v2));
  }
  if (rec) { rec[3 * i] = v0; rec[3 * i + 1] = v1; rec[3 * i + 2] = v2; }  // learned-MTS per-atom forces
}

// forces += (F - Fnet/N) * 2 * scale
__global__ void k_spme_apply(int natms, const double* __restrict__ f, const double* __restrict__ sums, double scale2,
                             double rn, double* fx, double* fy, double* fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natms) return;
  const double m0 = sums[1] * rn, m1 = sums[2] * rn, m2 = sums[3] * rn;
  fx[i] += (f[3 * i] - m0) * scale2;
  fy[i] += (f[3 * i + 1] - m1) * scale2;
  fz[i] += (f[3 * i + 2] - m2) * scale2;
}

__global__ void k_spme_apply_fix(int natms, const double* __restrict__ f, const double* __restrict__ sums,
                                 double scale2, double rn, unsigned long long* fixp, float* rec) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natms) return;
  const double s = 1099511627776.0;
  for (int d = 0; d < 3; ++d) {
    double v = (f[3 * i + d] - sums[1 + d] * rn) * scale2;
    if (fixp) atomicAdd(&fixp[3 * i + d], (unsigned long long)__double2ll_rn(v * s));
    if (rec) rec[3 * i + d] = (float)v;
  }
}

template <typename T>
__global__ void k_cvt(const double* a, T* b, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (T)a[i];
}

inline int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

FftPlan make_plan(int N) {
  FftPlan pl{};
  pl.N = N;
  int m = N;
  while (m % 4 == 0) { pl.rad[pl.nrad++] = 4; m /= 4; }
  while (m % 3 == 0) { pl.rad[pl.nrad++] = 3; m /= 3; }
  while (m % 5 == 0) { pl.rad[pl.nrad++] = 5; m /= 5; }
  while (m % 2 == 0) { pl.rad[pl.nrad++] = 2; m /= 2; }
  if (m != 1) throw (int)GB_ERR_ARG;  // only 2^a 3^b 5^c lengths (parallel_fft.F90:2031)
  return pl;
}

// One SPME grid: geometry, per-atom spline data, bricks, grids, influence
// function and twiddles.  The force path owns the main grid (the CONTROL
// kmax and spline order); the learned multiple-time-step form adds a coarse
// FP32 grid whose increments carry the long-range change of the reciprocal
// force between full steps.
struct SpmeGrid {
  bool ready = false;
  bool fp64 = true;  // FP64 grid buffers allocated (main grid only)
  int K[3] = {0, 0, 0}, B[3] = {0, 0, 0}, nb[3] = {0, 0, 0}, nbricks = 0, p = 0;
  FftPlan plan[3];
  SpmeGeom sg;
  double* spl = nullptr;       // natms * 3 * p splines (floor convention; FP32 view in the mixed form)
  int* nidx = nullptr;         // natms * 3 grid indices
  int *brick_of = nullptr, *brick_count = nullptr, *brick_start = nullptr, *brick_fill = nullptr,
      *brick_atoms = nullptr;
  double* Q = nullptr;
  double2* G = nullptr;
  float* Qf = nullptr;
  float2* Gf = nullptr;
  double *theta = nullptr, *psi = nullptr;
  float *theta_f = nullptr, *psi_f = nullptr;
  double2* tw[3] = {nullptr, nullptr, nullptr};
  float2* twf[3] = {nullptr, nullptr, nullptr};
  FftPlan planh;                 // x pass: half-length complex transform of the packed real rows
  double2* twh = nullptr;        // its twiddles e^{+2 pi i t/(K1/2)}
  float2* twhf = nullptr;
  int Kx = 0;                    // K1/2 + 1 complex columns of the half spectrum
  double* fspme = nullptr;     // 3*natms reciprocal forces (before scale, net removal)
  void* spread_ext = nullptr;  // per-brick spread tiles (nbricks x (B+p-1)^3)
  int* gidx = nullptr;         // warp gather: first grid index per dimension (truncation convention)
  float* gw = nullptr;         // warp gather: fractional coordinate per dimension (3n), then (at 6n) the
                               // double-float charges (2n)
  double* gsp = nullptr;       // double-float gather (main grid): natms x 6p splines (dfr)
  float* fout_f = nullptr;     // warp gather: unscaled reciprocal forces
  // double-float copies for the FP64 form (main grid): influence function, stress
  // factor and twiddles; the grids themselves reuse the FP64 buffers (same sizes)
  dfr *theta_d = nullptr, *psi_d = nullptr;
  dfc* tw_d[3] = {nullptr, nullptr, nullptr};
  dfc* twh_d = nullptr;
};

SpmeGrid S_main, S_coarse;
// FP32 grids: the tile spread (no atomics, atoms in index order per brick) unless
// GB_SPREAD_FIX=1 selects the int64 fixed-point spread with shared-memory atomics
bool g_spread_fix = false;

// Brick edge: a divisor of K of at least p-1 (a brick's atoms reach at most the
// next brick).  Larger bricks cut the halo overlap (B+p-1)^3 / B^3 of the tiles
// the fixed-order reduction reads back, so prefer one of at least bpref (BPREF for
// the force grid; the coarse grid of the multiple-time-step form, with 8x fewer
// points, prefers BPREF_COARSE so that its bricks hold as few atoms and are as many).
constexpr int BPREF = 12, BPREF_COARSE = 8;
int choose_brick(int K, int p, int bpref) {
  for (int B = std::max(p - 1, bpref); B <= BMAX; ++B)
    if (K % B == 0) return B;
  for (int B = p - 1; B <= BMAX; ++B)
    if (K % B == 0) return B;
  return -1;
}

size_t fft_smem(int N, int lines, size_t esz) { return (size_t)2 * lines * N * esz; }

}  // namespace

namespace gbspme {
// the all-FP64 form keeps the runtime-plan transform at every length
template <>
FftKernels<double, double2> fft_kernels<double, double2>(int M, int K2, int K3) {
  return fft_pick<double, double2>(FftLens<>(), FftLens<>(), M, K2, K3);
}
}  // namespace gbspme

extern void invert_host(const double* a, double* b, double* d);
extern void dcell_host(const double* aaa, double* bbb);

// ====================================================================== host
namespace {

// raise a kernel's dynamic shared-memory limit, never lowering a larger
// setting made for the other grid
template <typename K>
void raise_smem(K kernel, int bytes) {
  cudaFuncAttributes a;
  GB_CUDA(cudaFuncGetAttributes(&a, kernel));
  if (a.maxDynamicSharedSizeBytes < bytes)
    GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

// threads per FFT block: enough for one butterfly of the smallest radix per
// thread over the block's lines (at most 256), in whole warps
int fft_threads(const FftPlan& pl, int nlines) {
  int rmin = 5;
  for (int s = 0; s < pl.nrad; ++s) rmin = std::min(rmin, pl.rad[s]);
  const int need = nlines * pl.N / std::max(rmin, 1);
  return std::min(256, std::max(32, (need + 31) / 32 * 32));
}

void grid_free(SpmeGrid& S) {
  void* ptrs[] = {S.spl, S.nidx, S.brick_of, S.brick_count, S.brick_start, S.brick_fill, S.brick_atoms, S.Q, S.G,
                  S.Qf, S.Gf, S.theta, S.psi, S.theta_f, S.psi_f, S.tw[0], S.tw[1], S.tw[2], S.twf[0], S.twf[1],
                  S.twf[2], S.twh, S.twhf, S.fspme, S.spread_ext, S.gidx, S.gw, S.gsp, S.fout_f, S.theta_d, S.psi_d,
                  S.tw_d[0], S.tw_d[1], S.tw_d[2], S.twh_d};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  S = SpmeGrid();
}

// grid of K[0..2] points and spline order p; fp64 = also the FP64 buffers
// dynamic shared-memory limit of the FFT kernels this grid launches
template <typename T, typename T2>
void raise_fft(const SpmeGrid& S, int smem) {
  const FftKernels<T, T2> k = fft_kernels<T, T2>(S.planh.N, S.K[1], S.K[2]);
  raise_smem(k.x_fwd, smem);
  raise_smem(k.x_inv, smem);
  raise_smem(k.y_fwd, smem);
  raise_smem(k.y_inv, smem);
  raise_smem(k.z_conv, smem);
}

void grid_setup(SpmeGrid& S, const int* Kin, int p, bool fp64, int bpref) {
  grid_free(S);
  if (p > PMAX || p < 3) throw (int)GB_ERR_ARG;
  for (int d = 0; d < 3; ++d) S.K[d] = Kin[d];
  if (S.K[0] % 2) throw (int)GB_ERR_ARG;  // real-to-complex x pass on packed pairs
  S.p = p;
  S.fp64 = fp64;
  for (int d = 0; d < 3; ++d) S.plan[d] = make_plan(S.K[d]);
  S.planh = make_plan(S.K[0] / 2);
  S.Kx = S.K[0] / 2 + 1;
  for (int d = 0; d < 3; ++d) {
    S.B[d] = choose_brick(S.K[d], p, bpref);
    if (S.B[d] < 0) {
      // fall back to the whole dimension as one brick if it is small enough
      if (S.K[d] <= BMAX) S.B[d] = S.K[d];
      else throw (int)GB_ERR_ARG;
    }
    S.nb[d] = S.K[d] / S.B[d];
  }
  S.nbricks = S.nb[0] * S.nb[1] * S.nb[2];
  double det;
  invert_host(g.cell, S.sg.rc, &det);
  for (int k = 0; k < 9; ++k) df_split(S.sg.rc[k], &S.sg.rch[k], &S.sg.rcl[k]);
  for (int d = 0; d < 3; ++d) {
    S.sg.K[d] = S.K[d];
    S.sg.Kr[d] = (double)S.K[d];
    S.sg.B[d] = S.B[d];
    S.sg.nb[d] = S.nb[d];
  }
  S.sg.p = p;
  const size_t NG = (size_t)S.K[0] * S.K[1] * S.K[2];
  if (NG > (size_t)INT_MAX) throw (int)GB_ERR_ARG;  // the gathers index grid points with int offsets
  const size_t n = (size_t)g.natms;
  GB_CUDA(cudaMalloc(&S.spl, sizeof(double) * n * 3 * p));
  GB_CUDA(cudaMalloc(&S.nidx, sizeof(int) * 3 * n));
  GB_CUDA(cudaMalloc(&S.brick_of, sizeof(int) * n));
  GB_CUDA(cudaMalloc(&S.brick_count, sizeof(int) * (S.nbricks + 2)));
  GB_CUDA(cudaMalloc(&S.brick_start, sizeof(int) * (S.nbricks + 2)));
  GB_CUDA(cudaMalloc(&S.brick_fill, sizeof(int) * (S.nbricks + 2)));
  GB_CUDA(cudaMalloc(&S.brick_atoms, sizeof(int) * n));
  GB_CUDA(cudaMalloc(&S.theta, sizeof(double) * NG));
  GB_CUDA(cudaMalloc(&S.psi, sizeof(double) * NG));
  if (fp64) {
    GB_CUDA(cudaMalloc(&S.Q, sizeof(double) * NG));
    GB_CUDA(cudaMalloc(&S.G, sizeof(double2) * NG));
  }
  GB_CUDA(cudaMalloc(&S.fspme, sizeof(double) * 3 * n));
  GB_CUDA(cudaMalloc(&S.gidx, sizeof(int) * 3 * n));
  GB_CUDA(cudaMalloc(&S.gw, sizeof(float) * 8 * n));
  if (fp64) GB_CUDA(cudaMalloc(&S.gsp, sizeof(double) * n * 6 * p));
  GB_CUDA(cudaMalloc(&S.fout_f, sizeof(float) * 3 * n));
  {
    const size_t tsize = (size_t)(S.B[0] + p - 1) * (S.B[1] + p - 1) * (S.B[2] + p - 1);
    GB_CUDA(cudaMalloc(&S.spread_ext, sizeof(double) * tsize * S.nbricks));
    raise_smem(k_spme_spread_tile<double, 8>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(double)));
    raise_smem(k_spme_spread_tile<double, 0>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(double)));
    raise_smem(k_spme_spread_tile<dfr, 8>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(dfr)));
    raise_smem(k_spme_spread_tile<dfr, 0>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(dfr)));
    raise_smem(k_spme_spread_tile<float, 8, 256>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(float)));
    raise_smem(k_spme_spread_tile<float, 6>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(float)));
    raise_smem(k_spme_spread_tile<double, 6>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(double)));
    raise_smem(k_spme_spread_tile<dfr, 6>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(dfr)));
    raise_smem(k_spme_spread_tile<float, 0>, (int)spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(float)));
    raise_smem(k_spme_spread_fix<8>, (int)(tsize * sizeof(long long)));
    raise_smem(k_spme_spread_fix<6>, (int)(tsize * sizeof(long long)));
    raise_smem(k_spme_spread_fix<0>, (int)(tsize * sizeof(long long)));
  }
  // |b(m)|^2 (bspline_coeffs_gen, bspline.F90:73-190) on the host in FP64
  std::vector<double> norm2[3];
  {
    std::vector<double> cs(p + 1, 0.0);
    cs[2] = 1.0;
    for (int k = 3; k <= p; ++k)
      for (int j = k; j >= 2; --j) cs[j] = ((double)(j - 1) * cs[j] + (double)(k - j + 1) * cs[j - 1]) * (1.0 / (double)(k - 1));
    const double twopi = 2.0 * 3.14159265358979323846264338327950288;
    for (int d = 0; d < 3; ++d) {
      int K = S.K[d];
      std::vector<double> wr(K), wi(K);
      wr[0] = 1.0; wi[0] = 0.0;
      for (int i = 1; i <= K / 2; ++i) {
        double arg = (twopi / (double)K) * (double)i;
        wr[i] = std::cos(arg); wi[i] = std::sin(arg);
        wr[K - i] = wr[i]; wi[K - i] = -wi[i];
      }
      norm2[d].resize(K);
      for (int i = 0; i < K; ++i) {
        double tr = 0, ti = 0;
        for (int k = 0; k <= p - 2; ++k) {
          int id = (int)(((long)i * k) % K);
          tr += cs[k + 2] * wr[id]; ti += cs[k + 2] * wi[id];
        }
        int id = (int)(((long)i * (p - 1)) % K);
        double nr = wr[id], ni = wi[id];
        double den = tr * tr + ti * ti;
        double cr = (nr * tr + ni * ti) / den, ci = (ni * tr - nr * ti) / den;
        norm2[d][i] = cr * cr + ci * ci;
      }
    }
  }
  // influence function theta and stress factor psi (ewald_spole.F90:1306-1374)
  {
    const double pi = 3.14159265358979323846264338327950288, sqrpi = std::sqrt(pi);
    double rc[9];
    invert_host(g.cell, rc, &det);
    double rcp[10];
    dcell_host(rc, rcp);
    double recip_conv_fac = pi / g.p.alpha;
    double test_fac = (1.0e-6 / recip_conv_fac) * (1.0e-6 / recip_conv_fac);
    double cut = 0.5 * 1.05 * std::min((double)S.K[0] * rcp[6], std::min((double)S.K[1] * rcp[7], (double)S.K[2] * rcp[8]));
    double cut2 = cut * cut;
    std::vector<double> th(NG), ps(NG);
    const int K1 = S.K[0], K2 = S.K[1], K3 = S.K[2];
    for (int l = 0; l < K3; ++l) {
      int ll = l; if (2 * ll > K3) ll -= K3;
      for (int k = 0; k < K2; ++k) {
        int kk = k; if (2 * kk > K2) kk -= K2;
        for (int j = 0; j < S.Kx; ++j) {  // the half spectrum: m_x = 0..K1/2
          int jj = j; if (2 * jj > K1) jj -= K1;
          double r0 = (double)ll * rc[2] + (double)kk * rc[1] + (double)jj * rc[0];
          double r1 = (double)ll * rc[5] + (double)kk * rc[4] + (double)jj * rc[3];
          double r2 = (double)ll * rc[8] + (double)kk * rc[7] + (double)jj * rc[6];
          double k2 = r0 * r0 + r1 * r1 + r2 * r2;
          size_t gi = ((size_t)k * S.Kx + j) * K3 + l;  // z-contiguous per (x,y) line for the z pass
          if (k2 <= cut2 && k2 > test_fac) {
            double bb = norm2[2][l] * norm2[1][k] * norm2[0][j];
            double f = std::sqrt(k2) * recip_conv_fac;
            th[gi] = bb * std::exp(-(f * f)) / (sqrpi * f * f);
            ps[gi] = th[gi] * (-2.0 * ((1.0 + f * f) / k2));
          } else {
            th[gi] = 0.0; ps[gi] = 0.0;
          }
        }
      }
    }
    GB_CUDA(cudaMemcpy(S.theta, th.data(), sizeof(double) * NG, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(S.psi, ps.data(), sizeof(double) * NG, cudaMemcpyHostToDevice));
  }
  // twiddles e^{+2 pi i t / K}
  auto mk_tw = [&S](int K, double2** dd, float2** df, dfc** dc) {
    std::vector<double2> t(K);
    std::vector<float2> tf(K);
    std::vector<dfc> tc(K);
    const double twopi = 2.0 * 3.14159265358979323846264338327950288;
    for (int i = 0; i < K; ++i) {
      double a = twopi * (double)i / (double)K;
      t[i] = make_double2(std::cos(a), std::sin(a));
      tf[i] = make_float2((float)t[i].x, (float)t[i].y);
      tc[i].x = dfr(t[i].x);
      tc[i].y = dfr(t[i].y);
    }
    GB_CUDA(cudaMalloc(dd, sizeof(double2) * K));
    GB_CUDA(cudaMalloc(df, sizeof(float2) * K));
    GB_CUDA(cudaMemcpy(*dd, t.data(), sizeof(double2) * K, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(*df, tf.data(), sizeof(float2) * K, cudaMemcpyHostToDevice));
    if (S.fp64) {
      GB_CUDA(cudaMalloc(dc, sizeof(dfc) * K));
      GB_CUDA(cudaMemcpy(*dc, tc.data(), sizeof(dfc) * K, cudaMemcpyHostToDevice));
    }
  };
  for (int d = 0; d < 3; ++d) mk_tw(S.K[d], &S.tw[d], &S.twf[d], &S.tw_d[d]);
  mk_tw(S.K[0] / 2, &S.twh, &S.twhf, &S.twh_d);
  // FP32 copies for the mixed form
  GB_CUDA(cudaMalloc(&S.Qf, sizeof(float) * NG));
  GB_CUDA(cudaMalloc(&S.Gf, sizeof(float2) * NG));
  GB_CUDA(cudaMalloc(&S.theta_f, sizeof(float) * NG));
  GB_CUDA(cudaMalloc(&S.psi_f, sizeof(float) * NG));
  k_cvt<float><<<nblocks((long long)NG, 256), 256, 0, g.stream>>>(S.theta, S.theta_f, NG);
  GB_LAUNCHED();
  k_cvt<float><<<nblocks((long long)NG, 256), 256, 0, g.stream>>>(S.psi, S.psi_f, NG);
  GB_LAUNCHED();
  if (S.fp64) {  // double-float copies for the FP64 form
    GB_CUDA(cudaMalloc(&S.theta_d, sizeof(dfr) * NG));
    GB_CUDA(cudaMalloc(&S.psi_d, sizeof(dfr) * NG));
    k_cvt<dfr><<<nblocks((long long)NG, 256), 256, 0, g.stream>>>(S.theta, S.theta_d, NG);
    GB_LAUNCHED();
    k_cvt<dfr><<<nblocks((long long)NG, 256), 256, 0, g.stream>>>(S.psi, S.psi_d, NG);
    GB_LAUNCHED();
  }
  // dynamic shared memory limits
  const int maxN = std::max(S.K[0], std::max(S.K[1], S.K[2]));
  int smem = (int)std::max(fft_smem(maxN, TX, sizeof(double2)), fft_smem(S.K[0], 8, sizeof(double2)));
  smem = std::max(smem, 48 * 1024);
  raise_fft<double, double2>(S, smem);
  raise_fft<float, float2>(S, smem);
  if (S.fp64) raise_fft<dfr, dfc>(S, smem);
  GB_CUDA(cudaStreamSynchronize(g.stream));
  S.ready = true;
}

// One reciprocal-space evaluation on grid S.  The main grid adds its forces
// into the context's FP64 or fixed-point forces (and, when given, stores the
// applied per-atom forces in rec); the coarse grid only stores them in rec.
template <typename T, typename T2>
void grid_run(SpmeGrid& S, bool coarse, float* rec, double* eng_rc, double* vir_rc, double* stress9) {
  cudaStream_t st = g.stream;
  const int n = g.natms, p = S.p;
  constexpr bool DF = std::is_same<T, dfr>::value;  // FP64 form in double-float
  constexpr bool F64 = std::is_same<T, double>::value || DF;  // FP64-accuracy kernels and buffers
  auto pid = [coarse](int id) {
    if (!coarse) return id;
    if (id == P_SPME_PREP) return (int)P_COARSE_PREP;
    if (id == P_SPME_SPREAD) return (int)P_COARSE_SPREAD;
    if (id == P_SPME_GATHER) return (int)P_COARSE_GATHER;
    return (int)P_COARSE_FFT;
  };
  T* spl = reinterpret_cast<T*>(S.spl);
  T* Q = F64 ? reinterpret_cast<T*>(S.Q) : reinterpret_cast<T*>(S.Qf);
  T2* G = F64 ? reinterpret_cast<T2*>(S.G) : reinterpret_cast<T2*>(S.Gf);
  const T* th = DF ? reinterpret_cast<const T*>(S.theta_d)
                   : (F64 ? reinterpret_cast<const T*>(S.theta) : reinterpret_cast<const T*>(S.theta_f));
  const T* ps = DF ? reinterpret_cast<const T*>(S.psi_d)
                   : (F64 ? reinterpret_cast<const T*>(S.psi) : reinterpret_cast<const T*>(S.psi_f));
  const T2* tw1 = DF ? reinterpret_cast<const T2*>(S.tw_d[0])
                     : (F64 ? reinterpret_cast<const T2*>(S.tw[0]) : reinterpret_cast<const T2*>(S.twf[0]));
  const T2* tw2 = DF ? reinterpret_cast<const T2*>(S.tw_d[1])
                     : (F64 ? reinterpret_cast<const T2*>(S.tw[1]) : reinterpret_cast<const T2*>(S.twf[1]));
  const T2* tw3 = DF ? reinterpret_cast<const T2*>(S.tw_d[2])
                     : (F64 ? reinterpret_cast<const T2*>(S.tw[2]) : reinterpret_cast<const T2*>(S.twf[2]));
  const int K1 = S.K[0], K2 = S.K[1], K3 = S.K[2];
  // splines + brick binning
  GB_CUDA(cudaMemsetAsync(S.brick_count, 0, sizeof(int) * (S.nbricks + 2), st));
  GB_CUDA(cudaMemsetAsync(S.brick_fill, 0, sizeof(int) * (S.nbricks + 2), st));
  prof_begin(pid(P_SPME_PREP));
  const bool warp_gather = (!F64 || DF) && (p == 8 || p == 6);
  auto prep = p == 8 ? k_spme_prep<T, 8> : (p == 6 ? k_spme_prep<T, 6> : k_spme_prep<T, 0>);
  prep<<<nblocks(n, PREP_AT), 3 * PREP_AT, 0, st>>>(n, g.x, g.y, g.z, g.chge, S.sg, spl, S.nidx, S.brick_of, S.brick_count,
                                         warp_gather ? S.gidx : nullptr, warp_gather && !DF ? S.gw : nullptr,
                                         warp_gather && DF ? reinterpret_cast<float2*>(S.gw + 6 * (size_t)n) : nullptr,
                                         warp_gather && DF ? reinterpret_cast<T*>(S.gsp) : nullptr);
  GB_LAUNCHED();

  scan_exclusive(S.brick_count, S.brick_start, S.nbricks + 1);
  // the tile spread adds a brick's atoms in ascending index order (deterministic sums);
  // the fixed-point spread of the mixed form (GB_SPREAD_FIX=1) does not depend on it
  const bool tile_spread = F64 || !g_spread_fix;
  if (tile_spread) {
    int* tmp = gb_scan_scratch(n + 1);
    k_brick_scatter<<<nblocks(n, 256), 256, 0, st>>>(n, S.brick_of, S.brick_start, S.brick_fill, tmp);
    GB_LAUNCHED();
    k_brick_sort<<<nblocks((long long)S.nbricks * 32, 256), 256, 0, st>>>(S.nbricks, S.brick_start, tmp,
                                                                          S.brick_atoms);
    GB_LAUNCHED();
  } else {  // fixed-point sums do not depend on the order of a brick's atoms
    k_brick_scatter<<<nblocks(n, 256), 256, 0, st>>>(n, S.brick_of, S.brick_start, S.brick_fill, S.brick_atoms);
    GB_LAUNCHED();
  }
  prof_end(pid(P_SPME_PREP));
  // spreading: tile scatter per brick, then the fixed-order halo reduction
  {
    T* ext = reinterpret_cast<T*>(S.spread_ext);
    const size_t smem = spread_smem(S.B[0], S.B[1], S.B[2], p, sizeof(T));
    const size_t NG = (size_t)K1 * K2 * K3;
    const int red_nt = std::min(256, (K1 + 31) / 32 * 32);  // halo reduction: x in the block, y and z in the grid
    const dim3 red_grid((unsigned)nblocks(K1, red_nt), (unsigned)K2, (unsigned)K3);
    prof_begin(pid(P_SPME_SPREAD));
    if (tile_spread) {
      // order 8 in FP32: eight warps of two points per lane (every tile point is one FMA, so
      // the per-atom indexing dominates and halves); the double-float and FP64 tiles keep
      // sixteen warps, whose longer update chains need the warps more than the shared indexing
      constexpr bool EIGHT = std::is_same<T, float>::value;
      constexpr int NT8 = EIGHT ? 256 : SPREAD_NT;
      auto spread = p == 8 ? k_spme_spread_tile<T, 8, NT8> : (p == 6 ? k_spme_spread_tile<T, 6> : k_spme_spread_tile<T, 0>);
      spread<<<S.nbricks, p == 8 ? NT8 : SPREAD_NT, smem, st>>>(S.sg, S.brick_start, S.brick_atoms, spl, S.nidx, g.chge,
                                                              ext);
      GB_LAUNCHED();
      k_spme_tile_reduce<T><<<red_grid, red_nt, 0, st>>>(S.sg, ext, Q);
      GB_LAUNCHED();
    } else {
      long long* exti = reinterpret_cast<long long*>(S.spread_ext);
      const size_t tsz = (size_t)(S.B[0] + p - 1) * (S.B[1] + p - 1) * (S.B[2] + p - 1);
      auto kern = p == 8 ? k_spme_spread_fix<8> : (p == 6 ? k_spme_spread_fix<6> : k_spme_spread_fix<0>);
      kern<<<S.nbricks, 256, tsz * sizeof(long long), st>>>(S.sg, S.brick_start, S.brick_atoms,
                                                            reinterpret_cast<const float*>(spl), S.nidx, g.chge, exti);
      GB_LAUNCHED();
      k_spme_tile_reduce_fix<<<red_grid, red_nt, 0, st>>>(S.sg, exti, reinterpret_cast<float*>(Q));
      GB_LAUNCHED();
    }
    prof_end(pid(P_SPME_SPREAD));
  }
  // FFT + convolution: real-to-complex x pass, y and z passes on the Kx = K1/2+1 columns
  const int lines = 8;
  const int rows = K2 * K3;
  const int Kx = S.Kx, M = K1 / 2;
  const T2* twh = DF ? reinterpret_cast<const T2*>(S.twh_d)
                     : (F64 ? reinterpret_cast<const T2*>(S.twh) : reinterpret_cast<const T2*>(S.twhf));
  const int ntx = (Kx + TX - 1) / TX;
  prof_begin(pid(P_FFT_XF));
  const FftKernels<T, T2> fk = fft_kernels<T, T2>(M, K2, K3);
  const int thx = fft_threads(S.planh, lines), thy = fft_threads(S.plan[1], TX), thz = fft_threads(S.plan[2], TX);
  fk.x_fwd<<<nblocks(rows, lines), thx, fft_smem(M, lines, sizeof(T2)), st>>>(Q, G, S.planh, twh, tw1,
                                                                                            rows, lines);
  GB_LAUNCHED();
  prof_end(pid(P_FFT_XF));
  prof_begin(pid(P_FFT_Y));
  fk.y_fwd<<<ntx * K3, thy, fft_smem(K2, TX, sizeof(T2)), st>>>(G, Kx, K2, S.plan[1], tw2);
  GB_LAUNCHED();
  prof_end(pid(P_FFT_Y));
  const int nbz = ntx * K2;
  double* blkz = gb_blkacc(nbz * 6 + nblocks((long long)n * 32, 128) * 4);
  prof_begin(pid(P_FFT_Z));
  fk.z_conv<<<nbz, thz, fft_smem(K3, TX, sizeof(T2)) + K3 * sizeof(T), st>>>(G, K1, K2, K3, S.plan[2], tw3,
                                                                                       th, ps, S.sg, blkz);
  GB_LAUNCHED();
  prof_end(pid(P_FFT_Z));
  prof_begin(pid(P_FFT_Y));
  fk.y_inv<<<ntx * K3, thy, fft_smem(K2, TX, sizeof(T2)), st>>>(G, Kx, K2, S.plan[1], tw2);
  GB_LAUNCHED();
  prof_end(pid(P_FFT_Y));
  prof_begin(pid(P_FFT_XI));
  fk.x_inv<<<nblocks(rows, lines), thx, fft_smem(M, lines, sizeof(T2)), st>>>(G, Q, S.planh, twh, tw1,
                                                                                            rows, lines);
  GB_LAUNCHED();
  prof_end(pid(P_FFT_XI));
  // gather
  double rc[9];
  for (int k = 0; k < 9; ++k) rc[k] = S.sg.rc[k];
  double rk[3];
  for (int a = 0; a < 3; ++a) rk[a] = rc[a] * S.sg.Kr[0] + rc[a + 3] * S.sg.Kr[1] + rc[a + 6] * S.sg.Kr[2];
  static int occ_g = 0;
  if (!occ_g) GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_g, k_spme_gather_f32<8>, 256, 0));
  static int occ_gd = 0;
  if (DF && !occ_gd) GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_gd, k_spme_gather_wdf<8>, 256, 0));
  const int nbg = warp_gather ? std::max(1, std::min((DF ? occ_gd : occ_g) * g.nsm,
                                                     nblocks((long long)n * 32 / GATHER_AB, 256)))
                              : nblocks(n, 128);
  double* blkg = blkz + (size_t)nbz * 6;
  prof_begin(pid(P_SPME_GATHER));
  if (warp_gather && DF) {
    auto kern = p == 8 ? k_spme_gather_wdf<8> : k_spme_gather_wdf<6>;
    float2 rkd[3];
    for (int a = 0; a < 3; ++a) df_split(rk[a], &rkd[a].x, &rkd[a].y);
    kern<<<nbg, 256, 0, st>>>(n, S.sg, S.gidx, reinterpret_cast<const dfr*>(S.gsp),
                              reinterpret_cast<const float2*>(S.gw + 6 * (size_t)n), reinterpret_cast<const dfr*>(Q),
                              rkd[0], rkd[1], rkd[2], reinterpret_cast<float2*>(S.fspme), blkg);
  } else if (warp_gather) {
    auto kern = p == 8 ? k_spme_gather_f32<8> : k_spme_gather_f32<6>;
    kern<<<nbg, 256, 0, st>>>(n, reinterpret_cast<const float*>(g.xf), S.sg, S.gidx, S.gw,
                              reinterpret_cast<const float*>(Q), (float)rk[0], (float)rk[1], (float)rk[2], S.fout_f,
                              blkg);
  } else {
    auto gather = p == 8 ? k_spme_gather<T, 8> : k_spme_gather<T, 0>;
    gather<<<nbg, 128, 0, st>>>(n, g.x, g.y, g.z, g.chge, S.sg, Q, rk[0], rk[1], rk[2], S.fspme, blkg);
  }
  GB_LAUNCHED();
  prof_end(pid(P_SPME_GATHER));
  gb_reduce_blocks(blkz, nbz, 6, &g.sc->acc[A_SPME_STR]);
  gb_reduce_blocks(blkg, nbg, 4, &g.sc->acc[A_GATHER]);
  const double pi = 3.14159265358979323846264338327950288;
  const double scale = pi * std::sqrt(pi) * std::pow(g.p.alpha, 1 - 3) * (0.5 / g.volm) * g.scaling;
  unsigned long long* fixp = coarse ? nullptr : (unsigned long long*)g.fixp;
  prof_begin(pid(P_SPME_GATHER));
  if (DF && warp_gather) {
    k_spme_apply_df<<<nblocks(n, 256), 256, 0, st>>>(n, reinterpret_cast<const float2*>(S.fspme),
                                                      &g.sc->acc[A_GATHER], 2.0 * scale, 1.0 / (double)n, g.fx, g.fy,
                                                      g.fz);
  } else if (F64) {
    k_spme_apply<<<nblocks(n, 256), 256, 0, st>>>(n, S.fspme, &g.sc->acc[A_GATHER], 2.0 * scale, 1.0 / (double)n,
                                                   g.fx, g.fy, g.fz);
  } else if (warp_gather) {
    k_spme_apply_fix_f32<<<nblocks(n, 256), 256, 0, st>>>(n, S.fout_f, &g.sc->acc[A_GATHER], (float)(2.0 * scale),
                                                           (float)(1.0 / (double)n), fixp, rec);
  } else {
    k_spme_apply_fix<<<nblocks(n, 256), 256, 0, st>>>(n, S.fspme, &g.sc->acc[A_GATHER], 2.0 * scale,
                                                       1.0 / (double)n, fixp, rec);
  }
  GB_LAUNCHED();
  prof_end(pid(P_SPME_GATHER));
  if (g.defer_scalars && !coarse) return;  // the MD loop reads the sums after its last step
  gb_sync_scalars();
  spme_scalars(g.hsc, eng_rc, vir_rc, stress9);
}

}  // namespace

// reciprocal energy (with the self-interaction), virial and stress from the device sums
void spme_scalars(const DevScalars* h, double* eng_rc, double* vir_rc, double* stress9) {
  const double pi = 3.14159265358979323846264338327950288;
  const double scale = pi * std::sqrt(pi) * std::pow(g.p.alpha, 1 - 3) * (0.5 / g.volm) * g.scaling;
  const double* A = h->acc;
  double eng = A[A_GATHER] * scale;
  double s6[6];
  for (int k = 0; k < 6; ++k) s6[k] = A[A_SPME_STR + k] * scale;
  double stt[9] = {s6[0], s6[1], s6[2], s6[1], s6[3], s6[4], s6[2], s6[4], s6[5]};
  *eng_rc = eng + g.self_interaction;
  stt[0] += eng; stt[4] += eng; stt[8] += eng;
  for (int k = 0; k < 9; ++k) stress9[k] += stt[k];
  *vir_rc = -(stt[0] + stt[4] + stt[8]);
}

void spme_setup() {
  const char* e = getenv("GB_SPREAD_FIX");
  g_spread_fix = e && e[0] == '1';
  grid_setup(S_main, g.p.kmax, g.p.nsplines, true, BPREF);
}

void spme_free() {
  grid_free(S_main);
  grid_free(S_coarse);
}

void spme_forces(double* eng_rc, double* vir_rc, double* stress9) {
  float* rec = mts_rec_out();
  if (g.precision == GB_FP64 && g.fp64_native) grid_run<double, double2>(S_main, false, rec, eng_rc, vir_rc, stress9);
  else if (g.precision == GB_FP64) grid_run<dfr, dfc>(S_main, false, rec, eng_rc, vir_rc, stress9);
  else grid_run<float, float2>(S_main, false, rec, eng_rc, vir_rc, stress9);
}

void spme_coarse_setup(const int* K, int p) { grid_setup(S_coarse, K, p, false, BPREF_COARSE); }

bool spme_coarse_ready() { return S_coarse.ready; }

void spme_coarse_forces(double* eng_rc, double* vir_rc, double* stress9, float* rec) {
  if (!S_coarse.ready) throw (int)GB_ERR_NOT_INIT;
  grid_run<float, float2>(S_coarse, true, rec, eng_rc, vir_rc, stress9);
}
