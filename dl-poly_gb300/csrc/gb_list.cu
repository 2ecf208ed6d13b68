// gb_list.cu - halo images and the link-cell Verlet list on the device.
//
// Follows, in serial (one-domain) semantics:
//   pbcshift            source/numerics.F90:1851-1907
//   set_halo_particles  source/halo.F90:153-356 (+ export_atomic_data deport_data.F90:1673-1900)
//   refresh_halo_positions source/halo.F90:47-114
//   link_cell_pairs     source/neighbours.F90:356-1414
// Every quantity that decides membership (cell index, halo flag, rsq <= rcsq)
// is computed with explicitly rounded FP64 operations (no FMA contraction) in
// the reference's operation order, so the pair set is bit-identical to the
// FP64 oracle.  Distance tests run first in FP32 with a proven error margin;
// only candidates inside the margin band are re-tested in exact FP64.
#include <cfloat>
#include <cmath>
#include <cstring>

#include "gb_common.cuh"

namespace {

constexpr int SCAN_BLOCK = 1024;
constexpr int MAX_SBC = 1024;  // semi-ball offsets capacity

__constant__ int c_off[MAX_SBC];   // linear cell offset of each semi-ball cell
__constant__ int c_nix[MAX_SBC], c_niy[MAX_SBC], c_niz[MAX_SBC];
__constant__ unsigned char c_nir[MAX_SBC];
__constant__ unsigned char c_row[MAX_SBC];  // cell-tile row (dy, dz) of each semi-ball cell
// The semi-ball cells in the reference order form, row by row, runs of consecutive cells
// along x (contiguous sorted positions); a segment is such a run with one nir flag.
__constant__ int c_seg_off0[MAX_SBC], c_seg_off1[MAX_SBC];  // linear offsets of its first and last cell
__constant__ unsigned char c_seg_row[MAX_SBC], c_seg_nir[MAX_SBC];

struct HaloGeom {
  double rc[9];
  double ecw[3], cw[3];
};

struct CellGeom {
  double rc[9];
  double xdc, ydc, zdc;
  int nlp, nlx, nly, nlz, NX, NY, NZ;
  double rcsq;
  float rcsq_lo, rcsq_hi;
  double half_plus;
};

HaloGeom h_halo;
CellGeom h_cg;
double h_add[6][3];  // export add vectors for mdir -1,1,-2,2,-3,3

// ---------------------------------------------------------------- kernels
__global__ void k_pbcshift(int n, double* x, double* y, double* z, double a0, double a4, double a8,
                           double c0, double c4, double c8, double half_minus) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xss = mul_rn(a0, x[i]), yss = mul_rn(a4, y[i]), zss = mul_rn(a8, z[i]);
  xss = sub_rn(xss, round(xss)); if (xss >= half_minus) xss = -xss;
  yss = sub_rn(yss, round(yss)); if (yss >= half_minus) yss = -yss;
  zss = sub_rn(zss, round(zss)); if (zss >= half_minus) zss = -zss;
  x[i] = mul_rn(c0, xss);
  y[i] = mul_rn(c4, yss);
  z[i] = mul_rn(c8, zss);
}

__device__ __forceinline__ double red_coord(const double* rc, int d, double x, double y, double z) {
  return add_rn(add_rn(mul_rn(rc[d], x), mul_rn(rc[d + 3], y)), mul_rn(rc[d + 6], z));
}

__global__ void k_halo_flags(int n, const double* x, const double* y, const double* z, HaloGeom hg,
                             int* ixyz, int* src, int* shcode, DevScalars* sc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) { sc->nlast = n; sc->nlast_prev = n; }
  if (i >= n) return;
  double xx = red_coord(hg.rc, 0, x[i], y[i], z[i]);
  double yy = red_coord(hg.rc, 1, x[i], y[i], z[i]);
  double zz = red_coord(hg.rc, 2, x[i], y[i], z[i]);
  int v = 0;
  if (xx <= hg.ecw[0]) v += 1;
  if (xx >= hg.cw[0]) v += 2;
  if (yy <= hg.ecw[1]) v += 10;
  if (yy >= hg.cw[1]) v += 20;
  if (zz <= hg.ecw[2]) v += 100;
  if (zz >= hg.cw[2]) v += 200;
  ixyz[i] = v;
  src[i] = i;
  shcode[i] = 13;
}

__device__ __forceinline__ bool export_sel(int v, int kx, int ky, int kz, int jxyz) {
  if (v <= 0) return false;
  int ix = v % 10;
  int iy = (v - ix) % 100;
  int iz = (v - (ix + iy)) % 1000;
  int j = ix * kx + iy * ky + iz * kz;
  return (j == jxyz) || (j > jxyz && j % 3 == 0);
}

__global__ void k_export_count(const int* ixyz, const DevScalars* sc, int kx, int ky, int kz, int jxyz,
                               int* blkcount) {
  const int n = sc->nlast;
  const int base = blockIdx.x * SCAN_BLOCK;
  int cnt = 0;
  for (int t = threadIdx.x; t < SCAN_BLOCK; t += blockDim.x) {
    int i = base + t;
    if (i < n && export_sel(ixyz[i], kx, ky, kz, jxyz)) ++cnt;
  }
  cnt = warp_sumi(cnt);
  __shared__ int s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s[w];
    blkcount[blockIdx.x] = tot;
  }
}

// Exclusive scan of n ints in a single block (n up to a few million).
__global__ void k_scan_single(const int* in, int* out, int n, int* total) {
  __shared__ int part[1024];
  const int T = blockDim.x;
  const int per = (n + T - 1) / T;
  const int b = threadIdx.x * per;
  int s = 0;
  for (int k = 0; k < per; ++k) if (b + k < n) s += in[b + k];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < T; o <<= 1) {
    int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = part[threadIdx.x] - s;
  for (int k = 0; k < per; ++k)
    if (b + k < n) { out[b + k] = run; run += in[b + k]; }
  if (threadIdx.x == T - 1 && total) *total = part[T - 1];
}

__global__ void k_export_commit(const int* blkcount, int nblk, int* blkoff, DevScalars* sc, int mxatms) {
  // single thread: offsets were produced by k_scan_single into blkoff; grow nlast
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int tot = blkoff[nblk - 1] + blkcount[nblk - 1];
  int n = sc->nlast;
  sc->nlast_prev = n;
  if (n + tot > mxatms) {
    sc->status |= ST_HALO_OVERFLOW;
    tot = mxatms - n;
  }
  sc->nlast = n + tot;
}

__global__ void k_export_write(double* x, double* y, double* z, int* ltg, int* src, int* shcode, int* ixyz,
                               const int* blkoff, const DevScalars* sc, int kx, int ky, int kz, int jxyz,
                               int kxyz, double ax, double ay, double az, int dshift, int mxatms) {
  const int n = sc->nlast_prev;
  const int base = blockIdx.x * SCAN_BLOCK;
  __shared__ int wsum[32];
  __shared__ int chunk_base;
  if (threadIdx.x == 0) chunk_base = 0;
  __syncthreads();
  // process the block's 1024 items in chunks of blockDim, preserving order
  for (int c = 0; c < SCAN_BLOCK; c += blockDim.x) {
    int i = base + c + threadIdx.x;
    int v = (i < n && c + threadIdx.x < SCAN_BLOCK) ? ixyz[i] : 0;
    bool sel = (i < n) && export_sel(v, kx, ky, kz, jxyz);
    unsigned m = __ballot_sync(0xffffffffu, sel);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int pre = __popc(m & ((1u << lane) - 1u));
    if (lane == 0) wsum[w] = __popc(m);
    __syncthreads();
    int wpre = 0;
    for (int k = 0; k < w; ++k) wpre += wsum[k];
    if (sel) {
      int dst = n + blkoff[blockIdx.x] + chunk_base + wpre + pre;
      if (dst < mxatms) {
        x[dst] = add_rn(x[i], ax);
        y[dst] = add_rn(y[i], ay);
        z[dst] = add_rn(z[i], az);
        ltg[dst] = ltg[i];
        src[dst] = src[i];
        shcode[dst] = shcode[i] + dshift;
        int ix = v % 10, iy = (v - ix) % 100, iz = (v - (ix + iy)) % 1000;
        int j = ix * kx + iy * ky + iz * kz;
        ixyz[dst] = v - (j == jxyz ? jxyz : kxyz);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += wsum[k];
      chunk_base += t;
    }
    __syncthreads();
  }
}

// halo properties from the local source atom
__global__ void k_halo_props(int natms, const DevScalars* sc, const int* src, int* ltype, double* chge,
                             double* weight, int* lfrzn) {
  int i = natms + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc->nlast) return;
  int s = src[i];
  ltype[i] = ltype[s];
  chge[i] = chge[s];
  weight[i] = weight[s];
  lfrzn[i] = lfrzn[s];
}

// refresh_halo_positions: the same export chain applied to the source position
__global__ void k_halo_refresh(int natms, const DevScalars* sc, const int* src, const int* shcode, double* x,
                               double* y, double* z, const double* adds /*6x3*/) {
  int i = natms + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc->nlast) return;
  int s = src[i], c = shcode[i];
  int sx = c % 3 - 1, sy = (c / 3) % 3 - 1, sz = c / 9 - 1;
  double xx = x[s], yy = y[s], zz = z[s];
  // adds[0..2] is the -x export (image at +L), adds[3..5] the +x export (image at -L), etc.
  if (sx != 0) { const double* a = adds + 3 * (sx > 0 ? 0 : 1); xx = add_rn(xx, a[0]); yy = add_rn(yy, a[1]); zz = add_rn(zz, a[2]); }
  if (sy != 0) { const double* a = adds + 3 * (sy > 0 ? 2 : 3); xx = add_rn(xx, a[0]); yy = add_rn(yy, a[1]); zz = add_rn(zz, a[2]); }
  if (sz != 0) { const double* a = adds + 3 * (sz > 0 ? 4 : 5); xx = add_rn(xx, a[0]); yy = add_rn(yy, a[1]); zz = add_rn(zz, a[2]); }
  x[i] = xx; y[i] = yy; z[i] = zz;
}

__global__ void k_set_check(int n, const double* x, const double* y, const double* z, double* xb, double* yb,
                            double* zb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  xb[i] = x[i]; yb[i] = y[i]; zb[i] = z[i];
}

// ----------------------------------------------------------------- binning
__global__ void k_bin(int natms, const DevScalars* sc, const double* x, const double* y, const double* z,
                      CellGeom cg, int* which_cell, int* count) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nlast = sc->nlast;
  if (i >= nlast) return;
  const double xx = red_coord(cg.rc, 0, x[i], y[i], z[i]);
  const double yy = red_coord(cg.rc, 1, x[i], y[i], z[i]);
  const double zz = red_coord(cg.rc, 2, x[i], y[i], z[i]);
  const int nlp = cg.nlp, jx0 = nlp, jy0 = nlp, jz0 = nlp;
  const int nlx0e = nlp - 1, nly0e = nlp - 1, nlz0e = nlp - 1;
  const int nlx1s = cg.nlx + nlp, nly1s = cg.nly + nlp, nlz1s = cg.nlz + nlp;
  const int nlx1e = cg.nlx + 2 * nlp - 1, nly1e = cg.nly + 2 * nlp - 1, nlz1e = cg.nlz + 2 * nlp - 1;
  int icell;
  if (i < natms) {
    int ix = __double2int_rz(mul_rn(cg.xdc, add_rn(xx, 0.5))) + jx0;
    int iy = __double2int_rz(mul_rn(cg.ydc, add_rn(yy, 0.5))) + jy0;
    int iz = __double2int_rz(mul_rn(cg.zdc, add_rn(zz, 0.5))) + jz0;
    ix = max(min(ix, nlx1s - 1), nlx0e + 1);
    iy = max(min(iy, nly1s - 1), nly0e + 1);
    iz = max(min(iz, nlz1s - 1), nlz0e + 1);
    icell = 1 + ix + cg.NX * (iy + cg.NY * iz);
  } else {
    double dx, dy, dz;
    int ix, iy, iz;
    if (xx > -cg.half_plus) { dx = mul_rn(cg.xdc, add_rn(xx, 0.5)); ix = __double2int_rz(dx) + jx0; }
    else { dx = mul_rn(cg.xdc, fabs(add_rn(xx, 0.5))); ix = -__double2int_rz(dx) + jx0 - 1; }
    if (yy > -cg.half_plus) { dy = mul_rn(cg.ydc, add_rn(yy, 0.5)); iy = __double2int_rz(dy) + jy0; }
    else { dy = mul_rn(cg.ydc, fabs(add_rn(yy, 0.5))); iy = -__double2int_rz(dy) + jy0 - 1; }
    if (zz > -cg.half_plus) { dz = mul_rn(cg.zdc, add_rn(zz, 0.5)); iz = __double2int_rz(dz) + jz0; }
    else { dz = mul_rn(cg.zdc, fabs(add_rn(zz, 0.5))); iz = -__double2int_rz(dz) + jz0 - 1; }
    if (ix >= 0 && iy >= 0 && iz >= 0) {
      bool lx0 = ix > nlx0e, lx1 = ix < nlx1s, ly0 = iy > nly0e, ly1 = iy < nly1s, lz0 = iz > nlz0e, lz1 = iz < nlz1s;
      if ((lx0 && lx1) && (ly0 && ly1) && (lz0 && lz1)) {
        double x0 = fabs(sub_rn(dx, 0.0)), x1 = fabs(sub_rn(dx, (double)cg.nlx));
        dx = fmin(x0, x1);
        double y0 = fabs(sub_rn(dy, 0.0)), y1 = fabs(sub_rn(dy, (double)cg.nly));
        dy = fmin(y0, y1);
        double z0 = fabs(sub_rn(dz, 0.0)), z1 = fabs(sub_rn(dz, (double)cg.nlz));
        dz = fmin(z0, z1);
        if (dx <= dy && dx <= dz) {
          ix = x0 < x1 ? nlx0e : nlx1s;
          if (fabs(sub_rn(dx, dy)) < DBL_EPSILON) iy = y0 < y1 ? nly0e : nly1s;
          if (fabs(sub_rn(dx, dz)) < DBL_EPSILON) iz = z0 < z1 ? nlz0e : nlz1s;
        } else if (dy <= dx && dy <= dz) {
          iy = y0 < y1 ? nly0e : nly1s;
          if (fabs(sub_rn(dy, dz)) < DBL_EPSILON) iz = z0 < z1 ? nlz0e : nlz1s;
        } else {
          iz = z0 < z1 ? nlz0e : nlz1s;
        }
      }
      bool out = ix < 0 || ix > nlx1e || iy < 0 || iy > nly1e || iz < 0 || iz > nlz1e;
      icell = out ? 0 : 1 + ix + cg.NX * (iy + cg.NY * iz);
    } else {
      icell = 0;
    }
  }
  which_cell[i] = icell;
  atomicAdd(&count[icell], 1);
}

__global__ void k_cell_scatter(const DevScalars* sc, const int* which_cell, const int* start, int* fill,
                               int* tmp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc->nlast) return;
  int c = which_cell[i];
  int slot = atomicAdd(&fill[c], 1);
  tmp[start[c] + slot] = i;
}

// Stable order inside each cell (ascending atom index, as the reference's
// counting sort over i = 1..nlast): rank of each member by counting.
__global__ void k_cell_sort(int ncells_p1, const int* start, const int* tmp, int* at_list, int* sorted_pos,
                            const double* x, const double* y, const double* z, double4_32a* xs, float4* xsf) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= ncells_p1) return;
  int s = start[warp], e = start[warp + 1], n = e - s;
  if (warp == 0) {  // residual halo cell: never a neighbour cell, order irrelevant
    for (int a = lane; a < n; a += 32) {
      int v = tmp[s + a];
      at_list[s + a] = v;
      sorted_pos[v] = s + a;
      xs[s + a] = make_double4_32a(x[v], y[v], z[v], 0.0);
      xsf[s + a] = make_float4((float)x[v], (float)y[v], (float)z[v], 0.0f);
    }
    return;
  }
  for (int a = lane; a < n; a += 32) {
    int v = tmp[s + a];
    int r = 0;
    for (int b = 0; b < n; ++b) r += (tmp[s + b] < v);
    int pos = s + r;
    at_list[pos] = v;
    sorted_pos[v] = pos;
    double xv = x[v], yv = y[v], zv = z[v];
    xs[pos] = make_double4_32a(xv, yv, zv, 0.0);
    xsf[pos] = make_float4((float)xv, (float)yv, (float)zv, 0.0f);
  }
}

// Half-shell Verlet list (neighbours.F90:876-1184): one warp per local atom.
// Entries are appended in the reference order (semi-ball cell by cell, each
// cell's members in ascending order), with ballot-based compaction.
__global__ void __launch_bounds__(256) k_list_pairs(int natms, const DevScalars* sc_c, CellGeom cg, int nsbcll,
                                                    const int* at_list, const int* which_cell, const int* start,
                                                    const double4_32a* xs, const float4* xsf, int* list, int ld,
                                                    int* spos, int ldt, int max_list, DevScalars* sc) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nlast = sc_c->nlast;
  if (warp >= nlast) return;
  const int p = warp;  // sorted position
  const int i = at_list[p];
  if (i >= natms) return;
  const int ic = which_cell[i];
  const int icm = ic - 1;
  const int ix = icm % cg.NX;
  const int iz = icm / (cg.NX * cg.NY);
  const int iy = icm / cg.NX - cg.NY * iz;
  const double4_32a xi = xs[p];
  const float4 xif = xsf[p];
  const int nlp = cg.nlp;
  const int nlx0e = nlp - 1, nly0e = nlp - 1, nlz0e = nlp - 1;
  const int nlx1s = cg.nlx + nlp, nly1s = cg.nly + nlp, nlz1s = cg.nlz + nlp;
  int* li = list + (size_t)i * ld + 3;  // li[k] == list(k, i)
  int* si = spos + (size_t)i * ldt;
  int count = 0;
  int ncand64 = 0, nfwd = 0, nbwd = 0;
  const unsigned lt = (1u << lane) - 1u;
  for (int pass = 1; pass <= 2; ++pass) {
    if (pass == 2) {
      const int ix1 = ix - nlx0e, ix2 = ix - nlx1s, iy1 = iy - nly0e, iy2 = iy - nly1s, iz1 = iz - nlz0e,
                iz2 = iz - nlz1s;
      bool border = (ix1 >= 1 && ix1 <= nlp) || (ix2 <= -1 && ix2 >= -nlp) || (iy1 >= 1 && iy1 <= nlp) ||
                    (iy2 <= -1 && iy2 >= -nlp) || (iz1 >= 1 && iz1 <= nlp) || (iz2 <= -1 && iz2 >= -nlp);
      if (!border) break;
    }
    for (int kk = (pass == 1 ? 0 : 1); kk < nsbcll; ++kk) {
      int jc, s;
      if (pass == 1) {
        jc = ic + c_off[kk];
        s = (jc != ic) ? start[jc] : p + 1;
      } else {
        int jx = ix - c_nix[kk], jy = iy - c_niy[kk], jz = iz - c_niz[kk];
        if (!(jx <= nlx0e || jx >= nlx1s || jy <= nly0e || jy >= nly1s || jz <= nlz0e || jz >= nlz1s)) continue;
        jc = ic - c_off[kk];
        s = start[jc];
      }
      const int e = start[jc + 1];
      const bool nir = c_nir[kk] != 0;
      for (int b = s; b < e; b += 32) {
        const int jj = b + lane;
        bool acc = false;
        if (jj < e) {
          if (nir) {
            acc = true;
          } else {
            float4 xj = xsf[jj];
            float dx = xj.x - xif.x, dy = xj.y - xif.y, dz = xj.z - xif.z;
            float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < cg.rcsq_lo) {
              acc = true;
            } else if (r2 <= cg.rcsq_hi) {
              double4_32a xd = xs[jj];
              double ddx = sub_rn(xd.x, xi.x), ddy = sub_rn(xd.y, xi.y), ddz = sub_rn(xd.z, xi.z);
              double rsq = add_rn(add_rn(mul_rn(ddx, ddx), mul_rn(ddy, ddy)), mul_rn(ddz, ddz));
              acc = rsq <= cg.rcsq;
              ++ncand64;
            }
          }
        }
        const unsigned m = __ballot_sync(0xffffffffu, acc);
        if (acc) {
          const int k = count + __popc(m & lt) + 1;
          const int a = at_list[jj];
          if (pass == 1) nfwd += a >= natms;
          else ++nbwd;
          if (k <= max_list) {
            li[k] = a + 1;
            si[k] = pass == 1 ? jj : -1;
          }
        }
        count += __popc(m);
      }
    }
  }
  ncand64 = warp_sumi(ncand64);
  nfwd = warp_sumi(nfwd);
  nbwd = warp_sumi(nbwd);
  if (lane == 0) {
    if (nfwd) atomicAdd(&sc->halo_fwd, nfwd);
    if (nbwd) atomicAdd(&sc->halo_bwd, nbwd);
  }
  if (lane == 0) {
    // the stored length never exceeds max_list, so no later kernel can read
    // past the column even when the overflow status is ignored
    const int stored = min(count, max_list);
    li[0] = stored;
    li[-1] = stored;
    li[-2] = stored;
    li[-3] = stored;
    if (count > max_list) {
      atomicOr(&sc->status, ST_LIST_OVERFLOW);
      atomicMax(&sc->ibig, count);
    }
    if (ncand64) atomicAdd(&sc->ncand_fp64, ncand64);
  }
}

// Row tables of the cell tiles: per row (dy, dz) the first sorted position of its x run
// of cells and its slot base in the tile's staged set; per tile the staged total and the
// sorted-position range of its own (i) atoms.  Tiles above the capacity of the first
// launches go to tile_over for a second launch with more shared memory.
__global__ void k_tile_rows(TilePlan tp, CellGeom cg, const int* __restrict__ start, int* __restrict__ tile_rows,
                            int* __restrict__ tile_info, int cap, int* __restrict__ tile_over, DevScalars* sc) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tp.ntiles) return;
  const int tx = t % tp.ntx, ty = (t / tp.ntx) % tp.nty, tz = t / (tp.ntx * tp.nty);
  const int nlp = cg.nlp;
  const int x0 = nlp + tx * tp.m, x1 = min(x0 + tp.m, nlp + cg.nlx);  // own cells [x0, x1)
  const int y = nlp + ty, z = nlp + tz;
  int base = 0;
  for (int r = 0; r < tp.nrows; ++r) {
    const int plane = cg.NX * ((y + tp.dy[r]) + cg.NY * (z + tp.dz[r]));
    const int clo = 1 + (x0 + tp.dxlo[r]) + plane, chi = 1 + (x1 - 1 + tp.dxhi[r]) + plane;
    const int f = start[clo], e = start[chi + 1];
    tile_rows[2 * (t * tp.nrows + r)] = f;
    tile_rows[2 * (t * tp.nrows + r) + 1] = base;
    base += e - f;
  }
  const int plane = cg.NX * (y + cg.NY * z);
  tile_info[4 * t] = base;
  tile_info[4 * t + 1] = start[1 + x0 + plane];
  tile_info[4 * t + 2] = start[1 + (x1 - 1) + plane + 1];
  tile_info[4 * t + 3] = 0;
  if (base > cap) tile_over[atomicAdd(&sc->tile_over, 1)] = t;
  atomicMax(&sc->tile_max, base);
}

// Half-shell Verlet list (neighbours.F90:876-1184), one CTA per cell tile: the tile's
// forward half shell (FP32 positions and atom ids) is staged in shared memory and one
// warp per local atom walks it in the reference order (semi-ball cell by cell, each
// cell's members in ascending order), one run of consecutive cells at a time, with
// ballot compaction.  Beside list(k, i) the kernel writes spos(k, i): the partner's
// sorted position, or -1 for the entries of the backward halo pass (pass 2), whose
// pairs the partner atom's forward pass also lists, so that the pair kernels evaluate
// each pair once, from its forward copy.
__global__ void __launch_bounds__(256) k_list_tiles(int natms, CellGeom cg, TilePlan tp, int nsbcll, int nseg,
                                                    const int* __restrict__ tile_ids, int cap,
                                                    const int* __restrict__ tile_rows, const int* __restrict__ tile_info,
                                                    const int* __restrict__ at_list, const int* __restrict__ which_cell,
                                                    const int* __restrict__ start, const double4_32a* __restrict__ xs,
                                                    const float4* __restrict__ xsf, int* list, int ld, int* spos,
                                                    int ldt, int max_list, DevScalars* sc) {
  extern __shared__ float4 s_x[];  // cap staged FP32 positions, then cap atom ids
  int* s_at = reinterpret_cast<int*>(s_x + cap);
  __shared__ int s_first[TILE_MAX_ROWS], s_base[TILE_MAX_ROWS + 1];
  const int t = tile_ids ? tile_ids[blockIdx.x] : blockIdx.x;
  const int nst = tile_info[4 * t];
  if (nst > cap) return;  // the overflow launch builds this tile (uniform over the CTA)
  const int nrows = tp.nrows;
  if (threadIdx.x < nrows) {
    s_first[threadIdx.x] = tile_rows[2 * (t * nrows + threadIdx.x)];
    s_base[threadIdx.x] = tile_rows[2 * (t * nrows + threadIdx.x) + 1];
  }
  if (threadIdx.x == 0) s_base[nrows] = nst;
  __syncthreads();
  for (int r = 0; r < nrows; ++r) {
    const int b = s_base[r], cnt = s_base[r + 1] - b, f = s_first[r];
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      s_x[b + e] = xsf[f + e];
      s_at[b + e] = at_list[f + e];
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const int ip0 = tile_info[4 * t + 1], ip1 = tile_info[4 * t + 2];
  const int nlp = cg.nlp;
  const int nlx0e = nlp - 1, nly0e = nlp - 1, nlz0e = nlp - 1;
  const int nlx1s = cg.nlx + nlp, nly1s = cg.nly + nlp, nlz1s = cg.nlz + nlp;
  int ncand64 = 0, nfwd = 0, nbwd = 0;
  for (int p = ip0 + warp; p < ip1; p += nw) {
    const int i0s = s_base[tp.r00] - s_first[tp.r00];
    const int i = s_at[p + i0s];
    const int ic = which_cell[i];
    const int icm = ic - 1;
    const int ix = icm % cg.NX;
    const int iz = icm / (cg.NX * cg.NY);
    const int iy = icm / cg.NX - cg.NY * iz;
    const double4_32a xi = xs[p];
    const float4 xif = s_x[p + i0s];
    int* li = list + (size_t)i * ld + 3;  // li[k] == list(k, i)
    int* si = spos + (size_t)i * ldt;
    int count = 0;
    // pass 1: the forward half shell, all of it staged, one run of cells at a time
    for (int sg = 0; sg < nseg; ++sg) {
      const int r = c_seg_row[sg];
      const int sl0 = s_base[r] - s_first[r];  // slot = sorted position + sl0
      const int s0 = sg == 0 ? p + 1 : start[ic + c_seg_off0[sg]];  // segment 0 starts with the own cell
      const int e = start[ic + c_seg_off1[sg] + 1];
      const bool nir = c_seg_nir[sg] != 0;
      for (int b = s0; b < e; b += 32) {
        const int jj = b + lane;
        bool acc = false;
        if (jj < e) {
          if (nir) {
            acc = true;
          } else {
            const float4 xj = s_x[jj + sl0];
            const float dx = xj.x - xif.x, dy = xj.y - xif.y, dz = xj.z - xif.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < cg.rcsq_lo) {
              acc = true;
            } else if (r2 <= cg.rcsq_hi) {
              const double4_32a xd = xs[jj];
              const double ddx = sub_rn(xd.x, xi.x), ddy = sub_rn(xd.y, xi.y), ddz = sub_rn(xd.z, xi.z);
              const double rsq = add_rn(add_rn(mul_rn(ddx, ddx), mul_rn(ddy, ddy)), mul_rn(ddz, ddz));
              acc = rsq <= cg.rcsq;
              ++ncand64;
            }
          }
        }
        const unsigned m = __ballot_sync(0xffffffffu, acc);
        if (acc) {
          const int k = count + __popc(m & lt) + 1;
          const int a = s_at[jj + sl0];
          nfwd += a >= natms;
          if (k <= max_list) {
            li[k] = a + 1;
            si[k] = jj;
          }
        }
        count += __popc(m);
      }
    }
    // pass 2: backward cells that are halo cells (border atoms only), from global memory
    const int ix1 = ix - nlx0e, ix2 = ix - nlx1s, iy1 = iy - nly0e, iy2 = iy - nly1s, iz1 = iz - nlz0e,
              iz2 = iz - nlz1s;
    const bool border = (ix1 >= 1 && ix1 <= nlp) || (ix2 <= -1 && ix2 >= -nlp) || (iy1 >= 1 && iy1 <= nlp) ||
                        (iy2 <= -1 && iy2 >= -nlp) || (iz1 >= 1 && iz1 <= nlp) || (iz2 <= -1 && iz2 >= -nlp);
    if (border) {
      for (int kk = 1; kk < nsbcll; ++kk) {
        const int jx = ix - c_nix[kk], jy = iy - c_niy[kk], jz = iz - c_niz[kk];
        if (!(jx <= nlx0e || jx >= nlx1s || jy <= nly0e || jy >= nly1s || jz <= nlz0e || jz >= nlz1s)) continue;
        const int jc = ic - c_off[kk];
        const int s0 = start[jc], e = start[jc + 1];
        const bool nir = c_nir[kk] != 0;
        for (int b = s0; b < e; b += 32) {
          const int jj = b + lane;
          bool acc = false;
          if (jj < e) {
            if (nir) {
              acc = true;
            } else {
              const float4 xj = xsf[jj];
              const float dx = xj.x - xif.x, dy = xj.y - xif.y, dz = xj.z - xif.z;
              const float r2 = dx * dx + dy * dy + dz * dz;
              if (r2 < cg.rcsq_lo) {
                acc = true;
              } else if (r2 <= cg.rcsq_hi) {
                const double4_32a xd = xs[jj];
                const double ddx = sub_rn(xd.x, xi.x), ddy = sub_rn(xd.y, xi.y), ddz = sub_rn(xd.z, xi.z);
                const double rsq = add_rn(add_rn(mul_rn(ddx, ddx), mul_rn(ddy, ddy)), mul_rn(ddz, ddz));
                acc = rsq <= cg.rcsq;
                ++ncand64;
              }
            }
          }
          const unsigned m = __ballot_sync(0xffffffffu, acc);
          if (acc) {
            const int k = count + __popc(m & lt) + 1;
            ++nbwd;
            if (k <= max_list) {
              li[k] = at_list[jj] + 1;
              si[k] = -1;
            }
          }
          count += __popc(m);
        }
      }
    }
    if (lane == 0) {
      // the stored length never exceeds max_list, so no later kernel can read
      // past the column even when the overflow status is ignored
      const int stored = min(count, max_list);
      li[0] = stored;
      li[-1] = stored;
      li[-2] = stored;
      li[-3] = stored;
      if (count > max_list) {
        atomicOr(&sc->status, ST_LIST_OVERFLOW);
        atomicMax(&sc->ibig, count);
      }
    }
  }
  ncand64 = warp_sumi(ncand64);
  nfwd = warp_sumi(nfwd);
  nbwd = warp_sumi(nbwd);
  if (lane == 0) {
    if (ncand64) atomicAdd(&sc->ncand_fp64, ncand64);
    if (nfwd) atomicAdd(&sc->halo_fwd, nfwd);
    if (nbwd) atomicAdd(&sc->halo_bwd, nbwd);
  }
}

// Frozen (neighbours.F90:1198-1225) and excluded (:1229-1306) reordering, one
// thread per atom, sequential exactly as the reference swaps.
// The sorted positions in spos follow their list entries through every swap.
__global__ void k_list_reorder(int natms, int* list, int ld, int* spos, int ldt, const int* lfrzn,
                               const int* ltg, const int* list_excl, int ldx, int megfrz, int lbook) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natms) return;
  int* li = list + (size_t)i * ld + 3;
  int* ti = spos + (size_t)i * ldt;
  int l_end = li[0], m_end = l_end;
  if (megfrz > 1 && lfrzn[i] > 0) {
    for (int kk = l_end; kk >= 1; --kk) {
      int j = li[kk];
      if (lfrzn[j - 1] > 0) {
        if (kk < m_end) {
          li[kk] = li[m_end]; li[m_end] = j;
          const int tk = ti[kk]; ti[kk] = ti[m_end]; ti[m_end] = tk;
        }
        --m_end;
      }
    }
  }
  li[-2] = li[0];
  li[0] = m_end;
  if (lbook) {
    l_end = li[0];
    m_end = l_end;
    const int* ex = list_excl + (size_t)i * ldx;
    int ii = ex[0];
    if (ii > 0) {
      for (int kk = l_end; kk >= 1; --kk) {
        int j = li[kk];
        int jj = ltg[j - 1];
        bool hit = false;
        for (int t = 1; t <= ii; ++t) hit |= (ex[t] == jj);
        if (hit) {
          if (kk < m_end) {
            li[kk] = li[m_end]; li[m_end] = j;
            const int tk = ti[kk]; ti[kk] = ti[m_end]; ti[m_end] = tk;
          }
          --m_end;
        }
      }
    }
    li[-1] = li[0];
    li[0] = m_end;
    li[-3] = li[0];
  } else {
    li[-1] = li[0];
    li[-3] = li[0];
  }
}

// FP32 copy of positions + charge (mixed path and prefilter helpers)
// FP32 positions as an unevaluated sum hi + lo: in a large box the FP32
// coordinate alone carries an absolute error of up to half an ulp of |x|
// (7.6e-6 A at 180 A), while hi_i - hi_j + (lo_i - lo_j) keeps pair
// separations to FP32 precision of the separation itself.
// FP32 hi parts with the charge, and the lo remainders with the atom type in the
// fourth word (bit pattern), so a pair reads everything about j in two 16-byte loads
// Both records in one pass over the atoms (the FP64 values converted once): by atom index
// (xf, xlo: the type in xlo.w) and, for the sorted-position pair kernels, per sorted
// position sorted_pos[i] (xhs, xls: the charge's remainder in xls.w, tys)
__global__ void k_pos_records(const DevScalars* sc, const int* __restrict__ sorted_pos, const double* __restrict__ x,
                              const double* __restrict__ y, const double* __restrict__ z, const double* __restrict__ q,
                              const int* __restrict__ ltype, float4* xf, float4* xlo, float2* qdf, float4* xhs,
                              float4* xls, unsigned char* tys, uint2* xlh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc->nlast) return;
  const double xa = x[i], ya = y[i], za = z[i], qa = q[i];
  const int ta = ltype[i];
  const float hx = (float)xa, hy = (float)ya, hz = (float)za, hq = (float)qa;
  const float lx = (float)(xa - (double)hx), ly = (float)(ya - (double)hy), lz = (float)(za - (double)hz);
  xf[i] = make_float4(hx, hy, hz, hq);
  xlo[i] = make_float4(lx, ly, lz, __int_as_float(ta));
  const float lq = (float)(qa - (double)hq);
  if (qdf) qdf[i] = make_float2(hq, lq);
  if (xhs) {
    const int p = sorted_pos[i];
    xhs[p] = make_float4(hx, hy, hz, hq);
    if (xlh) {  // the mixed form's 8-byte record (pair_lo_type decodes it)
      xlh[p] = pack_lo_type(lx, ly, lz, ta);
    } else {
      xls[p] = make_float4(lx, ly, lz, lq);
      tys[p] = (unsigned char)ta;
    }
  }
}

inline int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// ====================================================================== host
extern void dcell_host(const double* aaa, double* bbb);
extern void invert_host(const double* a, double* b, double* d);

static void upload_adds();

void list_setup() {
  // set_halo_particles constants (halo.F90:184-247)
  double cut = g.rcutx + 1.0e-6;
  double cp[10];
  dcell_host(g.cell, cp);
  int nl[3];
  for (int d = 0; d < 3; ++d) nl[d] = (int)(cp[6 + d] / (cut * 1.0));
  double det;
  invert_host(g.cell, h_halo.rc, &det);
  for (int d = 0; d < 3; ++d) {
    double cw = 1.0 / (double)(nl[d] * 1);
    // SPME needs a wider negative-direction halo for its splines (halo.F90:218-231);
    // without electrostatics the link-cell width alone
    double ecw = g.has_coul ? std::max(cw, (double)g.p.spline_pad / (double)g.p.kmax[d]) : cw;
    h_halo.ecw[d] = std::nextafter((-0.5 + ecw) + 0.0 * 1.0, 2.0) + DBL_MIN;
    h_halo.cw[d] = std::nextafter((-0.5 - cw) + 1.0 * 1.0, -2.0) - DBL_MIN - (nl[d] == 1 ? cw * 1.0e-10 : 0.0);
  }
  // export add vectors (deport_data.F90:1790-1796)
  const double* c = g.cell;
  const double sh[6][3] = {{+1, 0, 0}, {-1, 0, 0}, {0, +1, 0}, {0, -1, 0}, {0, 0, +1}, {0, 0, -1}};
  for (int m = 0; m < 6; ++m) {
    double u = sh[m][0], v = sh[m][1], w = sh[m][2];
    h_add[m][0] = c[0] * u + c[3] * v + c[6] * w;
    h_add[m][1] = c[1] * u + c[4] * v + c[7] * w;
    h_add[m][2] = c[2] * u + c[5] * v + c[8] * w;
  }
  upload_adds();
  // link-cell geometry (neighbours.F90:396-463)
  double cut2 = g.rcutx + 1.0e-6;
  double disp[3] = {1.0 * cp[6] / cut2, 1.0 * cp[7] / cut2, 1.0 * cp[8] / cut2};
  int nlx = (int)disp[0], nly = (int)disp[1], nlz = (int)disp[2];
  int nlp = 1;
  double nlr2 = (double)g.natms;
  double dd = (nlx * nly * nlz) ? nlr2 / (double)(nlx * nly * nlz) : 0.0;
  while (nlx * nly * nlz > 0 && dd > g.p.pdplnc) {
    nlp = nlp + 1;
    double rr = (double)nlp;
    nlx = (int)(disp[0] * rr); nly = (int)(disp[1] * rr); nlz = (int)(disp[2] * rr);
    dd = nlr2 / (double)(nlx * nly * nlz);
  }
  g.nlx = nlx; g.nly = nly; g.nlz = nlz; g.nlp = nlp;
  g.NX = nlx + 2 * nlp; g.NY = nly + 2 * nlp; g.NZ = nlz + 2 * nlp;
  g.ncells = g.NX * g.NY * g.NZ;
  std::vector<int> off, nix, niy, niz;
  std::vector<unsigned char> nir;
  int nlp2 = nlp * nlp, nlp3 = (nlp - 1) * (nlp - 1);
  for (int iz = 0; iz <= nlp; ++iz) {
    int iz1 = iz > 0 ? (iz - 1) * (iz - 1) : 0, jz = iz * iz;
    for (int iy = -nlp; iy <= nlp; ++iy) {
      if (iz == 0 && iy < 0) continue;
      int a = std::abs(iy), iy1 = a > 0 ? (a - 1) * (a - 1) : 0, ll = iz1 + iy1;
      if (ll > nlp2) continue;
      int jy = jz + iy * iy;
      for (int ix = -nlp; ix <= nlp; ++ix) {
        if (iz == 0 && iy == 0 && ix < 0) continue;
        int b = std::abs(ix), ix1 = b > 0 ? (b - 1) * (b - 1) : 0;
        if (ll + ix1 > nlp2) continue;
        int jx = jy + ix * ix;
        nix.push_back(ix); niy.push_back(iy); niz.push_back(iz);
        nir.push_back(jx < nlp3 ? 1 : 0);
        off.push_back(ix + g.NX * (iy + g.NY * iz));
      }
    }
  }
  g.nsbcll = (int)off.size();
  if (g.nsbcll > MAX_SBC) throw (int)GB_ERR_ARG;
  // cell tiles: the rows (dy, dz) of the forward half shell in the order they first
  // appear, each with the range of dx its cells take
  {
    TilePlan& tp = g.tp;
    tp = TilePlan{};
    std::vector<unsigned char> row(off.size());
    for (size_t k = 0; k < off.size(); ++k) {
      int r = 0;
      while (r < tp.nrows && !(tp.dy[r] == niy[k] && tp.dz[r] == niz[k])) ++r;
      if (r == tp.nrows) {
        if (tp.nrows == TILE_MAX_ROWS) throw (int)GB_ERR_ARG;
        tp.dy[r] = niy[k]; tp.dz[r] = niz[k]; tp.dxlo[r] = nix[k]; tp.dxhi[r] = nix[k];
        ++tp.nrows;
      }
      tp.dxlo[r] = std::min(tp.dxlo[r], nix[k]);
      tp.dxhi[r] = std::max(tp.dxhi[r], nix[k]);
      row[k] = (unsigned char)r;
    }
    tp.r00 = row[0];  // offset (0, 0, 0) comes first; its row starts at dx = 0
    if (nix[0] != 0 || niy[0] != 0 || niz[0] != 0 || tp.dxlo[tp.r00] != 0) throw (int)GB_ERR_ARG;
    GB_CUDA(cudaMemcpyToSymbol(c_row, row.data(), row.size()));
    // segments: consecutive semi-ball cells of one row, adjacent along x, with one nir flag
    std::vector<int> s0, s1;
    std::vector<unsigned char> srow, snir;
    for (size_t k = 0; k < off.size(); ++k) {
      const bool joins = k > 0 && row[k] == row[k - 1] && nix[k] == nix[k - 1] + 1 && nir[k] == nir[k - 1];
      if (joins) {
        s1.back() = off[k];
      } else {
        s0.push_back(off[k]); s1.push_back(off[k]); srow.push_back(row[k]); snir.push_back(nir[k]);
      }
    }
    g.nseg = (int)s0.size();
    GB_CUDA(cudaMemcpyToSymbol(c_seg_off0, s0.data(), sizeof(int) * s0.size()));
    GB_CUDA(cudaMemcpyToSymbol(c_seg_off1, s1.data(), sizeof(int) * s1.size()));
    GB_CUDA(cudaMemcpyToSymbol(c_seg_row, srow.data(), srow.size()));
    GB_CUDA(cudaMemcpyToSymbol(c_seg_nir, snir.data(), snir.size()));
    // tile width: the widest run of cells whose staged set stays near the capacity the
    // pair kernel's shared memory allows at two CTAs per SM
    const double apc = (double)g.natms / ((double)nlx * nly * nlz);
    auto cells_of = [&](int m) {
      int c = 0;
      for (int r = 0; r < tp.nrows; ++r) c += m + tp.dxhi[r] - tp.dxlo[r];
      return c;
    };
    int m = 1;
    const char* em = getenv("GB_TILE_M");
    if (em && atoi(em) > 0) {
      m = std::min(atoi(em), nlx);
    } else {
      for (int t = 2; t <= std::min(nlx, 8); ++t)
        if (1.3 * cells_of(t) * apc + 64.0 <= (double)TILE_CAP_TARGET) m = t;
    }
    tp.m = m;
    tp.ntx = (nlx + m - 1) / m; tp.nty = nly; tp.ntz = nlz;
    tp.ntiles = tp.ntx * tp.nty * tp.ntz;
    int cap = (int)(1.3 * cells_of(m) * apc) + 64;
    const char* ec = getenv("GB_TILE_CAP");  // a smaller first-launch capacity sends more tiles to the second launch
    if (ec && atoi(ec) > 0) cap = atoi(ec);
    g.tile_cap_list = std::min(((cap + 31) / 32) * 32, (int)TILE_CAP_MAX);
    if (g.tiles_alloc < tp.ntiles) {
      cudaFree(g.tile_rows); cudaFree(g.tile_info); cudaFree(g.tile_over);
      GB_CUDA(cudaMalloc(&g.tile_rows, sizeof(int) * 2 * (size_t)tp.ntiles * TILE_MAX_ROWS));
      GB_CUDA(cudaMalloc(&g.tile_info, sizeof(int) * 4 * (size_t)tp.ntiles));
      GB_CUDA(cudaMalloc(&g.tile_over, sizeof(int) * (size_t)tp.ntiles));
      g.tiles_alloc = tp.ntiles;
    }
  }
  GB_CUDA(cudaMemcpyToSymbol(c_off, off.data(), sizeof(int) * off.size()));
  GB_CUDA(cudaMemcpyToSymbol(c_nix, nix.data(), sizeof(int) * nix.size()));
  GB_CUDA(cudaMemcpyToSymbol(c_niy, niy.data(), sizeof(int) * niy.size()));
  GB_CUDA(cudaMemcpyToSymbol(c_niz, niz.data(), sizeof(int) * niz.size()));
  GB_CUDA(cudaMemcpyToSymbol(c_nir, nir.data(), nir.size()));
  for (int k = 0; k < 9; ++k) h_cg.rc[k] = h_halo.rc[k];
  h_cg.xdc = (double)(nlx * 1); h_cg.ydc = (double)(nly * 1); h_cg.zdc = (double)(nlz * 1);
  h_cg.nlp = nlp; h_cg.nlx = nlx; h_cg.nly = nly; h_cg.nlz = nlz;
  h_cg.NX = g.NX; h_cg.NY = g.NY; h_cg.NZ = g.NZ;
  h_cg.rcsq = g.rcutx * g.rcutx;
  // FP32 prefilter band: the FP32 rsq of a pair differs from the exact FP64
  // one by < 4e-4 A^2 for |coordinates| < 300 A and r ~ rc (rounding of the
  // coordinates to FP32 plus the FP32 arithmetic); take 25x that bound, scaled
  // with the box size.
  double Lmax = std::max(std::max(cp[0], cp[1]), cp[2]) + 2.0 * g.rcutx;
  double band = 0.01 * std::max(1.0, Lmax / 300.0) * std::max(1.0, g.rcutx / 13.0);
  h_cg.rcsq_lo = (float)(h_cg.rcsq - band);
  h_cg.rcsq_hi = (float)(h_cg.rcsq + band);
  h_cg.half_plus = std::nextafter(0.5, 1.0);
  if (g.cells_alloc < g.ncells + 2) {
    cudaFree(g.cell_count); cudaFree(g.cell_start); cudaFree(g.cell_fill);
    GB_CUDA(cudaMalloc(&g.cell_count, sizeof(int) * (g.ncells + 2)));
    GB_CUDA(cudaMalloc(&g.cell_start, sizeof(int) * (g.ncells + 2)));
    GB_CUDA(cudaMalloc(&g.cell_fill, sizeof(int) * (g.ncells + 2)));
    g.cells_alloc = g.ncells + 2;
  }
}

int list_relocate_and_halo() {
  const int n = g.natms;
  g.spos_valid = false;  // new halo images: the sorted positions of the list are stale until the next build
  const int T = 256;
  cudaStream_t st = g.stream;
  prof_begin(P_HALO);
  // relocate_particles in serial: pbcshift (deport_data.F90:3190)
  {
    double a0 = 1.0 / g.cell[0], a4 = 1.0 / g.cell[4], a8 = 1.0 / g.cell[8];
    if (g.cubic) { a4 = a0; a8 = a0; }
    double c4 = g.cubic ? g.cell[0] : g.cell[4], c8 = g.cubic ? g.cell[0] : g.cell[8];
    k_pbcshift<<<nblocks(n, T), T, 0, st>>>(n, g.x, g.y, g.z, a0, a4, a8, g.cell[0], c4, c8,
                                            std::nextafter(0.5, 0.0));
    GB_LAUNCHED();
  }
  k_halo_flags<<<nblocks(n, T), T, 0, st>>>(n, g.x, g.y, g.z, h_halo, g.ixyz, g.src, g.shcode, g.sc);
  GB_LAUNCHED();
  const int nblk = nblocks(g.mxatms, SCAN_BLOCK);
  int* blkcount = gb_scan_scratch(2 * nblk + 2);
  int* blkoff = blkcount + nblk + 1;
  const int mdirs[6][5] = {{1, 0, 0, 1, 3}, {1, 0, 0, 2, 3}, {0, 1, 0, 10, 30},
                           {0, 1, 0, 20, 30}, {0, 0, 1, 100, 300}, {0, 0, 1, 200, 300}};
  const int dsh[6] = {+1, -1, +3, -3, +9, -9};
  for (int m = 0; m < 6; ++m) {
    const int* md = mdirs[m];
    k_export_count<<<nblk, 256, 0, st>>>(g.ixyz, g.sc, md[0], md[1], md[2], md[3], blkcount);
    GB_LAUNCHED();
    k_scan_single<<<1, 1024, 0, st>>>(blkcount, blkoff, nblk, nullptr);
    GB_LAUNCHED();
    k_export_commit<<<1, 32, 0, st>>>(blkcount, nblk, blkoff, g.sc, g.mxatms);
    GB_LAUNCHED();
    k_export_write<<<nblk, 256, 0, st>>>(g.x, g.y, g.z, g.ltg, g.src, g.shcode, g.ixyz, blkoff, g.sc, md[0], md[1],
                                          md[2], md[3], md[4], h_add[m][0], h_add[m][1], h_add[m][2], dsh[m],
                                          g.mxatms);
    GB_LAUNCHED();
  }
  k_halo_props<<<nblocks(g.mxatms - n, T), T, 0, st>>>(n, g.sc, g.src, g.ltype, g.chge, g.weight, g.lfrzn);
  GB_LAUNCHED();
  // vnl_set_check (neighbours.F90:305-343): local positions are the checkpoint
  k_set_check<<<nblocks(n, T), T, 0, st>>>(n, g.x, g.y, g.z, g.xbg, g.ybg, g.zbg);
  GB_LAUNCHED();
  prof_end(P_HALO);
  gb_sync_scalars();
  if (g.hsc->status & ST_HALO_OVERFLOW) return GB_ERR_HALO;
  return GB_OK;
}

// the image shifts on the device for the halo refresh: allocated and written where the
// list geometry is set up, copied again only when they change (a step captured into a CUDA
// graph then holds neither an allocation nor a copy from pageable host memory)
static double* d_adds = nullptr;
static double d_adds_host[18];
static void upload_adds() {
  if (!d_adds) GB_CUDA(cudaMalloc(&d_adds, sizeof(double) * 18));
  GB_CUDA(cudaMemcpy(d_adds, h_add, sizeof(double) * 18, cudaMemcpyHostToDevice));
  std::memcpy(d_adds_host, h_add, sizeof(d_adds_host));
}

int list_refresh_halo() {
  if (!d_adds || std::memcmp(d_adds_host, h_add, sizeof(d_adds_host)) != 0) upload_adds();
  k_halo_refresh<<<nblocks(g.mxatms - g.natms, 256), 256, 0, g.stream>>>(g.natms, g.sc, g.src, g.shcode, g.x, g.y,
                                                                          g.z, d_adds);
  GB_LAUNCHED();
  return GB_OK;
}

// The sorted positions of the local atoms, in sorted (cell) order: loc_sp[0, natms).  Per
// block of 1024 positions a count, then (after a scan of the counts) each block's local
// positions at its offset, ranked by a ballot prefix within each warp.
constexpr int LOC_NT = 1024;
__global__ void __launch_bounds__(LOC_NT) k_local_count(int natms, int mx, const DevScalars* sc,
                                                        const int* __restrict__ at_list, int* blkcount) {
  __shared__ int s[LOC_NT / 32];
  const int p = blockIdx.x * LOC_NT + threadIdx.x;
  const bool loc = p < min(sc->nlast, mx) && at_list[p] < natms;
  const unsigned b = __ballot_sync(0xffffffffu, loc);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < LOC_NT / 32; ++w) t += s[w];
    blkcount[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(LOC_NT) k_local_scatter(int natms, int mx, const DevScalars* sc,
                                                          const int* __restrict__ at_list,
                                                          const int* __restrict__ blkoff, int* loc_sp) {
  __shared__ int s[LOC_NT / 32];
  const int p = blockIdx.x * LOC_NT + threadIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool loc = p < min(sc->nlast, mx) && at_list[p] < natms;
  const unsigned b = __ballot_sync(0xffffffffu, loc);
  if (lane == 0) s[w] = __popc(b);
  __syncthreads();
  int before = 0;
  for (int k = 0; k < w; ++k) before += s[k];
  const int r = blkoff[blockIdx.x] + before + __popc(b & ((1u << lane) - 1u));
  if (loc && r < natms) loc_sp[r] = p;
}

int list_build() {
  const int T = 256;
  cudaStream_t st = g.stream;
  const int mx = g.mxatms;
  GB_CUDA(cudaMemsetAsync(g.cell_count, 0, sizeof(int) * (g.ncells + 2), st));
  GB_CUDA(cudaMemsetAsync(g.cell_fill, 0, sizeof(int) * (g.ncells + 2), st));
  prof_begin(P_BIN);
  k_bin<<<nblocks(mx, T), T, 0, st>>>(g.natms, g.sc, g.x, g.y, g.z, h_cg, g.which_cell, g.cell_count);
  GB_LAUNCHED();
  k_scan_single<<<1, 1024, 0, st>>>(g.cell_count, g.cell_start, g.ncells + 2, nullptr);
  GB_LAUNCHED();
  int* tmp = gb_scan_scratch(mx + 1);
  k_cell_scatter<<<nblocks(mx, T), T, 0, st>>>(g.sc, g.which_cell, g.cell_start, g.cell_fill, tmp);
  GB_LAUNCHED();
  k_cell_sort<<<nblocks((long long)(g.ncells + 1) * 32, T), T, 0, st>>>(g.ncells + 1, g.cell_start, tmp, g.at_list,
                                                                       g.sorted_pos, g.x, g.y, g.z, g.xs, g.xsf);
  GB_LAUNCHED();
  {
    const int nb = nblocks(mx, LOC_NT);
    int* cnt = gb_scan_scratch(2 * nb + 2);
    k_local_count<<<nb, LOC_NT, 0, st>>>(g.natms, mx, g.sc, g.at_list, cnt);
    GB_LAUNCHED();
    k_scan_single<<<1, 1024, 0, st>>>(cnt, cnt + nb + 1, nb, nullptr);
    GB_LAUNCHED();
    k_local_scatter<<<nb, LOC_NT, 0, st>>>(g.natms, mx, g.sc, g.at_list, cnt + nb + 1, g.loc_sp);
    GB_LAUNCHED();
  }
  prof_end(P_BIN);
  GB_CUDA(cudaMemsetAsync(&g.sc->ibig, 0, sizeof(int), st));
  GB_CUDA(cudaMemsetAsync(&g.sc->tile_over, 0, 4 * sizeof(int), st));  // tile_over, tile_max, halo_fwd, halo_bwd
  prof_begin(P_LIST);
  const TilePlan& tp = g.tp;
  const int cap = g.tile_cap_list;
  k_tile_rows<<<nblocks(tp.ntiles, 128), 128, 0, st>>>(tp, h_cg, g.cell_start, g.tile_rows, g.tile_info, cap,
                                                        g.tile_over, g.sc);
  GB_LAUNCHED();
  GB_CUDA(cudaFuncSetAttribute(k_list_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, 20 * TILE_CAP_MAX));
  k_list_tiles<<<tp.ntiles, 256, (size_t)cap * 20, st>>>(g.natms, h_cg, tp, g.nsbcll, g.nseg, nullptr, cap,
                                                          g.tile_rows, g.tile_info, g.at_list, g.which_cell,
                                                          g.cell_start, g.xs, g.xsf, g.list, g.ld, g.spos, g.ldt,
                                                          g.p.max_list, g.sc);
  GB_LAUNCHED();
  gb_sync_scalars();
  g.n_tile_over = g.hsc->tile_over;
  g.tile_max_staged = g.hsc->tile_max;
  if (g.n_tile_over > 0 && g.tile_max_staged <= TILE_CAP_MAX) {
    // the tiles above the capacity, with shared memory for the largest of them
    k_list_tiles<<<g.n_tile_over, 256, (size_t)g.tile_max_staged * 20, st>>>(
        g.natms, h_cg, tp, g.nsbcll, g.nseg, g.tile_over, g.tile_max_staged, g.tile_rows, g.tile_info, g.at_list,
        g.which_cell, g.cell_start, g.xs, g.xsf, g.list, g.ld, g.spos, g.ldt, g.p.max_list, g.sc);
    GB_LAUNCHED();
  } else if (g.n_tile_over > 0) {
    // a tile too dense for one CTA's shared memory: the whole list from the per-atom kernel
    GB_CUDA(cudaMemsetAsync(&g.sc->halo_fwd, 0, 2 * sizeof(int), st));
    k_list_pairs<<<nblocks((long long)mx * 32, T), T, 0, st>>>(g.natms, g.sc, h_cg, g.nsbcll, g.at_list,
                                                               g.which_cell, g.cell_start, g.xs, g.xsf, g.list, g.ld,
                                                               g.spos, g.ldt, g.p.max_list, g.sc);
    GB_LAUNCHED();
  }
  if (g.lbook || g.megfrz > 1) {
    k_list_reorder<<<nblocks(g.natms, 128), 128, 0, st>>>(g.natms, g.list, g.ld, g.spos, g.ldt, g.lfrzn, g.ltg,
                                                          g.list_excl, g.p.max_exclude + 1, g.megfrz,
                                                          g.lbook ? 1 : 0);
    GB_LAUNCHED();
  }
  prof_end(P_LIST);
  gb_sync_scalars();
  if (g.hsc->status & ST_LIST_OVERFLOW) return GB_ERR_LIST_OVERFLOW;
  // every pair across the periodic boundary is listed from both of its atoms, once in a
  // forward pass and once in the backward halo pass; the sorted-position pair kernels
  // evaluate the forward copy (else the atom-index kernels run, by the smaller global id)
  g.spos_valid = g.hsc->halo_fwd == g.hsc->halo_bwd;
  ++g.list_gen;  // the learned-MTS short list is rebuilt from this list on demand
  return GB_OK;
}

void list_pos_records(bool sorted) {
  k_pos_records<<<nblocks(g.mxatms, 256), 256, 0, g.stream>>>(
      g.sc, g.sorted_pos, g.x, g.y, g.z, g.chge, g.ltype, g.xf, g.xlo, g.precision == GB_FP64 ? g.qdf : nullptr,
      sorted ? g.xhs : nullptr, g.xls, g.tys, g.precision == GB_MIXED ? g.xlh : nullptr);
  GB_LAUNCHED();
}


