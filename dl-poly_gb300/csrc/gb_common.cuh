// gb_common.cuh - shared device context, error handling and small device
// helpers for the GB300 DL_POLY force/update path.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <vector>

#include "../../include/gb300_dlpoly.h"

#define GB_WARP 32

// Status word bits written by kernels (read back by the host after a stage).
enum : int {
  ST_LIST_OVERFLOW = 1,
  ST_HALO_OVERFLOW = 2,
  ST_SHAKE_FAIL = 4,
  ST_RATTLE_FAIL = 8,
  ST_NONFINITE = 16,
  ST_CELL_RANGE = 32,
  ST_SPME_RANGE = 64,
  ST_RNG = 128,          // a Box-Muller rejection loop hit its cap
  ST_METAL_TABLE = 256,  // a metal table read below its first point (error 506)
  ST_METAL_DENSITY = 512,  // a local density outside its embedding table (error 507)
  ST_DEVICE_WAIT = 1024,   // a kernel's wait on an mbarrier hit its iteration limit
};

// Device-resident scalars: one small block so a single copy returns them all.
struct DevScalars {
  int nlast;        // local + halo atoms
  int nlast_prev;   // halo size before the current export direction
  int status;       // ST_* bits
  int ibig;         // largest list length seen (overflow report)
  int update;       // vnl_check decision
  int shake_iters;
  int rattle_iters;
  int converged;    // constraint iteration flag
  int ncand_fp64;   // list-build candidates resolved in FP64
  int tile_over;    // cell tiles whose staged atoms exceed the first launch's capacity
  int tile_max;     // most staged atoms of any cell tile
  int halo_fwd;     // list entries with a halo image found in the forward half shell (evaluated)
  int halo_bwd;     // list entries with a halo image found in the backward halo pass (skipped)
  int pad[3];
  double maxdisp;   // largest displacement since the last rebuild
  unsigned long long npairs_list;  // half-list entries walked by the pair kernel
  unsigned long long npairs_rc;    // unique pairs inside the cutoff
  double acc[96];   // energy / virial / stress accumulators
  double th[8];     // thermostat state: chi_t, cint, scale, vom(3), engke, consv
};

// accumulator slots in DevScalars::acc
enum {
  A_PAIR = 0,         // 10 slots: engvdw, virvdw, engrl, virrl, stress(6)
  A_EXCL = 10,        // 8 slots: engex, virex, stress(6)
  A_SPME_STR = 20,    // 6 slots: reciprocal stress (before scale)
  A_GATHER = 30,      // 4 slots: reciprocal energy, net force (before scale)
  A_STRKIN = 40,      // 6 slots
  A_STRCON = 50,      // 6 slots
  A_KINMOM = 64,      // 9 slots: kinetic stress (6), momentum (3) of the thermostat stages
  A_METAL = 80,       // 9 slots: engmet, virmet, stress (6), engden
  A_NSLOTS = 96
};

// Cell tiles of the list build.  A tile is a run of m local link cells along x at one
// (y, z); its CTA stages in shared memory every atom of the cells that the forward half
// shell of its cells reaches, as one contiguous run of sorted positions per row
// (dy, dz) of that shell.
constexpr int TILE_MAX_ROWS = 32;
constexpr int TILE_CAP_TARGET = 1600;  // staged atoms per tile of the list build's first launch
constexpr int TILE_CAP_MAX = 8192;     // largest staged set a list CTA holds (20 B per atom)
struct TilePlan {
  int m;                    // local cells per tile along x
  int ntx, nty, ntz, ntiles;
  int nrows;                // rows (dy, dz) of the forward half shell
  int r00;                  // the row (0, 0): it starts with the tile's own cells
  int dy[TILE_MAX_ROWS], dz[TILE_MAX_ROWS], dxlo[TILE_MAX_ROWS], dxhi[TILE_MAX_ROWS];
};

// Kernel regions timed with CUDA events when profiling is on.
enum ProfId {
  P_HALO = 0, P_BIN, P_LIST, P_SHORTLIST, P_PAIR, P_EXCL, P_SPME_PREP, P_SPME_SPREAD, P_FFT_XF, P_FFT_Y,
  P_FFT_Z, P_FFT_XI, P_SPME_GATHER, P_VV, P_SHAKE, P_RATTLE, P_MLP, P_MTS_DESC, P_MLP_TRAIN, P_COARSE_PREP,
  P_COARSE_SPREAD, P_COARSE_FFT, P_COARSE_GATHER, P_METAL_DENSITY, P_METAL_FORCES, P_NPROF
};
void prof_begin(int id);
void prof_end(int id);

// All device pointers of the context.  Arrays of size mxatms hold local atoms
// in [0, natms) followed by halo images in [natms, nlast).
struct Dev {
  bool init = false;
  gb_params p{};
  int natms = 0, mxatms = 0;
  double cell[9], rcell[9], celprp[10], volm = 0, rcutx = 0;
  bool cubic = true;
  int precision = GB_FP64;
  cudaStream_t stream = nullptr;
  // The reciprocal-space sum runs on a second stream of higher priority while the pair
  // kernel runs on the first (GB_OVERLAP=0: both on the first).  During the SPME launches
  // `stream` is the side stream and `side` is set; the first stream waits for the side
  // stream before the pair forces are folded into the force arrays.
  cudaStream_t main_stream = nullptr, side_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool side = false, join_pending = false, use_overlap = true;
  int pair_apw = -1;  // atoms per warp of the sorted pair kernels' CTAs (GB_PAIR_APW; 0: resident CTAs, -1: by form)
  // work to put on the side stream once the pair kernel is launched (run by pair_forces
  // before it joins the side stream)
  void (*side_hook)(void*) = nullptr;
  void* side_hook_arg = nullptr;
  int pair_nt = 0;  // threads per CTA of the sorted pair kernels: 256 or 1024 (GB_PAIR_NT), 0: by form
  int nsm = 0;
  int64_t launches = 0;

  // atoms
  double *x = nullptr, *y = nullptr, *z = nullptr;  // mxatms
  float4* xf = nullptr;                             // FP32 copy (x,y,z,q) for prefilter / mixed
  float4* xlo = nullptr;                            // x - (double)xf.x etc.: the FP32 remainders (mixed)
  double *fx = nullptr, *fy = nullptr, *fz = nullptr;  // natms, FP64 forces
  long long* fixp = nullptr;                        // 3*natms fixed-point forces (mixed)
  double *vx = nullptr, *vy = nullptr, *vz = nullptr;
  double* hdw = nullptr;                            // natms: (tstep/2) / weight, 0 where weight <= 1e-6
  double *chge = nullptr, *weight = nullptr;        // mxatms
  int *ltype = nullptr, *ltg = nullptr, *lfrzn = nullptr;  // mxatms
  int *ixyz = nullptr, *src = nullptr;              // mxatms
  int* shcode = nullptr;                            // halo shift code (sx+1)+3(sy+1)+9(sz+1)
  double *xbg = nullptr, *ybg = nullptr, *zbg = nullptr;  // natms
  double *ox = nullptr, *oy = nullptr, *oz = nullptr;     // natms (SHAKE)

  // link cells / list
  int nlx = 0, nly = 0, nlz = 0, nlp = 0, NX = 0, NY = 0, NZ = 0, ncells = 0, nsbcll = 0, nseg = 0;
  int* which_cell = nullptr;   // mxatms
  int* cell_count = nullptr;   // ncells+2
  int* cell_start = nullptr;   // ncells+2 (0-based start)
  int* cell_fill = nullptr;    // ncells+2
  int* at_list = nullptr;      // mxatms (sorted atom ids)
  int* sorted_pos = nullptr;   // mxatms: position of atom in at_list
  double4_32a* xs = nullptr;       // mxatms sorted FP64 coordinates (x,y,z,pad)
  float4* xsf = nullptr;       // mxatms sorted FP32 coordinates
  int* list = nullptr;         // (max_list+4) * natms, Fortran layout, 1-based values
  int ld = 0;
  int cells_alloc = 0;
  int* blk = nullptr;          // scan scratch (blocks)
  int nblk_alloc = 0;
  int* list_excl = nullptr;    // (max_exclude+1)*natms
  bool lbook = false;
  int megfrz = 0;
  bool has_coul = true, has_vdw = true, has_metal = false;  // which force terms the system has
  bool fp64_native = false;    // FP64 form: pair loop in native FP64 (else double-float on FP32 pipes)
  float4* erfc_df = nullptr;   // double-float erfc tables: 3 float4 per interval
  float4* vdw_df = nullptr;    // double-float vdW tables: per key (max_grid + 3) x 3 float4
  float2* qdf = nullptr;       // charges as double-floats (mxatms), written with the FP32 positions
  // cell tiles (gb_list.cu plans and fills them at each list build)
  TilePlan tp{};
  int* tile_rows = nullptr;    // ntiles x nrows x (first sorted position, slot base)
  int* tile_info = nullptr;    // ntiles x 4: staged atoms, first and end sorted position of the i atoms
  int* tile_over = nullptr;    // ids of the tiles above the first launch's capacity
  int tiles_alloc = 0;
  int* spos = nullptr;         // natms x ldt: per list entry the partner's sorted position (-1: backward copy)
  int ldt = 0;
  int tile_cap_list = 0;       // staged atoms per tile of the list build's first launch
  int n_tile_over = 0, tile_max_staged = 0;   // from the last list build
  bool spos_valid = false;     // the last list pairs every halo entry with its backward copy
  bool use_sorted = true;      // sorted-position pair kernels (GB_PAIR_SORTED=0: the atom-index kernels)
  // NVE MD loop without constraints, thermostat, metals or learned MTS: the energy,
  // virial and stress sums of each step are copied to a pinned ring and read after the
  // last step, so the host waits only for the Verlet-list decision of each step
  bool defer_scalars = false;
  bool use_deferred = true;    // GB_MD_DEFER=0 keeps the per-step read-back
  // that loop as CUDA graphs (GB_GRAPHS=0: every kernel launched by the host): stage 1 with
  // the Verlet-list check, and a step without a list rebuild (halo refresh, forces, stage
  // 2), captured once per call and again after each rebuild; the launch counter adds each
  // graph's kernels per launch
  bool use_graphs = true;
  cudaGraphExec_t gx_vv1 = nullptr, gx_step = nullptr;
  int64_t gl_vv1 = 0, gl_step = 0;
  DevScalars* ring = nullptr;  // pinned, ring_cap steps
  int ring_cap = 0;
  // host state transfers: pinned and mapped caller buffers are read and written by one
  // kernel each way (GB_MAPPED_COPY=0: one cudaMemcpyAsync per array)
  bool use_mapped = true;
  int* hflag = nullptr;        // pinned, mapped: the upload kernel's non-finite flag
  int* dflag = nullptr;        // its device-side address
  int* loc_sp = nullptr;       // natms: the sorted positions of the local atoms, in sorted order
  float4* xhs = nullptr;       // per sorted position: FP32 high parts (x, y, z, q)
  float4* xls = nullptr;       // per sorted position: remainders (x, y, z, q) of the FP64 values
  unsigned char* tys = nullptr;  // per sorted position: atom type
  uint2* xlh = nullptr;        // mixed form, per sorted position: remainders x 2^20 as half floats, and the type
  long long* fixs = nullptr;   // 3 x mxatms fixed-point pair forces per sorted position
  double metal_e4[4] = {0, 0, 0, 0};  // engmet, virmet, engden, virden of the last evaluation
  // thermostat of the VV stages (gb_thermostat.cu)
  int ens = 0;                 // GB_NVE, GB_NVT_BERENDSEN, GB_NVT_NOSE_HOOVER, GB_NVT_LANGEVIN
  double temp = 0, tau_t = 0, chi_fric = 0;
  double sigma = 0, qmass = 0, ceng = 0, totmas = 0, degfre = 0;
  double lang_t0 = 0, lang_t1 = 0, lang_scr = 0, lang_scl = 0, lang_scv = 0;
  int seed[3] = {0, 0, 0};
  int nstep = 0;               // flow%step of the current (or next) stage-1 call
  long long list_gen = 0;      // incremented whenever the Verlet list is rebuilt

  // tables
  int nsamples = 0, max_grid = 0, nkey = 0;
  double erfc_rdr = 0, vdw_rdr = 0;
  double* erfc_coef = nullptr;   // per interval: e0,e1,e2,d0,d1,d2 (erfc/r and its derivative)
  float* erfc_coef_f = nullptr;
  double* vdw_coef = nullptr;    // per key per interval: f0,f1,f2,v0,v1,v2
  float* vdw_coef_f = nullptr;
  int* vdw_kind = nullptr;
  double* vdw_eps = nullptr;
  double* vdw_sig = nullptr;
  std::vector<int> h_vdw_kind;
  std::vector<double> h_vdw_eps, h_vdw_sig;
  double elrc = 0, vlrc = 0, self_interaction = 0, scaling = 0;

  // SPME grids live in gb_spme.cu (SpmeGrid); shared scratch here
  double* blkacc = nullptr;    // per-block partial accumulators
  int blkacc_n = 0;
  double* blkacc_s = nullptr;  // the same for launches on the side stream
  int blkacc_s_n = 0;

  // constraints
  int ntcons = 0;
  int *con_i = nullptr, *con_j = nullptr;
  double* con_d0 = nullptr;
  double *dxx = nullptr, *dyy = nullptr, *dzz = nullptr;
  double *dxt = nullptr, *dyt = nullptr, *dzt = nullptr, *dt2 = nullptr, *gam = nullptr;
  int* listot = nullptr;
  int *acon_start = nullptr, *acon_list = nullptr;  // per-atom constraint CSR (ordered by k)
  double *cxt = nullptr, *cyt = nullptr, *czt = nullptr;  // per-atom corrections

  DevScalars* sc = nullptr;    // device scalars
  DevScalars* hsc = nullptr;   // pinned host mirror

  // timing
  cudaEvent_t ev[8];
  double last_ms[8];

  // profiling
  bool prof_on = false;
  double prof_ms[P_NPROF];
  long long prof_n[P_NPROF];
  std::vector<cudaEvent_t> evpool;
  std::vector<int> pend;  // triples (id, ev_begin, ev_end)
  int ev_used = 0;
  int open_ev[P_NPROF];

  // learned MTS
  int mts_k = 1;
  double mts_tol = 1e-4;
  int mts_train = 0;
  void* mts = nullptr;
};

extern Dev g;

#define GB_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      std::fprintf(stderr, "gb300: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), \
                   __FILE__, __LINE__);                                            \
      throw (int)GB_ERR_CUDA;                                                      \
    }                                                                              \
  } while (0)

#define GB_LAUNCHED() \
  do {                \
    ++g.launches;     \
    GB_CUDA(cudaGetLastError()); \
  } while (0)

// ------------------------------------------------------------ device helpers
// The mixed form's per-sorted-position record of the FP32 remainders x - (float)x (at most
// half an FP32 ulp of the coordinate) and the atom type in 8 bytes: the remainders times
// 2^20 as half floats (11 significant bits of the remainder: ~1e-9 A for coordinates below
// 128 A; a remainder times 2^20 stays below the half range for coordinates below 2^19 A),
// the type in the top 16 bits.
__device__ __forceinline__ uint2 pack_lo_type(float lx, float ly, float lz, int type) {
  const __half2 h = __floats2half2_rn(lx * 1048576.0f, ly * 1048576.0f);
  uint2 r;
  r.x = *reinterpret_cast<const unsigned int*>(&h);
  r.y = (unsigned int)__half_as_ushort(__float2half_rn(lz * 1048576.0f)) | ((unsigned int)type << 16);
  return r;
}
__device__ __forceinline__ void pair_lo_type(uint2 r, float& lx, float& ly, float& lz, int& type) {
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&r.x));
  lx = a.x * 9.5367431640625e-07f;  // 2^-20
  ly = a.y * 9.5367431640625e-07f;
  lz = __half2float(__ushort_as_half((unsigned short)(r.y & 0xffffu))) * 9.5367431640625e-07f;
  type = (int)(r.y >> 16);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_sumi(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Exact-rounding FP64 helpers (never contracted into FMA): used wherever the
// result must match the FP64 oracle bit for bit (binning, pair-set tests).
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// x * 2^40 as int64, rounded toward zero, by integer operations only (on this
// part a float -> int64 conversion runs on the slow FP64 unit).  |x| < 2^23,
// the range of the 2^40 fixed-point format used for forces and grid charges.
__device__ __forceinline__ long long fix40(float x) {
  const unsigned u = __float_as_uint(x);
  const int sh = (int)((u >> 23) & 0xFFu) - 127 + 17;  // x = m 2^(e-23), m 24-bit: x 2^40 = m 2^(e+17)
  const unsigned m = (u & 0x7FFFFFu) | 0x800000u;
  // branchless: left shift for sh >= 0 (<= 39 in range), right shift otherwise (>= 24 gives 0)
  const unsigned long long up = (unsigned long long)m << min(max(sh, 0), 39);
  const unsigned long long dn = (unsigned long long)(m >> min(max(-sh, 0), 31));
  const long long v = (long long)(sh >= 0 ? up : dn);
  return (int)u < 0 ? -v : v;
}

// FP64 helpers for kernels bound by the FP64 pipe, where a compare or a conversion
// costs a full FP64 issue slot: they work on IEEE bit patterns with integer ops.
constexpr long long DBL_MIN_BITS = 0x0010000000000000ll;  // bits of DBL_MIN
constexpr long long ONE_BITS = 0x3FF0000000000000ll;      // bits of 1.0

// exact double of 0 <= k < 2^31 from its bits: (2^52 + k) - 2^52, one FP64 add
__device__ __forceinline__ double int_to_dbl(int k) {
  return __longlong_as_double(0x4330000000000000ll + (long long)k) - 4503599627370496.0;
}

// FP32 value of a positive normal double, mantissa truncated, by integer ops
__device__ __forceinline__ float dbl_to_flt_trunc(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned e = ((hi >> 20) & 0x7FFu) - 1023u + 127u;
  const unsigned m = ((hi & 0xFFFFFu) << 3) | ((unsigned)b >> 29);
  return __uint_as_float((e << 23) | m);
}

// exact FP64 value of a positive normal float, by integer ops
__device__ __forceinline__ double flt_to_dbl(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long e = (unsigned long long)(((u >> 23) & 0xFFu) - 127u + 1023u);
  return __longlong_as_double((long long)((e << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

// 1/sqrt(v) for a positive normal double: FP32 rsqrt seed of the truncated value and
// one FP64 Newton step (relative error < 1e-13), three FP64 instructions
__device__ __forceinline__ double rsqrt_seeded(double v) {
  const double r = flt_to_dbl(rsqrtf(dbl_to_flt_trunc(v)));
  return r * fma(-0.5 * v * r, r, 1.5);
}

// Block-wide reduction of NV doubles into per-block slots out[blockIdx.x*NV + k].
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double* out) {
  __shared__ double red[32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) red[wid][k] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = lane < nw ? red[lane][k] : 0.0;
      t = warp_sum(t);
      if (lane == 0) out[(size_t)blockIdx.x * NV + k] = t;
    }
  }
}

// FP32 variant: sums in FP32 and converts only the NV block totals (one thread)
// to FP64, so an FP32 kernel issues no FP64 instruction per warp.
template <int NV>
__device__ __forceinline__ void block_reduce_store(float (&v)[NV], double* out) {
  __shared__ float redf[32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sumf(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) redf[wid][k] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      float t = lane < nw ? redf[lane][k] : 0.f;
      t = warp_sumf(t);
      if (lane == 0) out[(size_t)blockIdx.x * NV + k] = (double)t;
    }
  }
}

// host helpers implemented in gb_api.cu
void gb_sync_scalars();           // copy device scalars to the pinned mirror (synchronises)
double* gb_blkacc(int n);         // per-block accumulator scratch with n doubles
void gb_reduce_blocks(const double* blk, int nblocks, int nv, double* out_dev);  // sums into out_dev[0..nv)
int* gb_scan_scratch(int n);
void side_join();                 // the first stream waits for the side stream (no-op without a fork)
void run_side_hook();             // enqueue the pending side-stream work (g.side_hook), if any

// module entry points (host)
int list_relocate_and_halo();     // pbcshift + halo + vnl_set_check (gb_list.cu)
int list_refresh_halo();          // refresh halo positions (gb_list.cu)
int list_build();                 // binning + pairs (gb_list.cu)
void list_setup();                // link-cell geometry (gb_list.cu)
void list_pos_records(bool sorted);  // FP32 hi/lo positions by atom index and (sorted) per sorted position
void scan_exclusive(const int* in, int* out, int n);
void pair_forces(double* eng6, double* stress9);  // gb_pair.cu (adds into forces)
void pair_setup();                // gb_pair.cu: per-key constants
void spme_setup();                // gb_spme.cu: the main grid
void spme_forces(double* eng_rc, double* vir_rc, double* stress9);  // adds into forces
void spme_free();                 // both grids
// coarse FP32 grid of the learned-MTS form: K per dimension and spline order p
void spme_coarse_setup(const int* K, int p);
bool spme_coarse_ready();
// scaled per-atom reciprocal forces of the coarse grid into rec (3*natms
// floats, net force removed); forces of the context are not touched
void spme_coarse_forces(double* eng_rc, double* vir_rc, double* stress9, float* rec);
void integ_vv(int stage, double* strkin, double* engke, int* iters, double* vircon, double* strcon);
// host-side results from a copy of the device scalars (the MD loop's deferred read-back)
void spme_scalars(const DevScalars* h, double* eng_rc, double* vir_rc, double* stress9);
void pair_scalars(const DevScalars* h, double* eng6, double* stress9);
void kin_scalars(const DevScalars* h, double* strkin, double* engke);
void integ_con_tags();            // constraints_tags: old bond vectors from the current positions
void integ_shake(int* iters, double* vircon, double* strcon);  // apply_shake (throws GB_ERR_SHAKE)
void integ_rattle_launch();       // apply_rattle, kit = 1 (status bit ST_RATTLE_FAIL)
int integ_vnl_check();
void integ_vnl_launch();          // the displacement check, its sums copied to the pinned scalars
int integ_vnl_result();           // its decision from the copied scalars (after a wait)
void integ_zero_forces();
void integ_forces_to_fp64();      // mixed: fixed point -> FP64 forces
void integ_setup_constraints(const int32_t* listcon, const double* prmcon);
// thermostats (gb_thermostat.cu)
void thermo_setup(int kind, double temp, double tau_t, double chi, const int32_t* seed, double degfre);
bool thermo_vv1(double hstep, double tstep);              // NH / Langevin stage-1 update; false: plain VV
bool thermo_vv2_finish(double* strkin, double* engke);   // stage 2 after RATTLE; false: plain kinstress
void thermo_state(double* chi_t, double* cint, double* consv);
void thermo_set_state(double chi_t, double cint);
void rng_eval(int mode, int n, const int64_t* a, const int64_t* b, const int64_t* c, double* out);
// tabulated EAM metals (gb_metal.cu)
int metal_setup(int ntab, const int32_t* kind, const int32_t* t1, const int32_t* t2, const int32_t* ngrid,
                const double* start, const double* finish, const double* values, const int32_t* listed);
void metal_free();
bool metal_active();
void metal_forces(double* e4, double* stress9);   // engmet, virmet, engden, virden
void metal_rho(double* out, int n);
// learned multiple-time-step form (gb_mlp.cu)
constexpr double MTS_RCUT_DESC = 6.0;  // reach of the network's neighbour sums (Angstrom)
void mts_set_topology(int ntcons, const int32_t* listcon, const double* weight);
void mts_setup();
void mts_free();
bool mts_active();
void mts_set_no_network(bool on);  // ablation: inner steps use the coarse-grid force alone
float* mts_rec_out();             // SPME per-atom reciprocal forces go here when active
bool mts_step_needs_spme();
void mts_coarse();
void mts_after_full(double erc, double vrc, const double* strec);
void mts_inner(double* erc, double* vrc, double* stress9);
void mts_stats(double* out, int nv);
int mlp_train_eval(int nb, const float* x, const float* target, const float* params, float* loss, float* grad,
                   float* yout);
int mlp_infer_eval(int nb, const float* x, const float* params, float* yout);
int mts_features(float* x, int nv, float* scal);
int mlp_param_count();
