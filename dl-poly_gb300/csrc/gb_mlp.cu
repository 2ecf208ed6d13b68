// gb_mlp.cu - learned multiple-time-step (MTS) surrogate for the SPME
// reciprocal-space force.  No counterpart exists in the reference: its
// electro%nstfce "infrequent k-space" key is parsed but two_body_forces
// evaluates SPME on every call (two_body.F90:298-302).  The plain SPME of
// gb_spme.cu is both the teacher and the fallback.
//
// Scheme: a time-reversible impulse multiple-time-step split (r-RESPA).  The
// force is split into a fast part, evaluated every step,
//     F_fast(x) = F_real(x) + S(x),   S_i(x) = C_i(x) + fs * R_i^T y_i(x),
// and a slow part F_slow = F_SPME - S, applied as an impulse every k steps: the
// force of a cycle-end step is F_fast + k F_slow (the velocity-Verlet half kicks
// before and after that step each carry k dt/2 of it).  C is the reciprocal force
// on a coarse FP32 grid (about two thirds of the points per dimension, spline order 6) and
// y = MLP(x_i) the network's correction of the coarse grid's error.  Both depend
// only on the current positions, so the inner steps integrate a fixed force field
// (C is the exact gradient of the coarse-grid energy) and no correction is carried
// over a cycle: the scheme is symmetric in time.  The net force of the network
// correction is removed, as SPME removes its own.  The reciprocal energy, virial
// and stress of an inner step are those of the last full step plus the coarse-grid
// changes since then.
// Inputs x_i (51):
//   48 = 8 Gaussians g_k(r_ij) (centres 0.5..6 A, width w = 0.45 A, cosine cut
//        at 6 A) x local-frame components of the charge-weighted radial sums
//          A_k  = q_i sum_j q_j g_k(r_ij) r^_ij                     (3)
//          A'_k = q_i sum_j q_j g_k(r_ij) ((r_ij - mu_k) / w) r^_ij  (3)
//        (the local charge environment, which fixes part of the coarse grid's
//        interpolation error);
//    3 = C_i(x) in the local frame;
// each scaled by the inverse RMS of the first labelled sample.  The local frame
// R_i of an atom of a 3-atom constrained molecule is that molecule's bisector
// frame (origin = heaviest atom); other atoms use the lab frame.
//
// Network 51 -> 128 -> 128 -> 3, SiLU, BF16 weights and activations with FP32
// accumulation.  Inference: mma.sync m16n8k16 BF16 tiles from shared memory,
// persistent CTAs.  Training: forward + MSE + backward on CUDA cores with
// BF16-rounded operands (weights, inputs, activations, activation gradients)
// and FP32 accumulation, per-CTA gradient partials summed in a fixed order,
// Adam on FP32 master weights.  Labels are R_i (F_SPME,i - C_i) / fs from the
// steps that run SPME (every step while training).  The check: at every cycle
// end after training, S of that step is compared with SPME; RMS(S - SPME) /
// RMS(total force) > tol switches to plain SPME every step (no impulses; training
// resumes) until a cycle end passes.  Each check also records the error of the
// coarse force alone (the network ablation) and of the reciprocal force of the
// previous full step held unchanged (the stale-force ablation).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "gb_common.cuh"

namespace {

constexpr int NIN = 51, KIN = 64, NH = 128, NOUT = 3, NOUTP = 16;
constexpr int NRAD = 8;  // 6 NRAD + 3 = NIN
constexpr float RCUT_DESC = (float)MTS_RCUT_DESC, GAUSS_W = 0.45f, GAUSS_MU0 = 0.5f;
constexpr int TILE_I = 256;            // atoms per inference tile (16 warps x 16 rows)
constexpr int INFER_NT = TILE_I * 2;   // its threads: one warp per 16 rows
constexpr int TILE_T = 32;  // atoms per training CTA
// FP32 parameter vector: W1[NIN][NH], b1[NH], W2[NH][NH], b2[NH], W3[NH][NOUT], b3[NOUT]
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NIN * NH, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH * NOUT, NPARAM = OFF_B3 + NOUT;
// padded shared-memory row strides (bf16 elements) that keep mma fragment loads conflict-free
constexpr int LDX = KIN + 8, LDH = NH + 8;

struct Net {  // published BF16 copy used by the inference kernel
  __nv_bfloat16 *w1t = nullptr, *w2t = nullptr, *w3t = nullptr;  // [out][in]
  float* bias = nullptr;                                         // b1 | b2 | b3 padded to NOUTP
};

struct TrainW {  // BF16 operand copies of the FP32 master weights (k_train_weights)
  __nv_bfloat16 *w1t = nullptr, *w2t = nullptr, *w3t = nullptr;  // [out][in]: forward B operands
  __nv_bfloat16 *w2b = nullptr, *w3b = nullptr;                  // [in][out]: backward B operands
  float* bias = nullptr;                                         // b1 | b2 | b3 padded to NOUTP
};

struct MtsDev {
  bool ready = false;
  int n = 0;
  float *master = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr, *gpart = nullptr, *loss_part = nullptr;
  int gpart_tiles = 0, batch = 0, train_tiles = 0;
  Net net;
  TrainW tw;                   // operands of the tensor-core training kernel
  __nv_bfloat16* X = nullptr;  // inputs [n][KIN]
  float* frec0 = nullptr;      // SPME reciprocal force of the last full step (3n)
  float* frec = nullptr;       // reciprocal force now: SPME result, or S on an inner step (3n)
  float* truth = nullptr;      // S at a full step, for the check and the impulse (3n)
  float* fc = nullptr;         // coarse-grid reciprocal force now (3n)
  int Kc[3] = {0, 0, 0}, pc = 6;
  double ec = 0.0, vc = 0.0, stc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};     // coarse now
  double ec0 = 0.0, vc0 = 0.0, stc0[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // coarse at t0
  double err_coarse = -1.0, err_stale = -1.0;
  int *sstart = nullptr, *scount = nullptr, *slist = nullptr;  // short neighbour list (CSR)
  int* stmp = nullptr;  // sort scratch of the atoms whose lists exceed the shared buffer
  int *sown = nullptr, *sfill = nullptr;  // own (half-list) entries per atom, reverse-entry fill counters
  long long scap = 0, gen_seen = -1;
  float* target = nullptr;     // labels (3n)
  float* frame = nullptr;      // local frame rows e1,e2,e3 (9n)
  int* triple = nullptr;       // frame atoms (a,b,c) per atom, -1 = lab frame
  float* scal = nullptr;       // [0,NIN) input scales, [NIN] force scale
  double* red = nullptr;       // reduction results
  int* idx = nullptr;          // training batch atom ids
  int adam_t = 0;
  int s = 0;                   // steps since t0
  int step = 0;                // MD steps since configuration
  bool have_t0 = false, scales_set = false, fallback = false, loss_pending = false;
  long long n_full = 0, n_inner = 0, n_fallback = 0, n_checked = 0;
  double last_err = -1.0, last_loss = -1.0, err_max = -1.0;
  int batch_offset = 0;
  // reciprocal energy/virial/stress of the last full step
  double erc0 = 0.0, vrc0 = 0.0, st0[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
};

MtsDev M;
std::vector<int> h_triple;  // host copy set at gb_init
bool g_no_network = false;  // ablation: S = C, the coarse force alone

inline int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

// SiLU with the approximate quotient (two instructions; within 2 ulp, far below the BF16
// rounding of the activations)
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ float bfr(float v) { return __bfloat162float(__float2bfloat16(v)); }
__device__ __forceinline__ unsigned ld2(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ------------------------------------------------------------ per-step inputs
// the local frame of every local atom
__global__ void k_mts_prep(int n, const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ z, const int* __restrict__ tri, double cell,
                           float* __restrict__ frame) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float L = (float)cell, rL = (float)(1.0 / cell);
  float e[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  const int ta = tri[3 * i], b = tri[3 * i + 1], c = tri[3 * i + 2];
  if (ta >= 0) {
    float bx = (float)(x[b] - x[ta]), by = (float)(y[b] - y[ta]), bz = (float)(z[b] - z[ta]);
    float cx = (float)(x[c] - x[ta]), cy = (float)(y[c] - y[ta]), cz = (float)(z[c] - z[ta]);
    bx -= L * rintf(bx * rL); by -= L * rintf(by * rL); bz -= L * rintf(bz * rL);
    cx -= L * rintf(cx * rL); cy -= L * rintf(cy * rL); cz -= L * rintf(cz * rL);
    float e1x = bx + cx, e1y = by + cy, e1z = bz + cz;
    float nr = rsqrtf(e1x * e1x + e1y * e1y + e1z * e1z);
    e1x *= nr; e1y *= nr; e1z *= nr;
    float ux = bx - cx, uy = by - cy, uz = bz - cz;
    const float pr = ux * e1x + uy * e1y + uz * e1z;
    ux -= pr * e1x; uy -= pr * e1y; uz -= pr * e1z;
    nr = rsqrtf(ux * ux + uy * uy + uz * uz);
    ux *= nr; uy *= nr; uz *= nr;
    e[0] = e1x; e[1] = e1y; e[2] = e1z;
    e[3] = ux; e[4] = uy; e[5] = uz;
    e[6] = e1y * uz - e1z * uy; e[7] = e1z * ux - e1x * uz; e[8] = e1x * uy - e1y * ux;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) frame[9 * i + k] = e[k];
}

// ------------------------------------------------------ short neighbour list
// Pairs within rs = 6 A + skin, rebuilt with the Verlet list: between rebuilds no
// atom moves more than half the skin, so every pair inside 6 A at any step of the
// list's lifetime is in it.  Built from the half list: an atom's entries are its own
// half-list entries within rs (a pair across the periodic boundary is listed from both
// sides, with the other side's halo image) plus, for each local partner that lists
// it, that partner (the reverse of a local-local entry).  Each atom's entries are then
// sorted by index, so the input sums do not depend on the fill order.
constexpr int SHORT_CAP = 256;  // entries sorted in shared memory per atom

// own entries within rs (sown) and the total per atom (scount, reverse entries by atomics)
__global__ void k_short_count(int n, const int* __restrict__ list, int ld, const float4* __restrict__ xf, float rs2,
                              int* __restrict__ sown, int* __restrict__ scount) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n) return;
  const float4 pi = xf[i];
  const int* li = list + (size_t)i * ld + 3;
  const int nx = li[0];  // non-excluded entries
  int c = 0;
  for (int base = 0; base < nx; base += 32) {
    bool in = false;
    if (base + lane < nx) {
      const int j = li[base + lane + 1] - 1;
      const float4 pj = xf[j];
      const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      in = dx * dx + dy * dy + dz * dz < rs2;
      if (in && j < n) atomicAdd(&scount[j], 1);
    }
    c += __popc(__ballot_sync(0xffffffffu, in));
  }
  if (lane == 0) {
    sown[i] = c;
    atomicAdd(&scount[i], c);
  }
}

// own entries first (list order), then the reverse entries at sown[j] + an atomic slot
__global__ void k_short_fill(int n, const int* __restrict__ list, int ld, const float4* __restrict__ xf, float rs2,
                             const int* __restrict__ sstart, const int* __restrict__ sown, int* __restrict__ sfill,
                             int* __restrict__ slist) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n) return;
  const float4 pi = xf[i];
  const int* li = list + (size_t)i * ld + 3;
  const int nx = li[0];
  const int s0 = sstart[i];
  int c = 0;
  for (int base = 0; base < nx; base += 32) {
    bool in = false;
    int j = 0;
    if (base + lane < nx) {
      j = li[base + lane + 1] - 1;
      const float4 pj = xf[j];
      const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      in = dx * dx + dy * dy + dz * dz < rs2;
    }
    const unsigned b = __ballot_sync(0xffffffffu, in);
    if (in) {
      slist[s0 + c + __popc(b & ((1u << lane) - 1u))] = j;
      if (j < n) slist[sstart[j] + sown[j] + atomicAdd(&sfill[j], 1)] = i;
    }
    c += __popc(b);
  }
}

// each atom's entries in ascending index order (rank sort; entries are distinct).  An
// atom with more entries than the shared buffer holds is ranked straight from global
// memory into stmp (same offsets as slist) and copied back, so every list is sorted.
__global__ void __launch_bounds__(256) k_short_sort(int n, const int* __restrict__ sstart, int* __restrict__ slist,
                                                    int* __restrict__ stmp) {
  __shared__ int buf[8][SHORT_CAP];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * 8 + w;
  if (i >= n) return;  // the whole warp leaves; no block-wide barrier below
  const int s0 = sstart[i], ns = sstart[i + 1] - s0;
  if (ns > SHORT_CAP) {
    for (int e = lane; e < ns; e += 32) {
      const int v = slist[s0 + e];
      int r = 0;
      for (int f = 0; f < ns; ++f) r += slist[s0 + f] < v;
      stmp[s0 + r] = v;
    }
    __syncwarp();
    for (int e = lane; e < ns; e += 32) slist[s0 + e] = stmp[s0 + e];
    return;
  }
  for (int e = lane; e < ns; e += 32) buf[w][e] = slist[s0 + e];
  __syncwarp();
  for (int e = lane; e < ns; e += 32) {
    const int v = buf[w][e];
    int r = 0;
    for (int f = 0; f < ns; ++f) r += buf[w][f] < v;
    slist[s0 + r] = v;
  }
}

// inputs: one thread per atom over its short neighbour list (local and halo j), in
// the list's (index-sorted) order, so every sum has a fixed order; the 48 sums stay in
// registers and are rotated into the atom's local frame at the end
__global__ void __launch_bounds__(128) k_mts_desc(int n, const int* __restrict__ fstart, const int* __restrict__ fcount,
                                                  const int* __restrict__ flist, const float4* __restrict__ xf,
                                                  const float* __restrict__ frame, const float* __restrict__ fc,
                                                  const float* __restrict__ scal, __nv_bfloat16* __restrict__ X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 pi = xf[i];
  float v[6 * NRAD];
#pragma unroll
  for (int k = 0; k < 6 * NRAD; ++k) v[k] = 0.f;
  const float rc2 = RCUT_DESC * RCUT_DESC;
  const float dmu = (RCUT_DESC - GAUSS_MU0) / (float)(NRAD - 1), c2 = 1.0f / (2.0f * GAUSS_W * GAUSS_W);
  const float rw = 1.0f / GAUSS_W;
  const float gam = __expf(-2.0f * dmu * dmu * c2);
  const float qi = pi.w;
  const int st = fstart[i], cnt = fcount[i];
  // four entries at a time: their indices, then their positions, are loaded before
  // any is used (independent loads in flight)
  for (int m0 = 0; m0 < cnt; m0 += 4) {
    int jj[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) jj[u] = m0 + u < cnt ? flist[st + m0 + u] : i;
    float4 pp[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) pp[u] = xf[jj[u]];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float rx = pp[u].x - pi.x, ry = pp[u].y - pi.y, rz = pp[u].z - pi.z;
      const float r2 = rx * rx + ry * ry + rz * rz;
      if (!(r2 < rc2 && r2 > 0.f)) continue;  // the padding entries (j = i) have r2 = 0
      const float rinv = rsqrtf(r2), r = r2 * rinv;
      const float wt = qi * pp[u].w * 0.5f * (1.0f + __cosf(3.14159265f * r * (1.0f / RCUT_DESC)));
      const float hx = rx * rinv, hy = ry * rinv, hz = rz * rinv;
      // g_k = exp(-(r - mu_k)^2 c2) by recurrence over the equally spaced centres:
      // g_{k+1} = g_k rho_k, rho_{k+1} = rho_k gam (two exponentials per pair, not NRAD)
      const float t0 = r - GAUSS_MU0;
      float gk = wt * __expf(-t0 * t0 * c2);
      float rho = __expf((2.0f * t0 * dmu - dmu * dmu) * c2);
#pragma unroll
      for (int k = 0; k < NRAD; ++k) {
        const float t = r - (GAUSS_MU0 + dmu * (float)k);
        const float hk = gk * t * rw;  // the first Hermite function of the same Gaussian
        v[6 * k + 0] = fmaf(gk, hx, v[6 * k + 0]);
        v[6 * k + 1] = fmaf(gk, hy, v[6 * k + 1]);
        v[6 * k + 2] = fmaf(gk, hz, v[6 * k + 2]);
        v[6 * k + 3] = fmaf(hk, hx, v[6 * k + 3]);
        v[6 * k + 4] = fmaf(hk, hy, v[6 * k + 4]);
        v[6 * k + 5] = fmaf(hk, hz, v[6 * k + 5]);
        gk *= rho;
        rho *= gam;
      }
    }
  }
  // triple 2k holds A_k, triple 2k + 1 holds A'_k; each goes out in the local frame,
  // then C_i
  float e[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) e[k] = frame[9 * (size_t)i + k];
  __nv_bfloat16* xo = X + (size_t)i * KIN;
#pragma unroll
  for (int t = 0; t < 2 * NRAD; ++t) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float val = e[3 * c] * v[3 * t] + e[3 * c + 1] * v[3 * t + 1] + e[3 * c + 2] * v[3 * t + 2];
      xo[3 * t + c] = __float2bfloat16(val * scal[3 * t + c]);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float val = e[3 * c] * fc[3 * i] + e[3 * c + 1] * fc[3 * i + 1] + e[3 * c + 2] * fc[3 * i + 2];
    xo[6 * NRAD + c] = __float2bfloat16(val * scal[6 * NRAD + c]);
  }
  for (int c = NIN; c < KIN; ++c) xo[c] = __float2bfloat16(0.f);
}

// ------------------------------------------------------------ inference (mma)
struct InferSmem {
  __nv_bfloat16 w1t[NH * LDX];
  __nv_bfloat16 w2t[NH * LDH];
  __nv_bfloat16 w3t[NOUTP * LDH];
  float bias[NH + NH + NOUTP];
  __nv_bfloat16 xin[TILE_I * LDX];
  __nv_bfloat16 act[TILE_I * LDH];
  float yo[TILE_I * NOUTP];
};

// one dense layer for a warp's 16 rows: out = act(in W + b)
template <int K, int N, bool SILU>
__device__ __forceinline__ void mlp_layer(const __nv_bfloat16* in, int ldin, const __nv_bfloat16* wt, int ldw,
                                          const float* bias, __nv_bfloat16* out, int ldout, float* yout) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  unsigned a[K / 16][4];
#pragma unroll
  for (int ks = 0; ks < K / 16; ++ks) {
    const int k0 = ks * 16 + 2 * t;
    a[ks][0] = ld2(in + g * ldin + k0);
    a[ks][1] = ld2(in + (g + 8) * ldin + k0);
    a[ks][2] = ld2(in + g * ldin + k0 + 8);
    a[ks][3] = ld2(in + (g + 8) * ldin + k0 + 8);
  }
  __syncwarp();
#pragma unroll 4
  for (int nt = 0; nt < N / 8; ++nt) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const __nv_bfloat16* wrow = wt + (nt * 8 + g) * ldw + 2 * t;
#pragma unroll
    for (int ks = 0; ks < K / 16; ++ks) mma_bf16(d, a[ks], ld2(wrow + ks * 16), ld2(wrow + ks * 16 + 8));
    const int c0 = nt * 8 + 2 * t;
    float v0 = d[0] + bias[c0], v1 = d[1] + bias[c0 + 1], v2 = d[2] + bias[c0], v3 = d[3] + bias[c0 + 1];
    if (SILU) { v0 = silu(v0); v1 = silu(v1); v2 = silu(v2); v3 = silu(v3); }
    if (out) {
      *reinterpret_cast<__nv_bfloat162*>(out + g * ldout + c0) = __floats2bfloat162_rn(v0, v1);
      *reinterpret_cast<__nv_bfloat162*>(out + (g + 8) * ldout + c0) = __floats2bfloat162_rn(v2, v3);
    } else {
      yout[g * NOUTP + c0] = v0; yout[g * NOUTP + c0 + 1] = v1;
      yout[(g + 8) * NOUTP + c0] = v2; yout[(g + 8) * NOUTP + c0 + 1] = v3;
    }
  }
  __syncwarp();
}

// persistent: each CTA stages the weights once and walks tiles of TILE_I = 256 atoms.
// out = base + fs * R^T y (lab frame)
__global__ void __launch_bounds__(INFER_NT) k_mlp_infer(int n, const __nv_bfloat16* __restrict__ X, Net net,
                                                   const float* __restrict__ base, const float* __restrict__ frame,
                                                   const float* __restrict__ scal, float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
  for (int e = threadIdx.x; e < NH * (KIN / 2); e += blockDim.x) {
    const int r = e / (KIN / 2), c = e % (KIN / 2);
    reinterpret_cast<unsigned*>(S.w1t + r * LDX)[c] = reinterpret_cast<const unsigned*>(net.w1t + r * KIN)[c];
  }
  for (int e = threadIdx.x; e < NH * (NH / 2); e += blockDim.x) {
    const int r = e / (NH / 2), c = e % (NH / 2);
    reinterpret_cast<unsigned*>(S.w2t + r * LDH)[c] = reinterpret_cast<const unsigned*>(net.w2t + r * NH)[c];
  }
  for (int e = threadIdx.x; e < NOUTP * (NH / 2); e += blockDim.x) {
    const int r = e / (NH / 2), c = e % (NH / 2);
    reinterpret_cast<unsigned*>(S.w3t + r * LDH)[c] = reinterpret_cast<const unsigned*>(net.w3t + r * NH)[c];
  }
  for (int e = threadIdx.x; e < NH + NH + NOUTP; e += blockDim.x) S.bias[e] = net.bias[e];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float fs = scal[NIN];
  const int ntiles = (n + TILE_I - 1) / TILE_I;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int a0 = tile * TILE_I;
    __syncthreads();  // weights staged; the previous tile's rows are consumed
    for (int e = threadIdx.x; e < TILE_I * (KIN / 8); e += blockDim.x) {
      const int r = e / (KIN / 8), c = e % (KIN / 8);
      uint4 v = make_uint4(0, 0, 0, 0);
      if (a0 + r < n) v = reinterpret_cast<const uint4*>(X + (size_t)(a0 + r) * KIN)[c];
      reinterpret_cast<uint4*>(S.xin + r * LDX)[c] = v;
    }
    __syncthreads();
    __nv_bfloat16* h = S.act + w * 16 * LDH;
    mlp_layer<KIN, NH, true>(S.xin + w * 16 * LDX, LDX, S.w1t, LDX, S.bias, h, LDH, nullptr);
    mlp_layer<NH, NH, true>(h, LDH, S.w2t, LDH, S.bias + NH, h, LDH, nullptr);
    mlp_layer<NH, NOUTP, false>(h, LDH, S.w3t, LDH, S.bias + 2 * NH, nullptr, 0, S.yo + w * 16 * NOUTP);
    if (lane < 16) {
      const int atom = a0 + w * 16 + lane;
      if (atom < n) {
        const float* yv = S.yo + (w * 16 + lane) * NOUTP;
        const float y0 = yv[0] * fs, y1 = yv[1] * fs, y2 = yv[2] * fs;
        const float* e = frame + 9 * (size_t)atom;
#pragma unroll
        for (int c = 0; c < 3; ++c)
          out[3 * (size_t)atom + c] = base[3 * (size_t)atom + c] + e[c] * y0 + e[3 + c] * y1 + e[6 + c] * y2;
      }
    }
  }
}

// ------------------------------------------------- inference (tcgen05 + TMEM)
// The same network on the fifth-generation tensor cores.  A CTA of eight warps takes
// tiles of 128 atoms (the MMA's M); operands sit in shared memory in the canonical
// K-major layout without swizzle, and each layer's FP32 accumulator sits in tensor
// memory (128 columns).  Warp w reads tensor-memory lanes 32 (w % 4) .. + 31 and half of
// the columns for the bias, SiLU and BF16 rounding that form the next layer's operand.
// One thread issues the MMAs; tcgen05.commit arrives on an mbarrier that the CTA waits on
// with an iteration limit (on expiry the kernel records ST_DEVICE_WAIT, frees its tensor
// memory and returns).  The next tile's inputs are fetched with cp.async while the
// current tile's second and third layers run.
namespace tc {
constexpr int TM = 128;          // atoms per tile (MMA M)
constexpr int NT = 256;          // threads
constexpr int TMEM_COLS = 128;   // FP32 accumulator columns (N of the widest layer)
constexpr int WAIT_LIMIT = 1 << 20;
// shared-memory image (byte offsets); every operand block is 1024-byte aligned
constexpr int S_A = 0;                        // X tile  [128 x 64]  bf16
constexpr int S_H = S_A + TM * KIN * 2;       // hidden  [128 x 128] bf16
constexpr int S_W1 = S_H + TM * NH * 2;       // W1^T    [128 x 64]
constexpr int S_W2 = S_W1 + NH * KIN * 2;     // W2^T    [128 x 128]
constexpr int S_W3 = S_W2 + NH * NH * 2;      // W3^T    [16 x 128]
constexpr int S_BIAS = S_W3 + NOUTP * NH * 2;
constexpr int S_BAR = S_BIAS + (2 * NH + NOUTP) * 4;
constexpr int S_SLOT = S_BAR + 8;
constexpr int SMEM = S_SLOT + 8;
static_assert(S_BAR % 8 == 0, "mbarrier alignment");

// byte offset of element (r, k) of a K-major operand with K columns: 8 x 16-byte core
// matrices, the K-adjacent ones 128 bytes apart (leading-dimension offset), 8-row groups
// K * 16 bytes apart (stride-dimension offset)
__device__ __forceinline__ int core_off(int r, int k, int K) {
  return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading and stride byte offsets (>> 4), the
// fixed version bit 46, base offset 0, no swizzle
__device__ __forceinline__ unsigned long long sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (unsigned long long)((addr & 0x3FFFFu) >> 4) | ((unsigned long long)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((unsigned long long)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, unsigned long long a, unsigned long long b, uint32_t idesc,
                                    uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 bytes global -> shared without a register round trip; src_bytes 0 writes zeros
__device__ __forceinline__ void cp16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's lane
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// a row-major [R][K] BF16 matrix into the canonical K-major layout (asynchronous copies)
__device__ __forceinline__ void stage(uint32_t dst, const __nv_bfloat16* __restrict__ src, int R, int K) {
  const int chunks = K / 8;
  for (int e = threadIdx.x; e < R * chunks; e += blockDim.x) {
    const int r = e / chunks, c = e - r * chunks;
    cp16(dst + core_off(r, 8 * c, K), src + (size_t)r * K + 8 * c, 16u);
  }
}

// the inputs of the tile starting at atom a0: 128 rows of 64 BF16 values (rows past n are zero)
__device__ __forceinline__ void load_tile(uint32_t dst, const __nv_bfloat16* __restrict__ X, int a0, int n) {
  for (int e = threadIdx.x; e < TM * (KIN / 8); e += blockDim.x) {
    const int r = e >> 3, c = e & 7;
    const bool in = a0 + r < n;
    cp16(dst + core_off(r, 8 * c, KIN), in ? X + (size_t)(a0 + r) * KIN + 8 * c : X, in ? 16u : 0u);
  }
  cp_commit();
}

// 32 consecutive FP32 columns of this thread's lane, without waiting for them
__device__ __forceinline__ void ld32_nowait(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

// bias, SiLU and BF16 rounding of 64 accumulator columns [c_lo, c_lo + 64) into the
// hidden operand: both 32-column loads are in flight before the one wait
__device__ __forceinline__ void hidden_epilogue(uint32_t tlane, int c_lo, const float* bias, unsigned char* H,
                                                int row) {
  uint32_t r[2][32];
  ld32_nowait(tlane + (uint32_t)c_lo, r[0]);
  ld32_nowait(tlane + (uint32_t)(c_lo + 32), r[1]);
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int h = 0; h < 2; ++h) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {  // 8 columns: one 16-byte row of a core matrix
      const int c0 = c_lo + 32 * h + 8 * q;
      uint32_t pk[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float v0 = __uint_as_float(r[h][8 * q + 2 * k]), v1 = __uint_as_float(r[h][8 * q + 2 * k + 1]);
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(silu(v0 + bias[c0 + 2 * k]), silu(v1 + bias[c0 + 2 * k + 1]));
        pk[k] = *reinterpret_cast<const uint32_t*>(&b2);
      }
      *reinterpret_cast<uint4*>(H + core_off(row, c0, NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
  }
}
}  // namespace tc

// persistent: each CTA stages the weights once and walks tiles of 128 atoms;
// out = base + fs * R^T y (lab frame), as k_mlp_infer
__global__ void __launch_bounds__(tc::NT) k_mlp_infer_tc(int n, const __nv_bfloat16* __restrict__ X, Net net,
                                                         const float* __restrict__ base,
                                                         const float* __restrict__ frame,
                                                         const float* __restrict__ scal, float* __restrict__ out,
                                                         int* status) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char sm[];
  const int w = threadIdx.x >> 5;
  const int row = 32 * (w & 3) + (threadIdx.x & 31);  // tensor-memory lane = atom row of the tile
  const int half = w >> 2;                            // column half of the hidden layers
  float* bias = reinterpret_cast<float*>(sm + S_BIAS);
  const uint32_t bar = smem_addr(sm + S_BAR);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + S_SLOT);
  const uint32_t aA = smem_addr(sm + S_A), aH = smem_addr(sm + S_H);
  const uint32_t aW1 = smem_addr(sm + S_W1), aW2 = smem_addr(sm + S_W2), aW3 = smem_addr(sm + S_W3);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  stage(aW1, net.w1t, NH, KIN);
  stage(aW2, net.w2t, NH, NH);
  stage(aW3, net.w3t, NOUTP, NH);
  cp_commit();
  for (int e = threadIdx.x; e < 2 * NH + NOUTP; e += blockDim.x) bias[e] = net.bias[e];
  const int ntiles = (n + TM - 1) / TM;
  if ((int)blockIdx.x < ntiles) load_tile(aA, X, blockIdx.x * TM, n);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *slot;
  const uint32_t tlane = tmem + ((uint32_t)(32 * (w & 3)) << 16);  // this warp's lanes
  const float fs = scal[NIN];
  uint32_t phase = 0;
  bool ok = true;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int a0 = tile * TM;
#pragma unroll 1
    for (int layer = 0; layer < 3 && ok; ++layer) {
      if (layer == 0) cp_wait_all();  // this thread's copies of the tile (and the weights) landed
      fence_async_smem();             // this thread's operand writes, visible to the tensor core
      fence_before();
      __syncthreads();
      if (threadIdx.x == 0) {
        fence_after();
        const int K = layer == 0 ? KIN : NH;
        const int N = layer == 2 ? NOUTP : NH;
        const uint32_t a = layer == 0 ? aA : aH;
        const uint32_t b = layer == 0 ? aW1 : (layer == 1 ? aW2 : aW3);
        const uint32_t id = idesc_bf16(TM, N);
        for (int s = 0; s < K / 16; ++s)
          mma(tmem, sdesc(a + 256u * s, 128u, (uint32_t)K * 16u), sdesc(b + 256u * s, 128u, (uint32_t)K * 16u), id,
              s > 0 ? 1u : 0u);
        commit(bar);
      }
      const bool done = bar_wait(bar, phase);
      phase ^= 1u;
      if (__syncthreads_or(!done)) {
        ok = false;
        break;
      }
      fence_after();
      if (layer == 0 && tile + (int)gridDim.x < ntiles)
        load_tile(aA, X, (tile + gridDim.x) * TM, n);  // the first layer has read the inputs
      if (layer < 2) {
        hidden_epilogue(tlane, half * (NH / 2), bias + layer * NH, sm + S_H, row);
      } else if (half == 0) {
        float y[16];
        ld16(tlane, y);
        const int atom = a0 + row;
        if (atom < n) {
          const float* bo = bias + 2 * NH;
          const float y0 = (y[0] + bo[0]) * fs, y1 = (y[1] + bo[1]) * fs, y2 = (y[2] + bo[2]) * fs;
          const float* e = frame + 9 * (size_t)atom;
#pragma unroll
          for (int c = 0; c < 3; ++c)
            out[3 * (size_t)atom + c] = base[3 * (size_t)atom + c] + e[c] * y0 + e[3 + c] * y1 + e[6 + c] * y2;
        }
      }
    }
  }
  cp_wait_all();  // no copy in flight when the CTA leaves
  if (!ok && threadIdx.x == 0) atomicOr(status, ST_DEVICE_WAIT);
  fence_before();
  __syncthreads();
  if (w == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ------------------------------------------------------ training (tcgen05 + TMEM)
// Forward, MSE and backward of one tile of 128 atoms of the batch on the tensor cores:
// the eight products of a training step,
//   forward   Z1 = X W1, Z2 = H1 W2, Y = H2 W3                       (M = atoms)
//   backward  dZ2' = dY W3^T, dZ1' = dZ2 W2^T                         (M = atoms)
//             dW3 = H2^T dY, dW2^T = dZ2^T H1, dW1^T = dZ1^T X       (M = hidden units)
// with BF16 operands (the rounding points of k_mlp_train: inputs, weights, activations and
// activation gradients) and FP32 accumulators in tensor memory, 512 columns:
//   Z1 [0,128)  Z2 [128,256)  Y [256,272)  dW3 [272,288)  dZ2' [384,512)
//   then dZ1' [128,256)  dW2^T [256,384)  dW1^T [384,448)  as the earlier ones are read.
// Every operand is K-major in shared memory: the epilogues write each activation (and
// activation gradient) both as [atoms][units] and transposed as [units][atoms], so the
// weight-gradient products contract over the atoms with the same descriptors as the
// forward ones.  One thread issues each phase's MMAs and commits them to an mbarrier;
// every wait has an iteration limit (ST_DEVICE_WAIT, tensor memory freed, no copy in
// flight).  Per-CTA gradient partials go to gpart as in k_mlp_train (fixed-order sum in
// k_grad_reduce), so a step is deterministic.

namespace tct {
using tc::core_off;
using tc::sdesc;
using tc::smem_addr;
constexpr int TM = 128, NT = 256, TMEM_COLS = 512;
// shared-memory image (byte offsets, operand blocks 4096-aligned)
constexpr int S_X = 0;                  // X [128][64]; after the first product: dY [128][16], dY^T [16][128]
constexpr int S_DY = S_X, S_DYT = S_X + TM * NOUTP * 2;
constexpr int S_XT = S_X + TM * KIN * 2;  // X^T [64][128]
constexpr int S_H1 = S_XT + KIN * TM * 2; // H1 [128][128]; later dZ2 [128][128]
constexpr int S_H1T = S_H1 + TM * NH * 2; // H1^T
constexpr int S_H2 = S_H1T + NH * TM * 2; // H2; later dZ2^T
constexpr int S_H2T = S_H2 + TM * NH * 2; // H2^T; later dZ1^T
constexpr int S_W = S_H2T + NH * TM * 2;  // W1^T [128][64] and W2^T [128][128]; later W2 [128][128], W3 [128][16]
constexpr int S_W1T = S_W, S_W2T = S_W + NH * KIN * 2;
constexpr int S_W2B = S_W, S_W3B = S_W + NH * NH * 2;
constexpr int S_W3T = S_W + NH * KIN * 2 + NH * NH * 2;  // W3^T [16][128]
constexpr int S_BIAS = S_W3T + NOUTP * NH * 2;
constexpr int S_RED = S_BIAS + (2 * NH + NOUTP) * 4;     // per-row squared errors
constexpr int S_BAR = S_RED + TM * 4;
constexpr int S_SLOT = S_BAR + 8;
constexpr int SMEM = S_SLOT + 8;
static_assert(S_BAR % 8 == 0, "mbarrier alignment");
static_assert(S_W3B + NH * NOUTP * 2 <= S_W3T, "backward weights fit the forward ones' space");
static_assert(SMEM <= 227 * 1024, "training tile exceeds shared memory");
constexpr uint32_t C_Z1 = 0, C_Z2 = 128, C_Y = 256, C_DW3 = 272, C_DZ2P = 384, C_DZ1P = 128, C_DW2 = 256,
                   C_DW1 = 384;

// K-steps of 16 of an M x N product with both operands K-major (K columns each)
__device__ __forceinline__ void mma_k(uint32_t d, uint32_t a, uint32_t b, int K, int N) {
  const uint32_t id = tc::idesc_bf16(TM, N);
  for (int s = 0; s < K / 16; ++s)
    tc::mma(d, sdesc(a + 256u * s, 128u, (uint32_t)K * 16u), sdesc(b + 256u * s, 128u, (uint32_t)K * 16u), id,
            s > 0 ? 1u : 0u);
}

// 2-byte store of one BF16 value into a K-major [R][K] operand at (r, k)
__device__ __forceinline__ void st_bf(unsigned char* base, int r, int k, int K, float v) {
  *reinterpret_cast<__nv_bfloat16*>(base + core_off(r, k, K)) = __float2bfloat16(v);
}
__device__ __forceinline__ float ld_bf(const unsigned char* base, int r, int k, int K) {
  return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(base + core_off(r, k, K)));
}

// 32 columns of this thread's lane
__device__ __forceinline__ void ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  tc::ld32_nowait(taddr, r);
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// bias, SiLU and BF16 rounding of this thread's 64 columns of a hidden layer: the row of
// H (K-major, 16-byte stores) and the column of H^T
__device__ __forceinline__ void act_epilogue(uint32_t tl, int c_lo, const float* bias, unsigned char* H,
                                             unsigned char* HT, int row) {
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    float v[32];
    ld32(tl + (uint32_t)(c_lo + 32 * h), v);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c0 = c_lo + 32 * h + 8 * q;
      uint32_t pk[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(silu(v[8 * q + 2 * k] + bias[c0 + 2 * k]),
                                                        silu(v[8 * q + 2 * k + 1] + bias[c0 + 2 * k + 1]));
        pk[k] = *reinterpret_cast<const uint32_t*>(&b2);
        *reinterpret_cast<__nv_bfloat16*>(HT + core_off(c0 + 2 * k, row, TM)) = b2.x;
        *reinterpret_cast<__nv_bfloat16*>(HT + core_off(c0 + 2 * k + 1, row, TM)) = b2.y;
      }
      *reinterpret_cast<uint4*>(H + core_off(row, c0, NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
  }
}

// dZ = BF16(dZ' * silu'(Z + b)) for this thread's 64 columns: into D ([atoms][units],
// when given) and DT ([units][atoms])
__device__ __forceinline__ void grad_epilogue(uint32_t tl, uint32_t c_pre, uint32_t c_z, int c_lo,
                                              const float* bias, unsigned char* D, unsigned char* DT, int row) {
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    float pv[32], zv[32];
    ld32(tl + c_pre + (uint32_t)(c_lo + 32 * h), pv);
    ld32(tl + c_z + (uint32_t)(c_lo + 32 * h), zv);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c0 = c_lo + 32 * h + 8 * q;
      uint32_t pk[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int e = 8 * q + 2 * k;
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(pv[e] * dsilu(zv[e] + bias[c0 + 2 * k]),
                                                        pv[e + 1] * dsilu(zv[e + 1] + bias[c0 + 2 * k + 1]));
        pk[k] = *reinterpret_cast<const uint32_t*>(&b2);
        *reinterpret_cast<__nv_bfloat16*>(DT + core_off(c0 + 2 * k, row, TM)) = b2.x;
        *reinterpret_cast<__nv_bfloat16*>(DT + core_off(c0 + 2 * k + 1, row, TM)) = b2.y;
      }
      if (D) *reinterpret_cast<uint4*>(D + core_off(row, c0, NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
  }
}

// sum over the 128 atoms of row u of a [units][atoms] operand, in atom order
__device__ __forceinline__ float row_sum(const unsigned char* T, int u) {
  float s = 0.f;
  for (int r = 0; r < TM; ++r) s += ld_bf(T, u, r, TM);
  return s;
}
}  // namespace tct

// BF16 operand copies of the master weights for the tensor-core training kernel
__global__ void k_train_weights(const float* __restrict__ w, TrainW t) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < NH * KIN) {
    const int o = e / KIN, k = e % KIN;
    t.w1t[e] = __float2bfloat16(k < NIN ? w[OFF_W1 + k * NH + o] : 0.f);
  }
  if (e < NH * NH) {
    const int o = e / NH, k = e % NH;
    t.w2t[e] = __float2bfloat16(w[OFF_W2 + k * NH + o]);  // [out][in]
    t.w2b[e] = __float2bfloat16(w[OFF_W2 + e]);           // [in][out]
  }
  if (e < NOUTP * NH) {
    const int o = e / NH, k = e % NH;
    t.w3t[e] = __float2bfloat16(o < NOUT ? w[OFF_W3 + k * NOUT + o] : 0.f);
    const int i = e / NOUTP, c = e % NOUTP;
    t.w3b[e] = __float2bfloat16(c < NOUT ? w[OFF_W3 + i * NOUT + c] : 0.f);  // [in][out padded]
  }
  if (e < NH) { t.bias[e] = w[OFF_B1 + e]; t.bias[NH + e] = w[OFF_B2 + e]; }
  if (e < NOUTP) t.bias[2 * NH + e] = e < NOUT ? w[OFF_B3 + e] : 0.f;
}

__global__ void __launch_bounds__(tct::NT, 1) k_mlp_train_tc(int nb, const int* __restrict__ idx,
                                                            const __nv_bfloat16* __restrict__ X,
                                                            const float* __restrict__ target, TrainW tw,
                                                            float inv_count, float* __restrict__ gpart,
                                                            float* __restrict__ loss_part, float* __restrict__ yout,
                                                            int* status) {
  using namespace tct;
  extern __shared__ __align__(1024) unsigned char sm[];
  const int w = threadIdx.x >> 5, tid = threadIdx.x;
  const int row = 32 * (w & 3) + (threadIdx.x & 31);  // tensor-memory lane
  const int half = w >> 2;
  float* bias = reinterpret_cast<float*>(sm + S_BIAS);
  float* red = reinterpret_cast<float*>(sm + S_RED);
  const uint32_t bar = smem_addr(sm + S_BAR);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + S_SLOT);
  const uint32_t base = smem_addr(sm);
  const int a0 = blockIdx.x * TM;
  float* gp = gpart + (size_t)blockIdx.x * NPARAM;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::stage(base + S_W1T, tw.w1t, NH, KIN);
  tc::stage(base + S_W2T, tw.w2t, NH, NH);
  tc::stage(base + S_W3T, tw.w3t, NOUTP, NH);
  for (int e = tid; e < TM * (KIN / 8); e += NT) {  // the tile's input rows, gathered by idx
    const int r = e >> 3, c = e & 7;
    const bool in = a0 + r < nb;
    tc::cp16(base + S_X + core_off(r, 8 * c, KIN), in ? X + (size_t)idx[a0 + r] * KIN + 8 * c : X, in ? 16u : 0u);
  }
  tc::cp_commit();
  for (int e = tid; e < 2 * NH + NOUTP; e += NT) bias[e] = tw.bias[e];
  tc::cp_wait_all();
  __syncthreads();
  for (int e = tid; e < KIN * TM; e += NT) {  // X^T for the last product
    const int k = e / TM, r = e % TM;
    *reinterpret_cast<__nv_bfloat16*>(sm + S_XT + core_off(k, r, TM)) =
        *reinterpret_cast<const __nv_bfloat16*>(sm + S_X + core_off(r, k, KIN));
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *slot;
  const uint32_t tl = tmem + ((uint32_t)(32 * (w & 3)) << 16);
  uint32_t phase = 0;
  bool ok = true;
  // one phase: operand writes visible to the tensor core, MMAs by one thread, the wait
  auto run = [&](int which) -> bool {
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      switch (which) {
        case 0: mma_k(tmem + C_Z1, base + S_X, base + S_W1T, KIN, NH); break;
        case 1: mma_k(tmem + C_Z2, base + S_H1, base + S_W2T, NH, NH); break;
        case 2: mma_k(tmem + C_Y, base + S_H2, base + S_W3T, NH, NOUTP); break;
        case 3:
          mma_k(tmem + C_DZ2P, base + S_DY, base + S_W3B, NOUTP, NH);
          mma_k(tmem + C_DW3, base + S_H2T, base + S_DYT, TM, NOUTP);
          break;
        case 4:
          mma_k(tmem + C_DZ1P, base + S_H1, base + S_W2B, NH, NH);   // dZ2 sits where H1 was
          mma_k(tmem + C_DW2, base + S_H2, base + S_H1T, TM, NH);    // dZ2^T where H2 was
          break;
        default: mma_k(tmem + C_DW1, base + S_H2T, base + S_XT, TM, KIN); break;  // dZ1^T where H2^T was
      }
      tc::commit(bar);
    }
    const bool done = tc::bar_wait(bar, phase);
    phase ^= 1u;
    if (__syncthreads_or(!done)) return false;
    tc::fence_after();
    return true;
  };
  const int c_lo = half * (NH / 2);
  // forward
  ok = run(0);
  if (ok) act_epilogue(tl + C_Z1, c_lo, bias, sm + S_H1, sm + S_H1T, row);
  if (ok) ok = run(1);
  if (ok) {
    tc::stage(base + S_W2B, tw.w2b, NH, NH);  // the forward weights W1^T, W2^T are read
    tc::stage(base + S_W3B, tw.w3b, NH, NOUTP);
    tc::cp_commit();
    act_epilogue(tl + C_Z2, c_lo, bias + NH, sm + S_H2, sm + S_H2T, row);
  }
  if (ok) ok = run(2);
  if (ok) {
    // output, loss and dY = BF16(2 (y - t) / count) (rows past the batch: zero)
    if (half == 0) {
      float y[16];
      tc::ld16(tl + C_Y, y);
      const int atom = a0 + row;
      float dy[NOUT] = {0.f, 0.f, 0.f}, l = 0.f;
      if (atom < nb) {
#pragma unroll
        for (int c = 0; c < NOUT; ++c) {
          const float yc = y[c] + bias[2 * NH + c];
          const float d = yc - target[3 * (size_t)idx[atom] + c];
          if (yout) yout[3 * (size_t)atom + c] = yc;
          dy[c] = 2.0f * d * inv_count;
          l += d * d;
        }
      }
      red[row] = l;
      for (int c = 0; c < NOUTP; ++c) {
        const float v = c < NOUT ? dy[c] : 0.f;
        st_bf(sm + S_DY, row, c, NOUTP, v);
        st_bf(sm + S_DYT, c, row, TM, v);
      }
    }
    tc::cp_wait_all();  // the backward weights landed
  }
  if (ok) ok = run(3);
  if (ok) {
    if (tid == 0) {
      float l = 0.f;
      for (int r = 0; r < TM; ++r) l += red[r];
      loss_part[blockIdx.x] = l * inv_count;
    }
    if (tid < NOUT) gp[OFF_B3 + tid] = row_sum(sm + S_DYT, tid);
    if (half == 0) {  // dW3 [hidden][out]
      float v[16];
      tc::ld16(tl + C_DW3, v);
#pragma unroll
      for (int c = 0; c < NOUT; ++c) gp[OFF_W3 + row * NOUT + c] = v[c];
    }
    // dZ2 over H1 ([atoms][units]) and H2 (transposed): both read by the last phase
    grad_epilogue(tl, C_DZ2P, C_Z2, c_lo, bias + NH, sm + S_H1, sm + S_H2, row);
  }
  if (ok) ok = run(4);
  if (ok) {
    if (tid < NH) gp[OFF_B2 + tid] = row_sum(sm + S_H2, tid);
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {  // dW2^T [out][in] -> W2[in][out]
      float v[32];
      ld32(tl + C_DW2 + (uint32_t)(c_lo + 32 * h), v);
#pragma unroll
      for (int k = 0; k < 32; ++k) gp[OFF_W2 + (size_t)(c_lo + 32 * h + k) * NH + row] = v[k];
    }
    grad_epilogue(tl, C_DZ1P, C_Z1, c_lo, bias, nullptr, sm + S_H2T, row);  // dZ1^T over H2^T
  }
  if (ok) ok = run(5);
  if (ok) {
    if (tid < NH) gp[OFF_B1 + tid] = row_sum(sm + S_H2T, tid);
    float v[32];  // dW1^T [hidden][in] -> W1[in][hidden]
    ld32(tl + C_DW1 + (uint32_t)(32 * half), v);
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      const int in = 32 * half + k;
      if (in < NIN) gp[OFF_W1 + (size_t)in * NH + row] = v[k];
    }
  }
  tc::cp_wait_all();  // no copy in flight when the CTA leaves
  if (!ok && tid == 0) atomicOr(status, ST_DEVICE_WAIT);
  tc::fence_before();
  __syncthreads();
  if (w == 0) {
    tc::fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ------------------------------------------------------------- training
// forward + MSE + backward of TILE_T atoms; per-CTA gradient partial in gpart.
// Row strides NH+1 keep the column walks of the backward pass conflict-free.
struct TrainSmem {
  float W1[NIN][NH];
  float W2[NH][NH + 1];
  float W3[NH][NOUT];
  float b1[NH], b2[NH], b3[4];
  float x[TILE_T][NIN];
  float z1[TILE_T][NH + 1], h1[TILE_T][NH + 1];
  float z2[TILE_T][NH + 1], h2[TILE_T][NH + 1];
  float dy[TILE_T][NOUT];
  float sq[TILE_T][NOUT];
};

__global__ void __launch_bounds__(256) k_mlp_train(int nb, const int* __restrict__ idx, const __nv_bfloat16* __restrict__ X,
                                                   const float* __restrict__ target, const float* __restrict__ master,
                                                   float inv_count, float* __restrict__ gpart,
                                                   float* __restrict__ loss_part, float* __restrict__ yout) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < NIN * NH; e += nt) S.W1[e / NH][e % NH] = bfr(master[OFF_W1 + e]);
  for (int e = tid; e < NH * NH; e += nt) S.W2[e / NH][e % NH] = bfr(master[OFF_W2 + e]);
  for (int e = tid; e < NH * NOUT; e += nt) S.W3[e / NOUT][e % NOUT] = bfr(master[OFF_W3 + e]);
  for (int e = tid; e < NH; e += nt) { S.b1[e] = master[OFF_B1 + e]; S.b2[e] = master[OFF_B2 + e]; }
  if (tid < NOUT) S.b3[tid] = master[OFF_B3 + tid];
  const int r0 = blockIdx.x * TILE_T;
  for (int e = tid; e < TILE_T * NIN; e += nt) {
    const int r = e / NIN, c = e % NIN;
    S.x[r][c] = r0 + r < nb ? __bfloat162float(X[(size_t)idx[r0 + r] * KIN + c]) : 0.f;
  }
  __syncthreads();
  for (int e = tid; e < TILE_T * NH; e += nt) {
    const int r = e / NH, c = e % NH;
    float s = S.b1[c];
    for (int k = 0; k < NIN; ++k) s = fmaf(S.x[r][k], S.W1[k][c], s);
    S.z1[r][c] = s;
    S.h1[r][c] = bfr(silu(s));
  }
  __syncthreads();
  for (int e = tid; e < TILE_T * NH; e += nt) {
    const int r = e / NH, c = e % NH;
    float s = S.b2[c];
    for (int k = 0; k < NH; ++k) s = fmaf(S.h1[r][k], S.W2[k][c], s);
    S.z2[r][c] = s;
    S.h2[r][c] = bfr(silu(s));
  }
  __syncthreads();
  if (tid < TILE_T * NOUT) {
    const int r = tid / NOUT, c = tid % NOUT;
    float s = S.b3[c];
    for (int k = 0; k < NH; ++k) s = fmaf(S.h2[r][k], S.W3[k][c], s);
    float d = 0.f;
    if (r0 + r < nb) {
      d = s - target[3 * (size_t)idx[r0 + r] + c];
      if (yout) yout[3 * (size_t)(r0 + r) + c] = s;
    }
    S.dy[r][c] = bfr(2.0f * d * inv_count);
    S.sq[r][c] = d * d;
  }
  __syncthreads();
  if (tid == 0) {
    float l = 0.f;
    for (int r = 0; r < TILE_T; ++r)
      for (int c = 0; c < NOUT; ++c) l += S.sq[r][c];
    loss_part[blockIdx.x] = l * inv_count;
  }
  float* gp = gpart + (size_t)blockIdx.x * NPARAM;
  for (int e = tid; e < NH * NOUT; e += nt) {
    const int k = e / NOUT, c = e % NOUT;
    float s = 0.f;
    for (int r = 0; r < TILE_T; ++r) s = fmaf(S.h2[r][k], S.dy[r][c], s);
    gp[OFF_W3 + e] = s;
  }
  if (tid < NOUT) {
    float s = 0.f;
    for (int r = 0; r < TILE_T; ++r) s += S.dy[r][tid];
    gp[OFF_B3 + tid] = s;
  }
  // dZ2 = (dY W3^T) . silu'(z2), stored over z2
  for (int e = tid; e < TILE_T * NH; e += nt) {
    const int r = e / NH, k = e % NH;
    float s = 0.f;
    for (int c = 0; c < NOUT; ++c) s = fmaf(S.dy[r][c], S.W3[k][c], s);
    S.z2[r][k] = bfr(s * dsilu(S.z2[r][k]));
  }
  __syncthreads();
  for (int e = tid; e < NH * NH; e += nt) {
    const int k = e / NH, c = e % NH;
    float s = 0.f;
    for (int r = 0; r < TILE_T; ++r) s = fmaf(S.h1[r][k], S.z2[r][c], s);
    gp[OFF_W2 + e] = s;
  }
  for (int c = tid; c < NH; c += nt) {
    float s = 0.f;
    for (int r = 0; r < TILE_T; ++r) s += S.z2[r][c];
    gp[OFF_B2 + c] = s;
  }
  // dZ1 = (dZ2 W2^T) . silu'(z1), stored over z1
  for (int e = tid; e < TILE_T * NH; e += nt) {
    const int r = e / NH, k = e % NH;
    float s = 0.f;
    for (int c = 0; c < NH; ++c) s = fmaf(S.z2[r][c], S.W2[k][c], s);
    S.z1[r][k] = bfr(s * dsilu(S.z1[r][k]));
  }
  __syncthreads();
  for (int e = tid; e < NIN * NH; e += nt) {
    const int k = e / NH, c = e % NH;
    float s = 0.f;
    for (int r = 0; r < TILE_T; ++r) s = fmaf(S.x[r][k], S.z1[r][c], s);
    gp[OFF_W1 + e] = s;
  }
  for (int c = tid; c < NH; c += nt) {
    float s = 0.f;
    for (int r = 0; r < TILE_T; ++r) s += S.z1[r][c];
    gp[OFF_B1 + c] = s;
  }
}

// fixed-order sum of the per-CTA partials
__global__ void k_grad_reduce(int ntiles, const float* __restrict__ gpart, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  float s = 0.f;
  for (int t = 0; t < ntiles; ++t) s += gpart[(size_t)t * NPARAM + p];
  grad[p] = s;
}

__global__ void k_adam(float* __restrict__ w, float* __restrict__ m1, float* __restrict__ m2,
                       const float* __restrict__ gr, float lr, float b1, float b2, float c1, float c2, float eps) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  const float gv = gr[p];
  const float a = b1 * m1[p] + (1.0f - b1) * gv;
  const float b = b2 * m2[p] + (1.0f - b2) * gv * gv;
  m1[p] = a;
  m2[p] = b;
  w[p] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// BF16 [out][in] copies for the inference kernel
__global__ void k_publish(const float* __restrict__ w, Net net) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < NH * KIN) {
    const int o = e / KIN, k = e % KIN;
    net.w1t[e] = __float2bfloat16(k < NIN ? w[OFF_W1 + k * NH + o] : 0.f);
  }
  if (e < NH * NH) {
    const int o = e / NH, k = e % NH;
    net.w2t[e] = __float2bfloat16(w[OFF_W2 + k * NH + o]);
  }
  if (e < NOUTP * NH) {
    const int o = e / NH, k = e % NH;
    net.w3t[e] = __float2bfloat16(o < NOUT ? w[OFF_W3 + k * NOUT + o] : 0.f);
  }
  if (e < NH) { net.bias[e] = w[OFF_B1 + e]; net.bias[NH + e] = w[OFF_B2 + e]; }
  if (e < NOUTP) net.bias[2 * NH + e] = e < NOUT ? w[OFF_B3 + e] : 0.f;
}

// labels: R (frec - fc) / fs, the coarse grid's error in the local frame
__global__ void k_mts_target(int n, const float* __restrict__ frec, const float* __restrict__ fc,
                             const float* __restrict__ frame, const float* __restrict__ scal,
                             float* __restrict__ target) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float inv = 1.0f / scal[NIN];
  float d[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) d[c] = frec[3 * i + c] - fc[3 * i + c];
  const float* e = frame + 9 * (size_t)i;
#pragma unroll
  for (int c = 0; c < 3; ++c) target[3 * i + c] = (e[3 * c] * d[0] + e[3 * c + 1] * d[1] + e[3 * c + 2] * d[2]) * inv;
}

// per-block squared errors against the SPME forces f of this step: [S with the mean
// of its network correction (net[]/n) removed, the coarse force alone, the stale force f0]
__global__ void k_err3(int n, const float* __restrict__ pred, const float* __restrict__ fc,
                       const double* __restrict__ net, float rn, const float* __restrict__ f0,
                       const float* __restrict__ f, double* blk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float v[3] = {0.f, 0.f, 0.f};
  if (i < n) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float t = f[3 * i + k];
      const float a = pred[3 * i + k] - (float)net[k] * rn - t, b = fc[3 * i + k] - t, c = f0[3 * i + k] - t;
      v[0] = fmaf(a, a, v[0]);
      v[1] = fmaf(b, b, v[1]);
      v[2] = fmaf(c, c, v[2]);
    }
  }
  block_reduce_store<3>(v, blk);
}

// per-block sum of squares of a 3n array
__global__ void k_sumsq(int n, const float* __restrict__ a, double* blk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float v[1] = {0.f};
  if (i < n) v[0] = a[3 * i] * a[3 * i] + a[3 * i + 1] * a[3 * i + 1] + a[3 * i + 2] * a[3 * i + 2];
  block_reduce_store<1>(v, blk);
}

// per-block sum of |F|^2 of the FP64 total forces
__global__ void k_fsq(int n, const double* __restrict__ fx, const double* __restrict__ fy,
                      const double* __restrict__ fz, double* blk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float v[1] = {0.f};
  if (i < n) {
    const float a = (float)fx[i], b = (float)fy[i], c = (float)fz[i];
    v[0] = a * a + b * b + c * c;
  }
  block_reduce_store<1>(v, blk);
}

// per-block sum of the network corrections f - fc (net force of the correction)
__global__ void k_net3(int n, const float* __restrict__ f, const float* __restrict__ fc, double* blk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float v[3] = {0.f, 0.f, 0.f};
  if (i < n) {
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = f[3 * i + k] - fc[3 * i + k];
  }
  block_reduce_store<3>(v, blk);
}

// inner step: S = f with the mean of the network correction removed, added into the
// fixed-point forces
__global__ void k_mts_apply(int n, float* __restrict__ f, const double* __restrict__ net, float rn,
                            unsigned long long* __restrict__ fixp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float m[3] = {(float)net[0] * rn, (float)net[1] * rn, (float)net[2] * rn};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float fv = f[3 * i + k] - m[k];
    f[3 * i + k] = fv;
    atomicAdd(&fixp[3 * i + k], (unsigned long long)fix40(fv));
  }
}

// cycle-end step: the SPME force is already in the fixed-point forces; add the rest of
// the impulse, (k - 1) (F_SPME - S), S with the mean of its network correction removed
__global__ void k_mts_impulse(int n, const float* __restrict__ frec, const float* __restrict__ pred,
                              const double* __restrict__ net, float rn, float km1,
                              unsigned long long* __restrict__ fixp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float sv = pred[3 * i + k] - (float)net[k] * rn;
    atomicAdd(&fixp[3 * i + k], (unsigned long long)fix40(km1 * (frec[3 * i + k] - sv)));
  }
}

__global__ void k_copy_f(long long n, const float* __restrict__ a, float* __restrict__ b) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

__global__ void k_seq_idx(int nb, int offset, int n, int* idx) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nb) idx[r] = (int)(((long long)offset + r) % n);
}

// per-feature mean square over all atoms (input normalisation)
__global__ void k_feat_ms(int n, const __nv_bfloat16* __restrict__ X, float* __restrict__ out) {
  const int c = blockIdx.x;
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float v = __bfloat162float(X[(size_t)i * KIN + c]);
    s = fmaf(v, v, s);
  }
  __shared__ float red[32];
  s = warp_sumf(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    out[c] = t / (float)n;
  }
}

constexpr size_t infer_smem = sizeof(InferSmem);
constexpr size_t train_smem = sizeof(TrainSmem);
static_assert(6 * NRAD + 3 == NIN, "input layout: 6 radial sums per Gaussian + the coarse force");
static_assert(sizeof(TrainSmem) <= 227 * 1024, "training tile exceeds shared memory");
static_assert(sizeof(InferSmem) <= 227 * 1024, "inference tile exceeds shared memory");

int g_infer_grid = 0;
int g_infer_tc_grid = 0;

void net_alloc(Net& n) {
  GB_CUDA(cudaMalloc(&n.w1t, sizeof(__nv_bfloat16) * NH * KIN));
  GB_CUDA(cudaMalloc(&n.w2t, sizeof(__nv_bfloat16) * NH * NH));
  GB_CUDA(cudaMalloc(&n.w3t, sizeof(__nv_bfloat16) * NOUTP * NH));
  GB_CUDA(cudaMalloc(&n.bias, sizeof(float) * (2 * NH + NOUTP)));
}
void net_free(Net& n) {
  for (void* p : {(void*)n.w1t, (void*)n.w2t, (void*)n.w3t, (void*)n.bias})
    if (p) cudaFree(p);
  n = Net();
}
void train_w_alloc(TrainW& t) {
  GB_CUDA(cudaMalloc(&t.w1t, sizeof(__nv_bfloat16) * NH * KIN));
  GB_CUDA(cudaMalloc(&t.w2t, sizeof(__nv_bfloat16) * NH * NH));
  GB_CUDA(cudaMalloc(&t.w3t, sizeof(__nv_bfloat16) * NOUTP * NH));
  GB_CUDA(cudaMalloc(&t.w2b, sizeof(__nv_bfloat16) * NH * NH));
  GB_CUDA(cudaMalloc(&t.w3b, sizeof(__nv_bfloat16) * NH * NOUTP));
  GB_CUDA(cudaMalloc(&t.bias, sizeof(float) * (2 * NH + NOUTP)));
}
void train_w_free(TrainW& t) {
  for (void* p : {(void*)t.w1t, (void*)t.w2t, (void*)t.w3t, (void*)t.w2b, (void*)t.w3b, (void*)t.bias})
    if (p) cudaFree(p);
  t = TrainW();
}

// GB_MLP_TC=0: the mma.sync inference kernel and the CUDA-core training kernel
bool use_tc() {
  const char* e = getenv("GB_MLP_TC");
  return !(e && e[0] == '0');
}

// forward, loss and backward of nb rows (per-tile gradient partials, their fixed-order
// sum in grad); returns the number of tiles, i.e. of loss partials
int launch_train(int nb, const int* idx, const __nv_bfloat16* X, const float* target, const float* master,
                 TrainW& tw, float* gpart, float* loss_part, float* yout, float* grad) {
  const float inv = 1.0f / (float)(nb * NOUT);
  int nt;
  if (use_tc()) {
    k_train_weights<<<nblocks(NH * NH, 256), 256, 0, g.stream>>>(master, tw);
    GB_LAUNCHED();
    nt = nblocks(nb, tct::TM);
    k_mlp_train_tc<<<nt, tct::NT, tct::SMEM, g.stream>>>(nb, idx, X, target, tw, inv, gpart, loss_part, yout,
                                                         &g.sc->status);
  } else {
    nt = nblocks(nb, TILE_T);
    k_mlp_train<<<nt, 256, train_smem, g.stream>>>(nb, idx, X, target, master, inv, gpart, loss_part, yout);
  }
  GB_LAUNCHED();
  k_grad_reduce<<<nblocks(NPARAM, 256), 256, 0, g.stream>>>(nt, gpart, grad);
  GB_LAUNCHED();
  return nt;
}

void publish(const float* master, Net& net) {
  k_publish<<<nblocks(NH * NH, 256), 256, 0, g.stream>>>(master, net);
  GB_LAUNCHED();
}

void set_attrs() {
  static int dev_done = -1;
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev_done == dev) return;
  GB_CUDA(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_smem));
  GB_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem));
  GB_CUDA(cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tct::SMEM));
  int occ = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mlp_infer, INFER_NT, infer_smem));
  g_infer_grid = std::max(1, occ) * g.nsm;
  GB_CUDA(cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM));
  // the whole carveout as shared memory: two CTAs of 103.5 KB per SM
  GB_CUDA(cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  // resident CTAs per SM from the SM's shared memory and registers (the occupancy query
  // reports one here, while two fit and run)
  cudaDeviceProp prop;
  GB_CUDA(cudaGetDeviceProperties(&prop, dev));
  cudaFuncAttributes fa;
  GB_CUDA(cudaFuncGetAttributes(&fa, k_mlp_infer_tc));
  const int by_smem = (int)(prop.sharedMemPerMultiprocessor / (tc::SMEM + prop.reservedSharedMemPerBlock));
  const int by_regs = prop.regsPerMultiprocessor / (((fa.numRegs + 7) / 8 * 8) * tc::NT);
  // every resident CTA holds TMEM_COLS of the SM's 512 tensor-memory columns
  occ = std::max(1, std::min(std::min(by_smem, by_regs), 512 / tc::TMEM_COLS));
  g_infer_tc_grid = occ * g.nsm;
  dev_done = dev;
}

void launch_infer(int n, const __nv_bfloat16* X, const Net& net, const float* base, const float* frame,
                  const float* scal, float* out) {
  if (use_tc()) {
    const int grid = std::max(1, std::min(g_infer_tc_grid, nblocks(n, tc::TM)));
    k_mlp_infer_tc<<<grid, tc::NT, tc::SMEM, g.stream>>>(n, X, net, base, frame, scal, out, &g.sc->status);
  } else {
    const int grid = std::max(1, std::min(g_infer_grid, nblocks(n, TILE_I)));
    k_mlp_infer<<<grid, INFER_NT, infer_smem, g.stream>>>(n, X, net, base, frame, scal, out);
  }
  GB_LAUNCHED();
}

// deterministic Glorot-uniform weights (splitmix64), zero biases, small output layer
std::vector<float> initial_params() {
  std::vector<float> w(NPARAM, 0.f);
  unsigned long long s = 0x9E3779B97F4A7C15ull;
  auto rnd = [&]() {
    s += 0x9E3779B97F4A7C15ull;
    unsigned long long z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](int off, int fin, int fout, double gain) {
    const double a = gain * std::sqrt(6.0 / (fin + fout));
    for (int k = 0; k < fin * fout; ++k) w[off + k] = (float)((2.0 * rnd() - 1.0) * a);
  };
  fill(OFF_W1, NIN, NH, 1.0);
  fill(OFF_W2, NH, NH, 1.0);
  fill(OFF_W3, NH, NOUT, 0.1);
  return w;
}

void read_scalars(const double* dev, double* host, int nv) {
  GB_CUDA(cudaMemcpyAsync(host, dev, sizeof(double) * nv, cudaMemcpyDeviceToHost, g.stream));
  GB_CUDA(cudaStreamSynchronize(g.stream));
}

// inputs of the current positions relative to t0
// short list of the current half list (positions of this step in xf)
void mts_short_list() {
  const int n = g.natms;
  const float rs = RCUT_DESC + (float)g.p.rpad;
  const float rs2 = rs * rs;
  GB_CUDA(cudaMemsetAsync(M.scount, 0, sizeof(int) * (n + 1), g.stream));
  GB_CUDA(cudaMemsetAsync(M.sfill, 0, sizeof(int) * n, g.stream));
  k_short_count<<<nblocks((long long)n * 32, 256), 256, 0, g.stream>>>(n, g.list, g.ld, g.xf, rs2, M.sown, M.scount);
  GB_LAUNCHED();
  scan_exclusive(M.scount, M.sstart, n + 1);
  int total = 0;
  GB_CUDA(cudaMemcpyAsync(&total, M.sstart + n, sizeof(int), cudaMemcpyDeviceToHost, g.stream));
  GB_CUDA(cudaStreamSynchronize(g.stream));
  if ((long long)total > M.scap) {
    if (M.slist) cudaFree(M.slist);
    if (M.stmp) cudaFree(M.stmp);
    M.scap = (long long)(total * 1.25) + 1024;
    GB_CUDA(cudaMalloc(&M.slist, sizeof(int) * M.scap));
    GB_CUDA(cudaMalloc(&M.stmp, sizeof(int) * M.scap));
  }
  k_short_fill<<<nblocks((long long)n * 32, 256), 256, 0, g.stream>>>(n, g.list, g.ld, g.xf, rs2, M.sstart, M.sown,
                                                                       M.sfill, M.slist);
  GB_LAUNCHED();
  k_short_sort<<<nblocks(n, 8), 256, 0, g.stream>>>(n, M.sstart, M.slist, M.stmp);
  GB_LAUNCHED();
  M.gen_seen = g.list_gen;
}

void mts_inputs() {
  const int n = g.natms;
  prof_begin(P_MTS_DESC);
  if (M.gen_seen != g.list_gen) {
    prof_begin(P_SHORTLIST);
    mts_short_list();
    prof_end(P_SHORTLIST);
  }
  k_mts_prep<<<nblocks(n, 256), 256, 0, g.stream>>>(n, g.x, g.y, g.z, M.triple, g.cell[0], M.frame);
  GB_LAUNCHED();
  k_mts_desc<<<nblocks(n, 128), 128, 0, g.stream>>>(n, M.sstart, M.scount, M.slist, g.xf, M.frame, M.fc, M.scal,
                                                    M.X);
  GB_LAUNCHED();
  prof_end(P_MTS_DESC);
}

void mts_labels() {
  k_mts_target<<<nblocks(g.natms, 256), 256, 0, g.stream>>>(g.natms, M.frec, M.fc, M.frame, M.scal, M.target);
  GB_LAUNCHED();
}

// input and output scales from the first labelled sample
void mts_set_scales() {
  const int n = g.natms;
  std::vector<float> sc(NIN + 1, 1.0f);
  GB_CUDA(cudaMemcpy(M.scal, sc.data(), sizeof(float) * (NIN + 1), cudaMemcpyHostToDevice));
  mts_inputs();
  k_feat_ms<<<NIN, 256, 0, g.stream>>>(n, M.X, M.target);
  GB_LAUNCHED();
  std::vector<float> ms(NIN);
  GB_CUDA(cudaMemcpyAsync(ms.data(), M.target, sizeof(float) * NIN, cudaMemcpyDeviceToHost, g.stream));
  GB_CUDA(cudaStreamSynchronize(g.stream));
  for (int c = 0; c < NIN; ++c) sc[c] = ms[c] > 1e-30f ? 1.0f / std::sqrt(ms[c]) : 1.0f;
  // force scale: RMS component of the unscaled labels
  mts_labels();
  const int nb = nblocks(n, 256);
  double* blk = gb_blkacc(nb);
  k_sumsq<<<nb, 256, 0, g.stream>>>(n, M.target, blk);
  GB_LAUNCHED();
  gb_reduce_blocks(blk, nb, 1, M.red);
  double r1[1];
  read_scalars(M.red, r1, 1);
  const double d_rms = std::sqrt(r1[0] / (3.0 * n));
  sc[NIN] = (float)(d_rms > 0 ? d_rms : 1.0);
  GB_CUDA(cudaMemcpy(M.scal, sc.data(), sizeof(float) * (NIN + 1), cudaMemcpyHostToDevice));
  M.scales_set = true;
  mts_inputs();  // with the final scales
}

void mts_train_step() {
  const int n = g.natms, nb = M.batch;
  k_seq_idx<<<nblocks(nb, 256), 256, 0, g.stream>>>(nb, M.batch_offset, n, M.idx);
  GB_LAUNCHED();
  M.batch_offset = (int)(((long long)M.batch_offset + nb) % n);
  prof_begin(P_MLP_TRAIN);
  M.train_tiles = launch_train(nb, M.idx, M.X, M.target, M.master, M.tw, M.gpart, M.loss_part, nullptr, M.grad);
  ++M.adam_t;
  const float lr = 1e-3f;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - std::pow(b1, (float)M.adam_t), c2 = 1.0f - std::pow(b2, (float)M.adam_t);
  k_adam<<<nblocks(NPARAM, 256), 256, 0, g.stream>>>(M.master, M.m1, M.m2, M.grad, lr, b1, b2, c1, c2, 1e-8f);
  GB_LAUNCHED();
  publish(M.master, M.net);
  prof_end(P_MLP_TRAIN);
}

// a full step ends one cycle and starts the next: its SPME force and the coarse-grid
// energy, virial and stress are the reference of the following inner steps
void mts_begin_cycle() {
  k_copy_f<<<nblocks(3LL * g.natms, 256), 256, 0, g.stream>>>(3LL * g.natms, M.frec, M.frec0);
  GB_LAUNCHED();
  M.ec0 = M.ec; M.vc0 = M.vc;
  for (int k = 0; k < 9; ++k) M.stc0[k] = M.stc[k];
  M.s = 0;
  M.have_t0 = true;
}

// smallest FFT length >= want that is 2^a 3^b 5^c and a multiple of 4
int coarse_length(int want) {
  for (int K = std::max(8, want);; ++K) {
    if (K % 4) continue;
    int m = K;
    for (int f : {2, 3, 5})
      while (m % f == 0) m /= f;
    if (m == 1) return K;
  }
}

bool training_now() { return M.step <= g.mts_train; }

}  // namespace

// ===================================================================== host
void mts_set_topology(int ntcons, const int32_t* listcon, const double* weight) {
  const int n = g.natms;
  h_triple.assign(3 * (size_t)n, -1);
  if (ntcons <= 0 || !listcon || !weight) return;
  // atoms joined by constraints; molecules of exactly 3 atoms get a frame
  std::vector<int> parent(n);
  for (int i = 0; i < n; ++i) parent[i] = i;
  auto find = [&](int a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
  };
  for (int k = 0; k < ntcons; ++k) {
    const int a = find(listcon[3 * k + 1] - 1), b = find(listcon[3 * k + 2] - 1);
    if (a != b) parent[std::max(a, b)] = std::min(a, b);
  }
  std::vector<std::vector<int>> mol(n);
  for (int i = 0; i < n; ++i) mol[find(i)].push_back(i);
  for (int r = 0; r < n; ++r) {
    const auto& m = mol[r];
    if (m.size() != 3) continue;
    int o = m[0];
    for (int a : m)
      if (weight[a] > weight[o]) o = a;
    int h[2], nh = 0;
    for (int a : m)
      if (a != o) h[nh++] = a;
    for (int a : m) {
      h_triple[3 * a] = o; h_triple[3 * a + 1] = h[0]; h_triple[3 * a + 2] = h[1];
    }
  }
}

void mts_free() {
  void* ptrs[] = {M.master, M.m1, M.m2, M.grad, M.gpart, M.loss_part, M.X, M.frec0, M.frec, M.truth, M.target,
                  M.fc, M.frame, M.triple, M.scal, M.red, M.idx, M.sstart, M.scount,
                  M.slist, M.stmp, M.sown, M.sfill};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  net_free(M.net);
  train_w_free(M.tw);
  M = MtsDev();
}

void mts_setup() {
  mts_free();
  const int n = g.natms;
  M.n = n;
  set_attrs();
  GB_CUDA(cudaMalloc(&M.master, sizeof(float) * NPARAM));
  GB_CUDA(cudaMalloc(&M.m1, sizeof(float) * NPARAM));
  GB_CUDA(cudaMalloc(&M.m2, sizeof(float) * NPARAM));
  GB_CUDA(cudaMalloc(&M.grad, sizeof(float) * NPARAM));
  GB_CUDA(cudaMemset(M.m1, 0, sizeof(float) * NPARAM));
  GB_CUDA(cudaMemset(M.m2, 0, sizeof(float) * NPARAM));
  M.batch = std::min(n, 8192);
  M.gpart_tiles = nblocks(M.batch, TILE_T);
  GB_CUDA(cudaMalloc(&M.gpart, sizeof(float) * NPARAM * (size_t)M.gpart_tiles));
  GB_CUDA(cudaMalloc(&M.loss_part, sizeof(float) * M.gpart_tiles));
  net_alloc(M.net);
  train_w_alloc(M.tw);
  GB_CUDA(cudaMalloc(&M.X, sizeof(__nv_bfloat16) * KIN * (size_t)n));
  for (float** p : {&M.frec0, &M.frec, &M.truth, &M.target, &M.fc})
    GB_CUDA(cudaMalloc(p, sizeof(float) * 3 * (size_t)n));
  // coarse grid: about two thirds of the main grid's points per dimension, order 6
  // (measured against the FP64 oracle on the NaCl melts: half the points leave an rms
  // force error of 7.5e-5 to 9.2e-5 of the total force, two thirds 2.5e-5 to 3.4e-5)
  for (int d = 0; d < 3; ++d) M.Kc[d] = coarse_length((2 * g.p.kmax[d] + 2) / 3);
  M.pc = 6;
  spme_coarse_setup(M.Kc, M.pc);
  GB_CUDA(cudaMalloc(&M.frame, sizeof(float) * 9 * (size_t)n));
  GB_CUDA(cudaMalloc(&M.triple, sizeof(int) * 3 * (size_t)n));
  GB_CUDA(cudaMalloc(&M.scal, sizeof(float) * (NIN + 1)));
  GB_CUDA(cudaMalloc(&M.red, sizeof(double) * 8));
  GB_CUDA(cudaMalloc(&M.idx, sizeof(int) * (size_t)M.batch));
  GB_CUDA(cudaMalloc(&M.sstart, sizeof(int) * ((size_t)n + 1)));
  GB_CUDA(cudaMalloc(&M.scount, sizeof(int) * ((size_t)n + 1)));
  GB_CUDA(cudaMalloc(&M.sown, sizeof(int) * (size_t)n));
  GB_CUDA(cudaMalloc(&M.sfill, sizeof(int) * (size_t)n));
  if ((int)h_triple.size() != 3 * n) h_triple.assign(3 * (size_t)n, -1);
  GB_CUDA(cudaMemcpy(M.triple, h_triple.data(), sizeof(int) * 3 * (size_t)n, cudaMemcpyHostToDevice));
  std::vector<float> sc(NIN + 1, 1.0f);
  GB_CUDA(cudaMemcpy(M.scal, sc.data(), sizeof(float) * (NIN + 1), cudaMemcpyHostToDevice));
  std::vector<float> w = initial_params();
  GB_CUDA(cudaMemcpy(M.master, w.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
  publish(M.master, M.net);
  GB_CUDA(cudaStreamSynchronize(g.stream));
  M.ready = true;
}

bool mts_active() { return M.ready && g.mts_k > 1; }

void mts_set_no_network(bool on) { g_no_network = on; }

// SPME writes its per-atom reciprocal forces here when MTS is active
float* mts_rec_out() { return mts_active() ? M.frec : nullptr; }

// at the start of the force evaluation of an MD step: the coarse-grid forces
// of this step, and whether the step needs the full SPME
// whether this MD step runs the full SPME (host state only: the step count, training,
// the fallback, the cycle position)
bool mts_step_needs_spme() {
  ++M.step;
  if (!M.have_t0) return true;
  return training_now() || M.fallback || M.s + 1 >= g.mts_k;
}

// the coarse-grid reciprocal forces of the current positions (every MD step: inner steps
// build S from them, full steps label and check against them)
void mts_coarse() {
  double st[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  spme_coarse_forces(&M.ec, &M.vc, st, M.fc);
  for (int k = 0; k < 9; ++k) M.stc[k] = st[k];
}

// after a full force evaluation of an MD step (SPME ran and its force is in the
// fixed-point sums): labels, the check, the impulse of a cycle end, training and the
// cycle bookkeeping
void mts_after_full(double erc, double vrc, const double* strec) {
  const int n = g.natms;
  M.n_full++;
  M.erc0 = erc; M.vrc0 = vrc;
  for (int k = 0; k < 9; ++k) M.st0[k] = strec[k];
  if (!M.have_t0) {
    mts_begin_cycle();
    return;
  }
  const int s_new = M.s + 1;
  const bool cycle_end = s_new >= g.mts_k;
  if (!M.scales_set) mts_set_scales();
  else mts_inputs();
  mts_labels();
  const bool trained = M.adam_t > 0 || g_no_network;
  const int nb = nblocks(n, 256);
  if (cycle_end && trained) {
    // S of this step, as the inner steps form it, against SPME (the check)
    prof_begin(P_MLP);
    if (g_no_network) {
      k_copy_f<<<nblocks(3LL * n, 256), 256, 0, g.stream>>>(3LL * n, M.fc, M.truth);
      GB_LAUNCHED();
    } else {
      launch_infer(n, M.X, M.net, M.fc, M.frame, M.scal, M.truth);
    }
    double* blk = gb_blkacc(nb * 7);
    k_net3<<<nb, 256, 0, g.stream>>>(n, M.truth, M.fc, blk + 4 * nb);
    GB_LAUNCHED();
    gb_reduce_blocks(blk + 4 * nb, nb, 3, M.red + 4);
    k_err3<<<nb, 256, 0, g.stream>>>(n, M.truth, M.fc, M.red + 4, 1.0f / (float)n, M.frec0, M.frec, blk);
    GB_LAUNCHED();
    k_fsq<<<nb, 256, 0, g.stream>>>(n, g.fx, g.fy, g.fz, blk + 3 * nb);
    GB_LAUNCHED();
    gb_reduce_blocks(blk, nb, 3, M.red);
    gb_reduce_blocks(blk + 3 * nb, nb, 1, M.red + 3);
    prof_end(P_MLP);
    double r4[4];
    read_scalars(M.red, r4, 4);
    const double ftot = std::max(std::sqrt(r4[3] / n), 1e-300);
    const double err = std::sqrt(r4[0] / n) / ftot;
    M.err_coarse = std::sqrt(r4[1] / n) / ftot;
    M.err_stale = std::sqrt(r4[2] / n) / ftot;
    M.last_err = err;
    M.err_max = std::max(M.err_max, err);
    M.n_checked++;
    if (!training_now()) {
      const bool was = M.fallback;
      M.fallback = err > g.mts_tol;
      if (M.fallback && !was) M.n_fallback++;
    }
    // the impulse: a passed cycle end carries k F_slow = k (F_SPME - S); F_SPME is in
    // the forces already.  Training steps and fallback steps run plain SPME.
    if (!training_now() && !M.fallback) {
      k_mts_impulse<<<nb, 256, 0, g.stream>>>(n, M.frec, M.truth, M.red + 4, 1.0f / (float)n,
                                              (float)(g.mts_k - 1), (unsigned long long*)g.fixp);
      GB_LAUNCHED();
    }
  }
  if ((training_now() || M.fallback) && !g_no_network) {
    mts_train_step();
    M.loss_pending = true;  // read when the counters are asked for, not every training step
  }
  if (cycle_end) mts_begin_cycle();
  else M.s = s_new;
}

// inner step: S = C + the network correction (its net force removed) into the
// fixed-point forces; the reciprocal energy, virial and stress are those of the last
// full step plus the coarse-grid changes since then
void mts_inner(double* erc, double* vrc, double* stress9) {
  const int n = g.natms;
  prof_begin(P_MLP);
  const int nb = nblocks(n, 256);
  if (g_no_network) {
    k_copy_f<<<nblocks(3LL * n, 256), 256, 0, g.stream>>>(3LL * n, M.fc, M.frec);
    GB_LAUNCHED();
    GB_CUDA(cudaMemsetAsync(M.red, 0, 3 * sizeof(double), g.stream));
  } else {
    prof_end(P_MLP);
    mts_inputs();
    prof_begin(P_MLP);
    launch_infer(n, M.X, M.net, M.fc, M.frame, M.scal, M.frec);
    double* blk = gb_blkacc(nb * 3);
    k_net3<<<nb, 256, 0, g.stream>>>(n, M.frec, M.fc, blk);
    GB_LAUNCHED();
    gb_reduce_blocks(blk, nb, 3, M.red);
  }
  k_mts_apply<<<nb, 256, 0, g.stream>>>(n, M.frec, M.red, 1.0f / (float)n, (unsigned long long*)g.fixp);
  GB_LAUNCHED();
  prof_end(P_MLP);
  *erc = M.erc0 + (M.ec - M.ec0);
  *vrc = M.vrc0 + (M.vc - M.vc0);
  for (int k = 0; k < 9; ++k) stress9[k] += M.st0[k] + (M.stc[k] - M.stc0[k]);
  M.n_inner++;
  M.s++;
}

void mts_stats(double* out, int nv) {
  if (M.loss_pending && M.loss_part) {
    std::vector<float> lp(M.train_tiles > 0 ? M.train_tiles : M.gpart_tiles);  // the last step's partials
    GB_CUDA(cudaMemcpyAsync(lp.data(), M.loss_part, sizeof(float) * lp.size(), cudaMemcpyDeviceToHost, g.stream));
    GB_CUDA(cudaStreamSynchronize(g.stream));
    double l = 0.0;
    for (float v : lp) l += v;
    M.last_loss = l;
    M.loss_pending = false;
  }
  const double v[13] = {M.last_err, (double)M.n_full, (double)M.n_inner, (double)M.n_fallback, M.last_loss,
                        (double)M.adam_t, M.err_max, M.fallback ? 1.0 : 0.0, (double)M.n_checked, (double)M.step,
                        M.err_coarse, M.err_stale, (double)M.Kc[0]};
  for (int k = 0; k < nv && k < 13; ++k) out[k] = v[k];
}

// ---------------------------------------------------------------- test hooks
// forward + MSE + backward of the training kernel on nb given rows
int mlp_train_eval(int nb, const float* x, const float* target, const float* params, float* loss, float* grad,
                   float* yout) {
  if (nb <= 0 || nb > 65536 || !x || !target || !params || !loss || !grad || !yout) return GB_ERR_ARG;
  set_attrs();
  const int nt = nblocks(nb, TILE_T);  // partials: at least as many as either kernel's tiles
  std::vector<__nv_bfloat16> hx((size_t)nb * KIN);
  for (int r = 0; r < nb; ++r)
    for (int c = 0; c < KIN; ++c) hx[(size_t)r * KIN + c] = __float2bfloat16(c < NIN ? x[(size_t)r * NIN + c] : 0.f);
  std::vector<int> hi(nb);
  for (int r = 0; r < nb; ++r) hi[r] = r;
  __nv_bfloat16* dX = nullptr;
  float *dT = nullptr, *dP = nullptr, *dG = nullptr, *dGp = nullptr, *dL = nullptr, *dY = nullptr;
  int* dI = nullptr;
  GB_CUDA(cudaMalloc(&dX, sizeof(__nv_bfloat16) * hx.size()));
  GB_CUDA(cudaMalloc(&dT, sizeof(float) * 3 * nb));
  GB_CUDA(cudaMalloc(&dP, sizeof(float) * NPARAM));
  GB_CUDA(cudaMalloc(&dG, sizeof(float) * NPARAM));
  GB_CUDA(cudaMalloc(&dGp, sizeof(float) * NPARAM * (size_t)nt));
  GB_CUDA(cudaMalloc(&dL, sizeof(float) * nt));
  GB_CUDA(cudaMalloc(&dY, sizeof(float) * 3 * nb));
  GB_CUDA(cudaMalloc(&dI, sizeof(int) * nb));
  GB_CUDA(cudaMemcpy(dX, hx.data(), sizeof(__nv_bfloat16) * hx.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(dT, target, sizeof(float) * 3 * nb, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(dP, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(dI, hi.data(), sizeof(int) * nb, cudaMemcpyHostToDevice));
  TrainW tw;
  train_w_alloc(tw);
  GB_CUDA(cudaMemsetAsync(&g.sc->status, 0, sizeof(int), g.stream));
  const int ntr = launch_train(nb, dI, dX, dT, dP, tw, dGp, dL, dY, dG);
  std::vector<float> hl(ntr);
  GB_CUDA(cudaMemcpyAsync(grad, dG, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, g.stream));
  GB_CUDA(cudaMemcpyAsync(hl.data(), dL, sizeof(float) * ntr, cudaMemcpyDeviceToHost, g.stream));
  GB_CUDA(cudaMemcpyAsync(yout, dY, sizeof(float) * 3 * nb, cudaMemcpyDeviceToHost, g.stream));
  gb_sync_scalars();
  float l = 0.f;
  for (float v : hl) l += v;
  *loss = l;
  for (void* p : {(void*)dX, (void*)dT, (void*)dP, (void*)dG, (void*)dGp, (void*)dL, (void*)dY, (void*)dI}) cudaFree(p);
  train_w_free(tw);
  return (g.hsc->status & ST_DEVICE_WAIT) ? GB_ERR_DEVICE_WAIT : GB_OK;
}

// the inference kernel on nb given rows (lab frame, zero base force, unit scales)
int mlp_infer_eval(int nb, const float* x, const float* params, float* yout) {
  if (nb <= 0 || nb > (1 << 22) || !x || !params || !yout) return GB_ERR_ARG;
  set_attrs();
  Net net;
  net_alloc(net);
  float* dP = nullptr;
  GB_CUDA(cudaMalloc(&dP, sizeof(float) * NPARAM));
  GB_CUDA(cudaMemcpy(dP, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
  publish(dP, net);
  std::vector<__nv_bfloat16> hx((size_t)nb * KIN);
  for (int r = 0; r < nb; ++r)
    for (int c = 0; c < KIN; ++c) hx[(size_t)r * KIN + c] = __float2bfloat16(c < NIN ? x[(size_t)r * NIN + c] : 0.f);
  std::vector<float> fr(9 * (size_t)nb, 0.f), sc(NIN + 1, 1.f);
  for (int r = 0; r < nb; ++r) { fr[9 * (size_t)r] = 1.f; fr[9 * (size_t)r + 4] = 1.f; fr[9 * (size_t)r + 8] = 1.f; }
  __nv_bfloat16* dX = nullptr;
  float *dF0 = nullptr, *dFr = nullptr, *dS = nullptr, *dOut = nullptr;
  GB_CUDA(cudaMalloc(&dX, sizeof(__nv_bfloat16) * hx.size()));
  GB_CUDA(cudaMalloc(&dF0, sizeof(float) * 3 * (size_t)nb));
  GB_CUDA(cudaMalloc(&dFr, sizeof(float) * fr.size()));
  GB_CUDA(cudaMalloc(&dS, sizeof(float) * sc.size()));
  GB_CUDA(cudaMalloc(&dOut, sizeof(float) * 3 * (size_t)nb));
  GB_CUDA(cudaMemcpy(dX, hx.data(), sizeof(__nv_bfloat16) * hx.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemset(dF0, 0, sizeof(float) * 3 * (size_t)nb));
  GB_CUDA(cudaMemcpy(dFr, fr.data(), sizeof(float) * fr.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(dS, sc.data(), sizeof(float) * sc.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemsetAsync(&g.sc->status, 0, sizeof(int), g.stream));
  launch_infer(nb, dX, net, dF0, dFr, dS, dOut);
  GB_CUDA(cudaMemcpyAsync(yout, dOut, sizeof(float) * 3 * (size_t)nb, cudaMemcpyDeviceToHost, g.stream));
  gb_sync_scalars();
  for (void* p : {(void*)dP, (void*)dX, (void*)dF0, (void*)dFr, (void*)dS, (void*)dOut}) cudaFree(p);
  net_free(net);
  return (g.hsc->status & ST_DEVICE_WAIT) ? GB_ERR_DEVICE_WAIT : GB_OK;
}

// copies the current inputs (nv <= natms rows of 51 floats) and the 52 scales
int mts_features(float* x, int nv, float* scal) {
  if (!M.ready) return GB_ERR_NOT_INIT;
  if (nv < 0 || nv > g.natms || (nv > 0 && !x)) return GB_ERR_ARG;
  GB_CUDA(cudaStreamSynchronize(g.stream));
  std::vector<__nv_bfloat16> hx((size_t)nv * KIN);
  if (nv > 0) GB_CUDA(cudaMemcpy(hx.data(), M.X, sizeof(__nv_bfloat16) * hx.size(), cudaMemcpyDeviceToHost));
  for (int r = 0; r < nv; ++r)
    for (int c = 0; c < NIN; ++c) x[(size_t)r * NIN + c] = __bfloat162float(hx[(size_t)r * KIN + c]);
  if (scal) GB_CUDA(cudaMemcpy(scal, M.scal, sizeof(float) * (NIN + 1), cudaMemcpyDeviceToHost));
  return GB_OK;
}

int mlp_param_count() { return NPARAM; }
