// gb_noalloc.cu - kinetic stress (kinstress, source/kinetics.F90:218-262) for
// callers that cannot allocate device memory.
//
// Some host programs cannot call cudaMalloc at the point where they need the
// kinetic stress: a driver that has handed its whole device-memory budget to
// a pool owned by another framework, or code that runs where allocation is not
// permitted (for example a step that must not change the device memory
// footprint once a long run has started).  gb_kinstress_noalloc serves them:
// it takes device pointers for its inputs and its output and allocates
// nothing.  Its per-block partial sums live in the file-scope array below,
// which every GPU that loads this library holds until the process exits.
#include "gb_common.cuh"

namespace {

constexpr int KIN_THREADS = 256;
constexpr int KIN_MAX_BLOCKS = 4096;                              // 4096 * 256 = 1,048,576 atoms
constexpr int KIN_MAX_ATOMS = KIN_MAX_BLOCKS * KIN_THREADS;
constexpr int KIN_MAX_DEVICES = 64;

// 6 partial sums per block: 4096 * 6 * 8 B = 196,608 B per device.
static __device__ __align__(256) double g_kin_scratch[KIN_MAX_BLOCKS * 6];

// Host side: the device address of g_kin_scratch on each device, looked up
// once per device.  (In host code the symbol name itself is only a host-side
// stand-in, never a device address.)
double* g_kin_scratch_addr[KIN_MAX_DEVICES] = {nullptr};

__global__ void k_kin_partial(int n, const double* __restrict__ w, const int* __restrict__ lfrzn,
                              const double* __restrict__ vx, const double* __restrict__ vy,
                              const double* __restrict__ vz, double* part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a[6] = {0, 0, 0, 0, 0, 0};
  if (i < n && (lfrzn == nullptr || lfrzn[i] == 0)) {
    const double m = w[i];
    a[0] = m * vx[i] * vx[i]; a[1] = m * vx[i] * vy[i]; a[2] = m * vx[i] * vz[i];
    a[3] = m * vy[i] * vy[i]; a[4] = m * vy[i] * vz[i]; a[5] = m * vz[i] * vz[i];
  }
  // every block writes its own 6 slots, so nothing has to be cleared first
  block_reduce_store<6>(a, part);
}

__global__ void k_kin_final(int nb, const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double red[32][6];
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int k = 0; k < 6; ++k) s[k] += part[(size_t)b * 6 + k];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < 6; ++k) s[k] = warp_sum(s[k]);
  if (lane == 0)
    for (int k = 0; k < 6; ++k) red[wid][k] = s[k];
  __syncthreads();
  if (wid == 0) {
    for (int k = 0; k < 6; ++k) {
      double t = lane < (int)(blockDim.x >> 5) ? red[lane][k] : 0.0;
      s[k] = warp_sum(t);
    }
    if (lane == 0) {
      out[0] = s[0]; out[1] = s[1]; out[2] = s[2];
      out[3] = s[1]; out[4] = s[3]; out[5] = s[4];
      out[6] = s[2]; out[7] = s[4]; out[8] = s[5];
    }
  }
}

}  // namespace

extern "C" int gb_kinstress_noalloc(const double* vx, const double* vy, const double* vz, const double* weight,
                                    const int32_t* lfrzn, int n, double* strkin_out, void* stream) {
  if (n < 0 || !strkin_out || (n > 0 && (!vx || !vy || !vz || !weight))) return GB_ERR_ARG;
  if (n > KIN_MAX_ATOMS) return GB_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= KIN_MAX_DEVICES) return GB_ERR_CUDA;
  if (!g_kin_scratch_addr[dev]) {
    // first call on this device: look up the device address of the scratch array
    double* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_kin_scratch) != cudaSuccess || !p) return GB_ERR_CUDA;
    g_kin_scratch_addr[dev] = p;
  }
  double* part = g_kin_scratch_addr[dev];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = n > 0 ? (n + KIN_THREADS - 1) / KIN_THREADS : 1;
  k_kin_partial<<<nb, KIN_THREADS, 0, st>>>(n, weight, lfrzn, vx, vy, vz, part);
  if (cudaGetLastError() != cudaSuccess) return GB_ERR_CUDA;
  k_kin_final<<<1, 256, 0, st>>>(nb, part, strkin_out);
  if (cudaGetLastError() != cudaSuccess) return GB_ERR_CUDA;
  return GB_OK;
}
