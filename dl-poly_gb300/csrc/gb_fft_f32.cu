// gb_fft_f32.cu - constant-length FP32 grid transforms (mixed form and the
// coarse grid of the learned multiple-time-step form).  x lengths are half the
// grid length (real-to-complex x pass); y and z lengths are the grid lengths:
// 48^3, 100^3, 160^3, 192^3 fine grids and the 32^3, 72^3, 128^3 coarse grids of
// those workloads.
#include "gb_fft.cuh"

namespace gbspme {
template <>
FftKernels<float, float2> fft_kernels<float, float2>(int M, int K2, int K3) {
  return fft_pick<float, float2>(FftLens<16, 24, 36, 50, 64, 80, 96>(), FftLens<32, 48, 72, 100, 128, 160, 192>(), M,
                                 K2, K3);
}
}  // namespace gbspme
