// gb_fft_f32.cu - constant-length FP32 grid transforms (mixed form and the
// coarse grid of the learned multiple-time-step form).  x lengths are half the
// grid length (real-to-complex x pass); y and z lengths are the grid lengths:
// 48^3, 100^3, 160^3, 192^3 fine grids and 24^3, 60^3, 96^3 coarse grids.
#include "gb_fft.cuh"

namespace gbspme {
template <>
FftKernels<float, float2> fft_kernels<float, float2>(int M, int K2, int K3) {
  return fft_pick<float, float2>(FftLens<12, 24, 30, 48, 50, 80, 96>(), FftLens<24, 48, 60, 96, 100, 160, 192>(), M,
                                 K2, K3);
}
}  // namespace gbspme
