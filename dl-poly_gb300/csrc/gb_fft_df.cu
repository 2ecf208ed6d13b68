// gb_fft_df.cu - constant-length double-float grid transforms (the FP64
// form's SPME grids: 48^3, 100^3, 160^3, 192^3; x lengths are half the grid
// length for the real-to-complex x pass).
#include "gb_fft.cuh"

namespace gbspme {
template <>
FftKernels<dfr, dfc> fft_kernels<dfr, dfc>(int M, int K2, int K3) {
  return fft_pick<dfr, dfc>(FftLens<24, 50, 80, 96>(), FftLens<48, 100, 160, 192>(), M, K2, K3);
}
}  // namespace gbspme
