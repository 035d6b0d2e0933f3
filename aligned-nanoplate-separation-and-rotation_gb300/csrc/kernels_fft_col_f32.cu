// kernels_fft_col_f32.cu -- the FP32 z-column pass of the batched 3-D FFT (templates in
// kernels_fft.cuh), in a translation unit of its own.
#include "kernels_fft.cuh"

namespace scft {

template cudaError_t launch_col_fft<float>(const LaunchShape &, const ColJob *, int, const DevGeom *,
                                           const void *, int, int, cudaStream_t);

}  // namespace scft
