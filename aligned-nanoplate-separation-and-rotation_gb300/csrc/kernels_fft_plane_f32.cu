// kernels_fft_plane_f32.cu -- the FP32 plane pass of the batched 3-D FFT (templates in
// kernels_fft.cuh), in a translation unit of its own.
#include "kernels_fft.cuh"

namespace scft {

template cudaError_t launch_plane_fft<float>(const LaunchShape &, const PlaneJob *, int, const DevGeom *,
                                             const void *, int, int, cudaStream_t);

}  // namespace scft
