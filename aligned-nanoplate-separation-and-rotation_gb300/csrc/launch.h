// launch.h -- host-side declarations of the kernel launchers of libscft.
#pragma once

#include "common.h"

namespace scft {

// Block size, dynamic shared memory and per-thread value bound (MAXV) of a
// launch; MAXV * threads must cover the largest plane or tile of the batch.
// gm: the plane does not fit in shared memory (FP64 planes above ~227 KB, e.g.
// 128 x 128): the plane kernels then transform it in place in its own array
// in global memory (L2-resident while the CTA works on it) and shared memory
// holds only the twiddles; smem is then that smaller size.
struct LaunchShape {
  int threads;
  int smem;
  int maxv;
  int gm;
  int pp = 0;     // FP32 transforms out of place between two buffers (smem includes the second one)
  int stage = 0;  // mixed plane pass: planes staged by bulk copy (smem includes that buffer too; needs pp)
};

template <typename T>
cudaError_t launch_plane_fft(const LaunchShape &ls, const PlaneJob *jobs, int njobs, const DevGeom *geoms,
                             const void *tw, int sign, int scale, cudaStream_t st);
template <typename T>
cudaError_t launch_col_fft(const LaunchShape &ls, const ColJob *jobs, int njobs, const DevGeom *geoms,
                           const void *tw, int mode, int scale, cudaStream_t st);

}  // namespace scft
