// launch.h -- host-side declarations of the kernel launchers of libscft.
#pragma once

#include "common.h"

namespace scft {

// Block size, dynamic shared memory and per-thread value bound (MAXV) of a
// launch; MAXV * threads must cover the largest plane or tile of the batch.
struct LaunchShape {
  int threads;
  int smem;
  int maxv;
};

template <typename T>
cudaError_t launch_plane_fft(const LaunchShape &ls, const PlaneJob *jobs, int njobs, const DevGeom *geoms,
                             const void *tw, int sign, int scale, cudaStream_t st);
template <typename T>
cudaError_t launch_col_fft(const LaunchShape &ls, const ColJob *jobs, int njobs, const DevGeom *geoms,
                           const void *tw, int mode, int scale, cudaStream_t st);

}  // namespace scft
