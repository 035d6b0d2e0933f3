// kernels_fft.cuh -- batched 3-D complex FFTs on per-instance grids.
//
// Kernel and launcher templates only: each (pass, precision) pair is
// instantiated in its own translation unit (kernels_fft_{plane,col}_f{32,64}.cu)
// so that the library's units compile in parallel.
//
// A 3-D transform is two passes over the array:
//   plane pass : one CTA per (array, z) loads the nx*ny plane into shared
//                memory, transforms rows (x) then columns (y), stores it;
//   column pass: one CTA per (array, y, x-tile) loads tx*nz values, transforms
//                along z and stores them.  With a k-space multiplier table the
//                column pass does forward-z, multiply, inverse-z in one go, which
//                is the whole k-space half of a convolution.
// The reference's fft_fwd_wrapper/fft_bck_wrapper (code/fft_wrappers.cpp:4-67)
// are forward scaled by 1/M and backward unscaled; the scale is folded into
// the last pass of a forward transform or into the multiplier.
#pragma once
#include "fft_core.cuh"
#include "launch.h"

namespace scft {

// GM: the plane is transformed in place in global memory (see LaunchShape).
// PP: out-of-place stages between two shared buffers (FP32 planes that leave
// room for the second one).
template <typename T, int SIGN, int MAXV, bool GM, bool PP>
__global__ void __launch_bounds__(512) k_plane_fft(const PlaneJob *__restrict__ jobs, const DevGeom *__restrict__ geoms,
                            const cx<T> *__restrict__ twbuf, int scale_by_M) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PlaneJob jb = jobs[blockIdx.x];
  const DevGeom g = geoms[jb.geom];
  const int E = g.nx * g.ny;
  C *a = reinterpret_cast<C *>(jb.ptr) + (long long)jb.z * E;
  C *plane = GM ? a : reinterpret_cast<C *>(smem_raw);
  C *twx = GM ? reinterpret_cast<C *>(smem_raw) : plane + (PP ? 2 : 1) * E;
  C *twy = twx + g.nx;
  load_tw<T>(twx, twbuf, g.ax[0]);
  load_tw<T>(twy, twbuf, g.ax[1]);
  if (!GM)
    for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = a[e];
  __syncthreads();
  if (PP)
    plane = fft_plane_pp<T, SIGN>(plane, plane + E, g, twx, twy);
  else
    fft_plane<T, SIGN, MAXV>(plane, g, twx, twy);
  if (scale_by_M) {
    const T s = (T)g.inv_m;
    for (int e = threadIdx.x; e < E; e += blockDim.x) a[e] = cscale(plane[e], s);
  } else if (!GM) {
    for (int e = threadIdx.x; e < E; e += blockDim.x) a[e] = plane[e];
  }
}

// MODE 0: forward z (sign -1); 1: inverse z (sign +1); 2: forward, multiply by
// kern[x,y,z] * scale, inverse; 3 (FP32 propagator of the mixed form):
// forward, drop the k = 0 coefficient (the mean is carried exactly in FP64 by
// the plane pass), multiply by (1 - h) / M with h = 1 - g(k) tabulated and 1/M
// applied as a two-float product, inverse.  Writing g = 1 - h keeps the
// low-k bond factors, which decide Q, exact to eps*h instead of eps.
// PP: out-of-place stages between two tile buffers (fft_lines_pp; the FP32
// passes, whose tiles leave room for the second buffer).
template <typename T, int MODE, int MAXV, bool PP>
__global__ void __launch_bounds__(512) k_col_fft(const ColJob *__restrict__ jobs, const DevGeom *__restrict__ geoms,
                          const cx<T> *__restrict__ twbuf, int scale_by_M) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const ColJob jb = jobs[blockIdx.x];
  const DevGeom g = geoms[jb.geom];
  const int tx = g.tx, nz = g.nz;
  const int E = tx * nz;
  C *tile0 = reinterpret_cast<C *>(smem_raw);
  C *tile1 = tile0 + E;  // second buffer (PP)
  C *twz = tile0 + (PP ? 2 : 1) * E;
  C *tile = tile0;       // buffer holding the tile
  load_tw<T>(twz, twbuf, g.ax[2]);
  C *a = reinterpret_cast<C *>(jb.ptr);
  const long long plane = (long long)g.nx * g.ny;
  const long long base = (long long)jb.y * g.nx + jb.x0;
  // tx is a power of two (16 halved until it divides nx); four independent
  // loads in flight per thread and round
  const int ltx = __ffs(tx) - 1;
  for (int e0 = threadIdx.x; e0 < E; e0 += 4 * blockDim.x) {
    C t4[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int e = e0 + u * blockDim.x;
      if (e < E) t4[u] = a[(e >> ltx) * plane + base + (e & (tx - 1))];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int e = e0 + u * blockDim.x;
      if (e < E) tile[e] = t4[u];
    }
  }
  __syncthreads();
  if (PP) {
    tile = (MODE == 1) ? fft_lines_pp<T, +1>(tile0, tile1, g.ax[2], tx, 1, tx, twz)
                       : fft_lines_pp<T, -1>(tile0, tile1, g.ax[2], tx, 1, tx, twz);
  } else if (MODE == 1) {
    fft_lines<T, +1, MAXV>(tile, g.ax[2], tx, 1, tx, twz);
  } else {
    fft_lines<T, -1, MAXV>(tile, g.ax[2], tx, 1, tx, twz);
  }
  if (MODE == 2) {
    const T *kern = reinterpret_cast<const T *>(jb.kern);
    const T s = scale_by_M ? (T)g.inv_m : (T)1;
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const int z = e >> ltx, x = e & (tx - 1);
      const T kv = kern[z * plane + base + x];
      tile[e] = cscale(cscale(tile[e], s), kv);
    }
    __syncthreads();
    if (PP)
      tile = fft_lines_pp<T, +1>(tile, tile == tile0 ? tile1 : tile0, g.ax[2], tx, 1, tx, twz);
    else
      fft_lines<T, +1, MAXV>(tile, g.ax[2], tx, 1, tx, twz);
  }
  if (MODE == 3) {
    const T *kern = reinterpret_cast<const T *>(jb.kern);
    const T s_hi = (T)g.inv_m_hi, s_lo = (T)g.inv_m_lo;
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const int z = e >> ltx, x = e & (tx - 1);
      const T h = kern[z * plane + base + x];
      const C v = tile[e];
      C t = mkc(fma(v.x, s_hi, v.x * s_lo), fma(v.y, s_hi, v.y * s_lo));
      t = mkc(fma(-h, t.x, t.x), fma(-h, t.y, t.y));
      if (e == 0 && jb.x0 == 0 && jb.y == 0) t = mkc((T)0, (T)0);
      tile[e] = t;
    }
    __syncthreads();
    if (PP)
      tile = fft_lines_pp<T, +1>(tile, tile == tile0 ? tile1 : tile0, g.ax[2], tx, 1, tx, twz);
    else
      fft_lines<T, +1, MAXV>(tile, g.ax[2], tx, 1, tx, twz);
  }
  const T s = (MODE == 0 && scale_by_M) ? (T)g.inv_m : (T)1;
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    const int z = e >> ltx, x = e & (tx - 1);
    a[z * plane + base + x] = (MODE == 0 && scale_by_M) ? cscale(tile[e], s) : tile[e];
  }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <typename T, int SIGN, int MAXV>
static cudaError_t launch_plane_t(const LaunchShape &ls, const PlaneJob *jobs, int njobs, const DevGeom *geoms,
                                  const void *tw, int scale, cudaStream_t st) {
  auto kfn = ls.gm ? k_plane_fft<T, SIGN, MAXV, true, false> : k_plane_fft<T, SIGN, MAXV, false, false>;
  if constexpr (sizeof(T) == sizeof(float)) {
    if (ls.pp) kfn = k_plane_fft<T, SIGN, 8, false, true>;  // the value bound does not apply out of place
  } else {
    if (ls.pp) return cudaErrorInvalidValue;  // FP32 only
  }
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, ls.smem);
  if (e != cudaSuccess) return e;
  kfn<<<njobs, ls.threads, ls.smem, st>>>(jobs, geoms, reinterpret_cast<const cx<T> *>(tw), scale);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_plane_fft(const LaunchShape &ls, const PlaneJob *jobs, int njobs, const DevGeom *geoms,
                             const void *tw, int sign, int scale, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (sign < 0) {
    if (ls.maxv <= 8) return launch_plane_t<T, -1, 8>(ls, jobs, njobs, geoms, tw, scale, st);
    if (ls.maxv <= 16) return launch_plane_t<T, -1, 16>(ls, jobs, njobs, geoms, tw, scale, st);
    return launch_plane_t<T, -1, 32>(ls, jobs, njobs, geoms, tw, scale, st);
  }
  if (ls.maxv <= 8) return launch_plane_t<T, 1, 8>(ls, jobs, njobs, geoms, tw, scale, st);
  if (ls.maxv <= 16) return launch_plane_t<T, 1, 16>(ls, jobs, njobs, geoms, tw, scale, st);
  return launch_plane_t<T, 1, 32>(ls, jobs, njobs, geoms, tw, scale, st);
}

template <typename T, int MODE, int MAXV, bool PP = false>
static cudaError_t launch_col_t(const LaunchShape &ls, const ColJob *jobs, int njobs, const DevGeom *geoms,
                                const void *tw, int scale, cudaStream_t st) {
  auto kfn = k_col_fft<T, MODE, MAXV, PP>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, ls.smem);
  if (e != cudaSuccess) return e;
  kfn<<<njobs, ls.threads, ls.smem, st>>>(jobs, geoms, reinterpret_cast<const cx<T> *>(tw), scale);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_col_fft(const LaunchShape &ls, const ColJob *jobs, int njobs, const DevGeom *geoms,
                           const void *tw, int mode, int scale, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if constexpr (sizeof(T) == sizeof(float)) {
    if (ls.pp) {  // the value bound does not apply out of place
      if (mode == 0) return launch_col_t<T, 0, 8, true>(ls, jobs, njobs, geoms, tw, scale, st);
      if (mode == 1) return launch_col_t<T, 1, 8, true>(ls, jobs, njobs, geoms, tw, scale, st);
      if (mode == 3) return launch_col_t<T, 3, 8, true>(ls, jobs, njobs, geoms, tw, scale, st);
      return launch_col_t<T, 2, 8, true>(ls, jobs, njobs, geoms, tw, scale, st);
    }
  } else {
    if (ls.pp) return cudaErrorInvalidValue;  // FP32 only
  }
#define SCFT_COL(MODE)                                                                          \
  do {                                                                                          \
    if (ls.maxv <= 8) return launch_col_t<T, MODE, 8>(ls, jobs, njobs, geoms, tw, scale, st);   \
    if (ls.maxv <= 16) return launch_col_t<T, MODE, 16>(ls, jobs, njobs, geoms, tw, scale, st); \
    return launch_col_t<T, MODE, 32>(ls, jobs, njobs, geoms, tw, scale, st);                    \
  } while (0)
  if (mode == 0) SCFT_COL(0);
  if (mode == 1) SCFT_COL(1);
  if (mode == 3) SCFT_COL(3);
  SCFT_COL(2);
#undef SCFT_COL
}

}  // namespace scft
