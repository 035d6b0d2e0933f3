// kernels_graft_f64.cu -- launcher of the FP64 graft propagator plane pass
// (k_graft_plane_f64); the kernels are in kernels_prop.cuh.
#include "kernels_prop.cuh"

namespace scft {

template <int MAXV>
static cudaError_t launch_graft_plane_t(const LaunchShape &ls, const PropJob *jobs, int njobs,
                                        const PropInst *insts, const DevGeom *geoms, const void *tw, int sweep,
                                        int n, cudaStream_t st) {
  auto kfn = ls.gm ? k_graft_plane_f64<MAXV, true> : k_graft_plane_f64<MAXV, false>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, ls.smem);
  if (e != cudaSuccess) return e;
  kfn<<<njobs, ls.threads, ls.smem, st>>>(jobs, insts, geoms, reinterpret_cast<const double2 *>(tw), sweep, n);
  return cudaGetLastError();
}

cudaError_t launch_graft_plane_f64(const LaunchShape &ls, const PropJob *jobs, int njobs, const PropInst *insts,
                                   const DevGeom *geoms, const void *tw, int sweep, int n, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (ls.maxv <= 8) return launch_graft_plane_t<8>(ls, jobs, njobs, insts, geoms, tw, sweep, n, st);
  if (ls.maxv <= 16) return launch_graft_plane_t<16>(ls, jobs, njobs, insts, geoms, tw, sweep, n, st);
  return launch_graft_plane_t<32>(ls, jobs, njobs, insts, geoms, tw, sweep, n, st);
}

}  // namespace scft
