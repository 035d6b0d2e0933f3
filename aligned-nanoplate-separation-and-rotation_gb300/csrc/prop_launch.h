// prop_launch.h -- launchers of the propagator and field kernels.
#pragma once

#include <cuda.h>

#include "inst.h"
#include "launch.h"

namespace scft {

cudaError_t launch_prop_plane_f64(const LaunchShape &ls, const PropJob *jobs, int njobs, const PropInst *insts,
                                  const DevGeom *geoms, const void *tw, int n, cudaStream_t st);

cudaError_t launch_graft_plane_f64(const LaunchShape &ls, const PropJob *jobs, int njobs, const PropInst *insts,
                                   const DevGeom *geoms, const void *tw, int sweep, int n, cudaStream_t st);
cudaError_t launch_graft_finalize(const FieldInst *fi, int ninst, int blocks, double2 *part, cudaStream_t st);
cudaError_t launch_qga_finalize(const FieldInst *fi, int ninst, int blocks, const double2 *part, cudaStream_t st);

cudaError_t launch_assemble(const FieldInst *fi, int ninst, int blocks, cudaStream_t st);
cudaError_t launch_boltzmann(const FieldInst *fi, int ninst, int blocks, cudaStream_t st);
cudaError_t launch_q_finalize(const FieldInst *fi, int ninst, cudaStream_t st);
cudaError_t launch_density(const FieldInst *fi, int ninst, int blocks, cudaStream_t st);
cudaError_t launch_update_1s(const FieldInst *fi, int ninst, int blocks, cudaStream_t st);
cudaError_t launch_h_partials(const FieldInst *fi, int ninst, int blocks, double2 *out, cudaStream_t st);

// err: error word set when a bounded wait of the staged form runs out (needed when ls.stage)
cudaError_t launch_mix_prop_plane(const LaunchShape &ls, const PropJob *jobs, int njobs, const MixInst *insts,
                                  const DevGeom *geoms, const void *tw, int n, int *err, cudaStream_t st);
// Instances of one 64^3 plane-pass launch, passed by value as the kernel
// parameter (15.4 KB: TMA descriptors of each instance's Boltzmann and
// history arrays, the instance views, the error word); larger batches are
// launched in chunks.
// The per-step launchers pass the smallest table that holds the launch's
// instances (CAP 4, 16 or 48): a kernel's parameter block is copied to the
// GPU with every launch, and the 48-instance table (15.4 KB) cost as much
// launch time as the kernel itself.
constexpr int kMix64MaxInst = 48;
template <int CAP> struct Mix64TableT {
  CUtensorMap tmE[CAP];  // E32 as 4096 rows x 128 floats, boxes of 64 rows x 32 floats, 128B swizzle
  CUtensorMap tmH[CAP];  // hist32 as 4096 (hmax + 1) rows x 128 floats, same boxes
  MixInst inst[CAP];
  int *err;              // set to 1 when an mbarrier wait runs out
  int nz;                // z planes per instance (64 x 64 xy planes)
};
typedef Mix64TableT<kMix64MaxInst> Mix64Table;
// The whole mixed sweep of a batch of 64 x 64 x 64 instances in one
// persistent launch (k_mix_sweep64): the kernel parameter adds to the plane
// pass's table each instance's per-axis h table of the z pass and the task
// counters.  Instances in job order (N non-increasing), at most
// kMix64MaxInst.
struct Sweep64Table {
  Mix64Table m;
  const float *ht[kMix64MaxInst];  // [hx | hy | hz] of each instance (z pass)
  unsigned *ctr;   // [0] next task, [1] abort flag, [2 + i] plane tasks done and [2 + ninst + i] z tasks done of instance i
  int ninst;
  unsigned total;  // tasks of the sweep
  float s_hi, s_lo;  // 1/M as a two-float pair
};
// Counters needed by launch_mix_sweep64 for ninst instances (unsigned ints).
inline int sweep64_counters(int ninst) { return 2 + 2 * ninst; }
// CTAs of k_mix_sweep64 resident at once on the current device.
cudaError_t sweep64_capacity(int *ctas);
// insts, tmE, tmH, ht: host arrays of the instances in job order; ctr: device
// array of sweep64_counters(ninst) unsigned ints (cleared by the launch);
// max_ctas: cap on the grid (0: as many CTAs as are resident at once)
cudaError_t launch_mix_sweep64(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH,
                               const float *const *ht, int ninst, const void *tw64, unsigned *ctr, int *err,
                               int max_ctas, cudaStream_t st);
// insts, tmE, tmH: host arrays of the active instances in job order (nz CTAs each)
cudaError_t launch_mix_plane64(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                               int nz, const void *tw64, int n, int *err, cudaStream_t st);
// The same plane pass with warp-local column transforms (k_mix_plane64w):
// bit-identical results, a different launch shape.
cudaError_t launch_mix_plane64w(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                                int nz, const void *tw64, int n, int *err, cudaStream_t st);
// z pass of the specialised instances for nz = 64, 128 or 256 (tw: the
// nz-point twiddles; jb.kern: the [hx | hy | hz] table); tx: x columns per
// CTA (8, 16 or 32); jobs built for that width
cudaError_t launch_mix_col64(const ColJob *jobs, int njobs, const void *tw, int nx, int ny, int nz, int tx,
                             cudaStream_t st);
cudaError_t launch_mix_col256(const ColJob *jobs, int njobs, const void *tw, int nx, int ny, int tx, cudaStream_t st);
// Plane pass of step n for 128 x 128 xy planes (kernels_mixed128.cu): four
// CTAs per plane; insts, tmE, tmH as for launch_mix_plane64 with tensor maps
// of rows of 128 float2; tw64, tw128: the 64- and 128-point twiddles.
cudaError_t launch_mix_plane128(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                                int nz, const void *tw64, const void *tw128, int n, int *err, cudaStream_t st);
// Plane pass of step n for 96 x 64 xy planes (kernels_mixed96.cu): three
// CTAs per plane; tensor maps of rows of 96 float2; tw64, tw32, tw96: the
// 64-, 32- and 96-point twiddles.
cudaError_t launch_mix_plane96(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                               int nz, const void *tw64, const void *tw32, const void *tw96, int n, int *err,
                               cudaStream_t st);
// Plane and z passes for 48 x 48 x 48 instances (kernels_mixed48.cu): one
// 192-thread CTA per plane; tensor maps of rows of 48 float2 with 48-row
// boxes; tw48: the 48-point twiddles; z-pass jobs of 16 columns.
cudaError_t launch_mix_plane48(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                               int nz, const void *tw48, int n, int *err, cudaStream_t st);
cudaError_t launch_mix_col48(const ColJob *jobs, int njobs, const void *tw48, int nx, int ny, cudaStream_t st);
// Graft sweep plane pass of the same family (four CTAs per plane): the
// grafted instances' views in sweep order (Ng non-increasing), by value.
template <int CAP> struct Graft128TableT {
  GraftMixInst inst[CAP];
  int nz;
};
cudaError_t launch_mix_graft_plane128(const GraftMixInst *insts, int ninst, int nz, const void *tw64,
                                      const void *tw128, int sweep, int n, cudaStream_t st);
cudaError_t launch_mix_graft_plane(const LaunchShape &ls, const PropJob *jobs, int njobs, const GraftMixInst *insts,
                                   const DevGeom *geoms, const void *tw, int sweep, int n, cudaStream_t st);
cudaError_t launch_mix_graft_finalize(const FieldInst *fi, int ninst, int blocks, double2 *part, cudaStream_t st);
cudaError_t launch_mix_smear(const FieldInst *fi, int ninst, int blocks, cudaStream_t st);
cudaError_t launch_mix_update(const FieldInst *fi, int ninst, int blocks, cudaStream_t st);
cudaError_t launch_mix_boltzmann(const FieldInst *fi, int ninst, int blocks, cudaStream_t st);
cudaError_t launch_mix_q_finalize(const FieldInst *fi, int ninst, cudaStream_t st);
cudaError_t launch_mix_rho_pack(const FieldInst *fi, int ninst, int blocks, int keep, cudaStream_t st);
cudaError_t launch_mix_h_partials(const FieldInst *fi, int ninst, int blocks, double2 *out, cudaStream_t st);

}  // namespace scft
