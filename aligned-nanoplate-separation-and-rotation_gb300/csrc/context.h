// context.h -- host-side state of an scft_ctx.
#pragma once

#include <cuda.h>

#include <complex>
#include <string>
#include <vector>

#include "../../include/scft.h"
#include "common.h"
#include "inst.h"
#include "launch.h"
#include "refrng.h"

#include <nvtx3/nvToolsExt.h>

// A named NVTX range for the lifetime of the object (no cost without a
// profiler attached): the library's phases show up as ranges in profiler
// timelines and can filter ncu captures (ncu --nvtx --nvtx-include).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

namespace scft {

typedef std::complex<double> cd;

struct Instance {
  scft_params p;
  // complex Langevin: the reference's random stream and the noise arrays in
  // the order the reference draws them (w+, then + and - of AB, BC, AC)
  scft::RefRng rng;
  double2 *eta[7] = {};        // device, real space then k-space
  double2 *eta_host = nullptr;  // pinned staging, 7 x M
  scft_info info;
  int N, Na, Ng;
  double fD, Rg2, cab, cbc, cac;
  int neg_ab, neg_bc, neg_ac;
  int graft;   // sigma > 0, Ng > 0 and explicit plates present
  int single;  // q-dagger equals q
  int hmax;
  int geom;
  long long M;
  // device arrays (complex FP64 unless noted)
  double2 *w[7] = {};
  double2 *sm[3] = {};
  double2 *rho[3] = {};
  double2 *expw[3] = {};
  double2 *acc[2][2] = {};
  double2 *work[2] = {};
  double2 *hist[2] = {};
  double2 *qpart = nullptr;
  double2 *scal = nullptr;
  double2 *exp_nrH = nullptr;
  double2 *grafts = nullptr;  // expl_grafts (real space)
  double *hhat = nullptr, *gaa = nullptr, *gab = nullptr, *gbb = nullptr, *gc = nullptr;
  double *pbond = nullptr, *rho_exp_nr = nullptr;
  double2 *gwork = nullptr, *ghist = nullptr, *gacc = nullptr;  // graft sweeps
  // mixed precision
  int mixed = 0;
  float2 *z32 = nullptr;  // FP32 field-transform array (FieldInst::z32)
  // mixed form with grafts
  double2 *zg = nullptr;
  float *Eg32 = nullptr, *ghist32 = nullptr, *gacc32 = nullptr;
  float2 *gwork32 = nullptr;
  int *gK = nullptr;
  double *gpart = nullptr;
  float2 *E32 = nullptr, *work32 = nullptr, *hist32 = nullptr;
  float *acc32[2] = {};
  double *part = nullptr;
  int *K = nullptr;
  float *h32 = nullptr;    // 1 - g(k), FP32
  double *shellU = nullptr;  // Lambda * shell profile on A segments (extension), real, or NULL
  float *htab32 = nullptr;  // [hx | hy | hz], h_d = 1 - exp(-k_d^2/6), FP32
  double *alpha[7] = {}, *beta[7] = {};  // tabulated 1S coefficients (mixed form)
};

struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
};

struct scft_ctx_impl;

}  // namespace scft

struct scft_ctx {
  int device = 0;
  cudaStream_t st = nullptr;
  std::vector<scft::Instance> inst;
  std::vector<scft::DevGeom> geoms;
  scft::DevGeom *d_geoms = nullptr;
  void *d_tw64 = nullptr;
  std::vector<void *> allocs;  // every cudaMalloc of this context
  scft::FieldInst *d_fi = nullptr;
  scft::PropInst *d_pi = nullptr;
  // job lists (device) and their shapes
  scft::PlaneJob *d_pj_upd = nullptr, *d_pj_fld = nullptr, *d_pj_sm = nullptr;
  int n_pj_upd = 0, n_pj_fld = 0, n_pj_sm = 0;
  scft::ColJob *d_cj_upd = nullptr, *d_cj_fld = nullptr, *d_cj_sm = nullptr;
  int n_cj_upd = 0, n_cj_fld = 0, n_cj_sm = 0;
  scft::PropJob *d_prop_pj = nullptr;
  scft::ColJob *d_prop_cj = nullptr;
  std::vector<int> prop_pj_count, prop_cj_count;  // jobs active at step n (prefix counts)
  int nmax = 0;
  scft::PropJob *d_graft_pj = nullptr;
  scft::ColJob *d_graft_cj = nullptr;
  std::vector<int> graft_pj_count, graft_cj_count;
  int ngmax = 0;
  double2 *d_gpart = nullptr;
  int gblocks = 0;
  // mixed precision
  int mixed = 0;
  int xy64 = 0;          // every instance has 64 x 64 xy planes and the same nz: specialised plane pass
  int colfast = 0;       // xy64 with nz = 64 or 128: specialised z pass
  // every instance has 128 x 128 xy planes and the same nz (64, 128 or 256):
  // the four-CTA cluster plane pass with parity-major k-space planes and the
  // specialised z pass (kernels_mixed128.cu)
  int xy128 = 0;
  void *d_tw32_128 = nullptr;           // the 128-point twiddle table inside d_tw32
  scft::ColJob *d_mix128_cj_tx[3] = {};  // z-pass jobs of the 128 x 128 kernels for 8, 16, 32 columns per CTA
  // graft sweep of the 128 x 128 family: views of the grafted instances in
  // sweep order (Ng non-increasing) and their z-pass jobs
  std::vector<scft::GraftMixInst> gmi128;
  scft::ColJob *d_mix128_gcj_tx[3] = {};
  void *d_tw32_z = nullptr;  // twiddles of that nz
  void *d_tw32_64 = nullptr;  // the 64-point twiddle table inside d_tw32
  void *d_tw32 = nullptr;
  scft::ColJob *d_mix64_cj_tx[3] = {};  // z-pass jobs of the 64^3 kernels for 8, 16, 32 columns per CTA
  int col64_tx = 16;                      // columns per CTA of the 64^3 z pass
  // the sweep of a group of 64 x 64 x 64 instances as one persistent launch
  // (k_mix_sweep64) instead of two launches per step; its task counters
  // (sweep64_counters(kMix64MaxInst) per group) and the CTAs resident at once
  int sweep_persistent = 0;
  // plane pass of the 64-point family: 0 = block-barrier exchanges
  // (k_mix_plane64), 1 = warp-local columns (k_mix_plane64w); bit-identical
  int plane64_form = 0;
  unsigned *d_sweep_ctr = nullptr;
  int sweep_ctr_groups = 0;
  int sweep64_cap = 0;
  scft::MixInst *d_mi = nullptr;
  scft::GraftMixInst *d_gmi = nullptr;  // per instance (zero for instances without grafts)
  std::vector<scft::MixInst> h_mi;       // host copy of d_mi
  std::vector<scft::GraftMixInst> h_gmi;  // host copy of d_gmi
  std::vector<scft::MixInst> mix64_tab;  // instances in job order (64^3 plane pass)
  std::vector<CUtensorMap> tmE, tmH;      // their TMA descriptors (Boltzmann, history)
  // d_err[0]: error word of the plane passes (1: an mbarrier wait ran out;
  // 2: a dependency wait of the persistent sweep ran out);
  // d_err[1]: polls of each plane-pass CTA's first mbarrier wait before it
  // records a timeout (kWaitPolls); d_err[2]: polls of a dependency wait
  // (kSpinPolls); scft_set_wait_limit lowers both
  int *d_err = nullptr;
  double *h_pin = nullptr;                // pinned read-back of the field checks (128 doubles per instance)
  // scft_set_fields (mixed form): check results, instance mask, job staging
  double *d_realout = nullptr;
  int *d_skip = nullptr, *h_skip = nullptr;
  char *d_jobs = nullptr;
  void *h_jobs = nullptr;
  size_t jobs_cap = 0;
  // The mixed sweep of a batch runs as `groups` independent chains of
  // launches on side streams (contiguous instance ranges in job order), so
  // that one group's column passes fill the last wave of another group's
  // plane pass; all of it sits in one captured graph.
  // Phases run one after another (each phase's working set can stay in L2);
  // the groups of one phase run concurrently.
  // fast: the group's instances are 64^3 grids of a batch of mixed grids and
  // run on the 64-point plane and z kernels (a batch of 64 x 64 planes only
  // uses them throughout: xy64)
  struct SweepGroup {
    int inst_begin, inst_end, pj_begin, pj_end, cj_begin, cj_end, phase, fast, fast96, fast48;
  };
  std::vector<SweepGroup> groups;
  int sweep_phases = 1;  // requested number of sequential phases
  std::vector<int> job_order, inst_pj_end, inst_cj_end;  // mixed job lists, by instance
  // batch of mixed grids: fast64[oi] = 1 for the 64^3 instances (job-order
  // position oi), which come first in job order; anyfast = some instance is one
  std::vector<char> fast64;
  int anyfast = 0;
  // batch with 96 x 64 x 64 instances: fast96[oi] = 1 for those (after the
  // 64^3 ones in job order), run by the three-CTA cluster plane pass
  // (kernels_mixed96.cu) and the 64-point z pass; first96 = job-order
  // position of the first of them
  std::vector<char> fast96;
  int any96 = 0, first96 = 0;
  // the same for 48 x 48 x 48 instances (after the 96 x 64 x 64 ones), run
  // by the 48-point plane and z passes (kernels_mixed48.cu)
  std::vector<char> fast48;
  int any48 = 0, first48 = 0;
  void *d_tw32_48 = nullptr;           // the 48-point twiddle table inside d_tw32
  scft::ColJob *d_mix48_cj = nullptr;  // their z-pass jobs (16 columns per CTA)
  void *d_tw32_32 = nullptr, *d_tw32_96 = nullptr;  // 32- and 96-point twiddle tables inside d_tw32
  scft::ColJob *d_mix96_cj_tx[3] = {};               // their z-pass jobs for 8, 16, 32 columns per CTA
  // mixed field-level data in job order: FieldInst table, the FP32 transform
  // jobs of z32 and the FP64 ones of zg (grafted instances); fld_end[4 oi + k]
  // = end of instance oi's jobs in list k (z32 plane, z32 column, zg plane,
  // zg column); the same lists serve both directions
  std::vector<scft::FieldInst> h_fi;
  scft::FieldInst *d_fi_ord = nullptr;
  scft::PlaneJob *d_zpj_ord = nullptr, *d_gpj_ord = nullptr;
  scft::ColJob *d_zcj_ord = nullptr, *d_gcj_ord = nullptr;
  std::vector<int> fld_end;
  int sweep_streams = 2;  // requested number of groups (1 = a single chain)
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> ev_join;
  std::vector<cudaEvent_t> ev_up;  // host-field calls: end of a group's uploads
  double2 *h_hsum = nullptr;  // host-field calls: pinned H partial sums (job order), then scalars (instance order)
  cudaEvent_t ev_fork = nullptr;
  scft::LaunchShape shp_mix{}, shp_col32{}, shp_plane32{};
  scft::LaunchShape shp_mixg{};  // mixed plane passes in place (shp_mix; 1024 threads for the largest planes)
  scft::LaunchShape shp_mixp{};  // generic mixed plane pass (out of place and staged where it fits, else shp_mixg)
  scft::LaunchShape shp_plane{}, shp_col{}, shp_prop{};
  int eblocks = 0;  // blocks per instance for pointwise kernels
  double2 *d_hpart = nullptr;
  int hblocks = 0;
  // scft_step_fields / scft_iterate_fields: the captured graph of the last
  // such call (uploads, checks, transforms, density builds, updates,
  // downloads), keyed by the call, its host pointers and iteration count; the
  // per-group FP64 transform jobs of the uploaded fields (job-order groups)
  // and, per group and round of three fields, the inverse transform jobs of
  // the downloaded fields (on the instances' rho[0..2] as scratch)
  cudaGraphExec_t g_step = nullptr;
  std::vector<const void *> step_ptrs;
  int step_iters = 0;
  std::vector<scft::PlaneJob *> step_pj;
  std::vector<scft::ColJob *> step_cj;
  std::vector<int> step_npj, step_ncj;
  std::vector<scft::PlaneJob *> out_pj;  // [3 * group + round]
  std::vector<scft::ColJob *> out_cj;
  std::vector<int> out_npj, out_ncj;
  std::vector<int> step_groups_sig;  // group boundaries the job lists were built for
  cudaGraphExec_t g_update = nullptr;
  cudaGraphExec_t g_density = nullptr;  // captured density build (after the first, eager one)
  long long launches_per_density = 0;
  int density_runs = 0;
  long long launches = 0;            // kernel launches issued (graph replays included)
  long long launches_per_update = 0;  // kernels in one captured update_1s iteration
  int update_runs = 0;
  int dirty_density = 1;
};
