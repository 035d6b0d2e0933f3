// inst.h -- per-instance device views used by the propagator and field kernels.
#pragma once

#include "common.h"

namespace scft {

// Device scalars of one instance (double2 slots).
enum ScalarSlot {
  kQd = 0,       // Q of the diblock (code/diblock_discrete.cpp:87)
  kFactor = 1,   // nD / Q / V (code/calc_poly_density.cpp:176)
  kQga = 2,      // Qga_exp (code/grafted_nanoparticle.cpp:112)
  kQg = 3,       // graft propagator check: count of points with Re q_g[Ng-1] <= 0 in .x
  kSmean = 4,    // mixed form: means of smwa (.x) and smwb (.y), kept out of the FP32 transform
  kSmean32 = 5,  // the same as two-float pairs (hi, lo of smwa, hi, lo of smwb) in the slot's 16 bytes
  kFactor32 = 6, // mixed form: nD / Q / V * 2^Kref as an FP32 mantissa (bytes 0-3) and exponent (int, bytes 4-7)
  kNumScalars = 7
};

// View of one instance for the propagator sweeps.  Propagator p = 0 is q
// (starts at the A end), p = 1 is q-dagger (starts at the B end).
struct PropInst {
  int geom;
  int N, Na;
  int single;  // q-dagger equals q (Na == 0 or Na == N, code/diblock_discrete.cpp:60-83)
  int hmax;    // last history slot kept: (N-1)/2
  void *work[2];
  void *hist[2];
  const double2 *expw[2];  // e^{-W_A}, e^{-W_B}
  double2 *acc[2][2];      // density accumulators [p][A or B]
  double2 *qpart;          // [nz] plane sums of q_{N-1}
  // grafted chains on explicit plates (code/grafted_nanoparticle.cpp:15-117)
  int graft, Ng;
  void *gwork;             // working array of the graft sweeps
  void *ghist;             // q_g, all Ng steps
  double2 *gacc;           // sum_j q_g[j] qdag_g[Ng-1-j]
  const double2 *gexpw;    // e^{-smwg}
  const double2 *grafts;   // normalised graft map (real space)
};

// View of one instance for the mixed-precision propagator sweep: q and qdag
// packed as the real and imaginary parts of one FP32 complex array.
struct MixInst {
  int geom, N, Na, hmax;
  float2 *work;    // z = q + i qdag of the current step
  float2 *hist;    // steps 0..hmax
  const float2 *E; // (e^{-smwa}, e^{-smwb})
  float *acc[2];   // density sums for A and B, scaled by 2^-K[2N]
  double *part;    // [2][N][nz] plane sums of the stored q, qdag (FP64)
  int *K;          // [2][N] power-of-two exponents, then K[2N] = reference exponent of acc
};

// View of one grafted instance for the mixed-precision graft sweeps
// (code/grafted_nanoparticle.cpp:15-117): q_g from the free end, all Ng steps
// stored (real, FP32), then qdag_g from the grafting surface, paired with
// the stored steps into the graft density.  The working array is complex FP32
// with imaginary part zero (a real field through the complex transform).
struct GraftMixInst {
  int geom, Ng;
  float2 *work;
  float *hist;            // [Ng][M] q_g, scaled by 2^-K[0][n]
  const float *Eg;        // e^{-smwg}
  float *acc;             // sum_j q_g[Ng-1-j] qdag_g[j] (true scale)
  double *part;           // [2][Ng][nz] FP64 plane sums of q_g, qdag_g
  int *K;                 // [2][Ng] power-of-two exponents
  const double2 *grafts;  // normalised graft map
};

struct PropJob {
  int inst;
  int p;
  int z;
};

// View of one instance for the field-level kernels.
struct FieldInst {
  long long M;
  int geom;
  double rho0, kappa, cab, cbc, cac;
  double ikappa;  // 1/kappa, 0 for kappa <= 0 (no w+^2 term)
  int euler;      // explicit Euler update (code/Euler_update.cpp) instead of 1S
  int neg_ab, neg_bc, neg_ac;
  double phiD, phiG, lam_pl, lam_mi, nD, V, dx[3];
  int N, Ng, np_chem, graft, single;
  double ng_per_np;
  int n_exp_nr;
  double2 *w[7];       // wpl, wabp, wabm, wbcp, wbcm, wacp, wacm
  double2 *sm[3];      // w_A, w_B, w_G, smeared in place into smwa, smwb, smwg
  double2 *rho[3];     // rhoda, rhodb, rhog_exp
  double2 *expw[3];    // e^{-smwa}, e^{-smwb}, e^{-smwg}
  const double *hhat, *gaa, *gab, *gbb, *gc, *rho_exp_nr;
  const double2 *exp_nrH;
  const double *shellU;  // A-segment shell potential (extension), or NULL
  double2 *acc[2][2];
  double2 *qpart;
  int nz;
  double2 *scal;       // kNumScalars device scalars
  double2 *gacc;       // graft density accumulator
  const double2 *ghist_last;  // q_g[Ng-1]
  const double2 *grafts;
  // mixed precision: w[] hold the k-space (1/M scaled) fields
  int nx, ny;
  // FP32 field-transform array: rho_A + i rho_B (real space), then its
  // transform; then hhat*(w_A + i w_B) (k-space) with the k = 0 term moved to
  // scal[kSmean] in FP64, then smwa + i smwb minus their means (real space)
  float2 *z32;
  float2 *E32;         // (e^{-smwa}, e^{-smwb})
  float *acc32[2];     // density sums, scaled by 2^-K[2N]
  int *K;              // [2][N] + 1
  double *part64;      // [2][N][nz] plane sums of the stored propagators
  // mixed precision, grafted instances: zg = rho_g (real space), then its
  // transform, then hhat w_G (k-space), then smwg (real space)
  double2 *zg;
  float *Eg32;           // e^{-smwg}
  float *gacc32;         // graft density sum (true scale)
  const float *ghist32_last;  // q_g[Ng-1], scaled by 2^-gK[Ng-1]
  const int *gK;
  // complex Langevin: k-space noise added to the update numerator of field f
  // (NULL: none); several fields may share one array, as in the reference
  const double2 *eta[7];
  // mixed precision: the 1S update of field f is w <- alpha_f(k) w - beta_f(k) F_f(k)
  // (NULL for fields whose chi is zero)
  const double *alpha[7], *beta[7];
};

}  // namespace scft
