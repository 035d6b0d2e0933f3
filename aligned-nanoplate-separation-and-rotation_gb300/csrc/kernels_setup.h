// kernels_setup.h -- launchers of the set-up table kernels (kernels_setup.cu).
#pragma once

#include <cuda_runtime.h>

namespace scft {

// One instance's grid, box and chain constants for its k-space tables.
struct SetupTableArgs {
  int nx, ny, nz;
  double L[3];
  double a2;       // smearing length squared
  double fD, Rg2;  // A fraction and Rg^2 = (N - 1) / 6 of the diblock
  double alpha_c;  // (Ng - 1) / (N - 1): grafted chain length in units of the diblock's
  int graft;       // sigma > 0: gc is the Debye function of the grafted chains (else 0)
};

// hh, pb, gaa, gab, gbb, gc: M doubles each; h32 (M floats, 1 - pb) or NULL.
cudaError_t launch_setup_tables(const SetupTableArgs &a, double *hh, double *pb, double *gaa, double *gab,
                                double *gbb, double *gc, float *h32, cudaStream_t st);

enum CoeffKind { kCoeffNone = 0, kCoeffSemi = 1, kCoeffExplicit = 2, kCoeffEuler = 3 };
// A(k) of a semi-implicit field (code/1s_update.cpp:67-329): w+, the
// semi-implicit member of each chi pair for chi > 0 and chi < 0.
enum CoeffFormula { kAPlus = 0, kAB, kABNeg, kBC, kBCNeg, kAC, kACNeg };

// Per field f of w <- alpha w - beta F (the mixed form's k-space update):
//   semi:     alpha = (1 + lam B) / (1 + lam A), beta = lam / (1 + lam A),
//             B = A - boff
//   explicit: alpha = 1 / d, beta = lam / d, d = 1 + lam 2 rho0 / c
//   Euler:    alpha = 1 - lam c, beta = lam          (code/Euler_update.cpp)
struct MixCoeffArgs {
  struct Field {
    int kind, formula;
    double lam, c, boff;
    double *alpha, *beta;
  } f[7];
  double rho0, kappa, N, Ng, phiD, phiG;
};

cudaError_t launch_mix_coeff(const MixCoeffArgs &a, long long M, const double *hh, const double *gaa,
                             const double *gab, const double *gbb, const double *gc, cudaStream_t st);

}  // namespace scft
