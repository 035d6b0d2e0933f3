// kernels_setup.cu -- per-instance k-space tables, built on the device at
// set-up (one thread per grid point): the smearing kernel hhat, the bond
// factor exp(-k^2/6) (and 1 - g(k) in FP32 for the mixed form), the Debye
// functions of the diblock and the grafted chains, and the mixed form's
// tabulated 1S / Euler coefficients.
//
//   get_k:           code/array_utils.cpp:239-272 (k_d = 2 pi n / L for
//                    n < N/2, else 2 pi (n - N) / L)
//   hhat:            code/initialize.cpp:97-102   exp(-k^2 a^2 / 2)
//   poly_bond_fft:   code/initialize.cpp:401-404  exp(-k^2 / 6)
//   gaa, gbb, gab:   code/calc_debye.cpp:5-51     with x = k^2 Rg^2 and the
//                    k = 0 limits fD^2, (1 - fD)^2, fD (1 - fD)
//   gc:              code/calc_debye.cpp:53-68    Debye function of a chain
//                    of Ng beads, 1 at k = 0
// The expressions are the reference's, evaluated in the same order, so the
// tables agree with its to the last bit or two (device exp against the host
// library's).
#include "kernels_setup.h"

namespace scft {

namespace {

constexpr double kPI_s = 3.14159265358979323846263383;  // code/globals.h:31

__global__ void k_setup_tables(SetupTableArgs a, double *hh, double *pb, double *gaa, double *gab, double *gbb,
                               double *gc, float *h32) {
  const long long M = (long long)a.nx * a.ny * a.nz;
  const int n3[3] = {a.nx, a.ny, a.nz};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
    int n[3];
    n[2] = (int)(i / a.ny / a.nx);
    n[1] = (int)(i / a.nx - (long long)n[2] * a.ny);
    n[0] = (int)(i - ((long long)n[1] + (long long)n[2] * a.ny) * a.nx);
    double k2 = 0.0;
    for (int d = 0; d < 3; d++) {
      const double k = (double(n[d]) < double(n3[d]) / 2.) ? 2 * kPI_s * double(n[d]) / a.L[d]
                                                           : 2 * kPI_s * double(n[d] - n3[d]) / a.L[d];
      k2 += k * k;
    }
    hh[i] = exp(-k2 * a.a2 / 2.0);
    const double b = exp(-k2 / 6.0);
    pb[i] = b;
    if (h32) h32[i] = (float)(1.0 - b);
    const double x = k2 * a.Rg2, fD = a.fD;
    if (i == 0) {
      gaa[i] = fD * fD;
      gbb[i] = (1.0 - fD) * (1.0 - fD);
      gab[i] = fD * (1.0 - fD);
    } else {
      gaa[i] = 2.0 * (exp(-x * fD) + fD * x - 1.0) / x / x;
      gbb[i] = 2.0 * (exp(-x * (1.0 - fD)) + (1.0 - fD) * x - 1.0) / x / x;
      gab[i] = (1.0 - exp(-x * fD)) * (1.0 - exp(-x * (1.0 - fD))) / x / x;
    }
    double g = 0.0;
    if (a.graft) {
      const double dm1 = k2 * a.Rg2 * a.alpha_c;
      g = (dm1 == 0.0) ? 1.0 : 2.0 * (exp(-dm1) + dm1 - 1.0) / dm1 / dm1;
    }
    gc[i] = g;
  }
}

// alpha, beta of the mixed form's update w <- alpha w - beta F per field
// (see MixCoeffArgs); the A(k) of each semi-implicit field is the
// reference's denominator term of code/1s_update.cpp:67-329.
__global__ void k_mix_coeff(MixCoeffArgs a, long long M, const double *__restrict__ hh,
                            const double *__restrict__ gaa, const double *__restrict__ gab,
                            const double *__restrict__ gbb, const double *__restrict__ gc) {
  const double rho0 = a.rho0, N = a.N, Ng = a.Ng, phiD = a.phiD, phiG = a.phiG;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
    const double h = hh[i];
    for (int f = 0; f < 7; f++) {
      const MixCoeffArgs::Field &F = a.f[f];
      if (F.kind == kCoeffNone) continue;
      double al, be;
      if (F.kind == kCoeffEuler) {
        al = 1.0 - F.lam * F.c;
        be = F.lam;
      } else if (F.kind == kCoeffExplicit) {
        const double d = 1.0 + F.lam * 2.0 * rho0 / F.c;
        al = 1.0 / d;
        be = F.lam / d;
      } else {
        double A;
        switch (F.formula) {
          case kAPlus:
            A = rho0 / a.kappa + phiD * rho0 * N * h * h * (gaa[i] + 2.0 * gab[i] + gbb[i]) +
                (phiG * Ng * gc[i]) * rho0 * h * h;
            break;
          case kAB:
            A = 2.0 * rho0 / F.c + phiD * rho0 * N * h * h * (gaa[i] + 2.0 * gab[i] + gbb[i]);
            break;
          case kABNeg:
            A = 2.0 * rho0 / F.c + phiD * rho0 * N * h * h * (gaa[i] - gbb[i]);
            break;
          case kBC:
            A = 2.0 * rho0 / F.c + phiD * rho0 * N * h * h * gbb[i] + phiG * rho0 * Ng * h * h * gc[i];
            break;
          case kBCNeg:
            A = 2.0 * rho0 / F.c + phiD * rho0 * N * h * h * gbb[i] - phiG * Ng * h * h * rho0 * gc[i];
            break;
          case kAC:
            A = 2.0 * rho0 / F.c + phiD * rho0 * N * h * h * gaa[i] + phiG * Ng * h * h * rho0 * gc[i];
            break;
          default:  // kACNeg
            A = 2.0 * rho0 / F.c + phiD * rho0 * N * h * h * gaa[i] - phiG * Ng * h * h * rho0 * gc[i];
            break;
        }
        const double B = A - F.boff;
        al = (1.0 + F.lam * B) / (1.0 + F.lam * A);
        be = F.lam / (1.0 + F.lam * A);
      }
      F.alpha[i] = al;
      F.beta[i] = be;
    }
  }
}

}  // namespace

cudaError_t launch_setup_tables(const SetupTableArgs &a, double *hh, double *pb, double *gaa, double *gab,
                                double *gbb, double *gc, float *h32, cudaStream_t st) {
  const long long M = (long long)a.nx * a.ny * a.nz;
  const int blocks = (int)((M + 255) / 256 < 4096 ? (M + 255) / 256 : 4096);
  k_setup_tables<<<blocks, 256, 0, st>>>(a, hh, pb, gaa, gab, gbb, gc, h32);
  return cudaGetLastError();
}

cudaError_t launch_mix_coeff(const MixCoeffArgs &a, long long M, const double *hh, const double *gaa,
                             const double *gab, const double *gbb, const double *gc, cudaStream_t st) {
  const int blocks = (int)((M + 255) / 256 < 4096 ? (M + 255) / 256 : 4096);
  k_mix_coeff<<<blocks, 256, 0, st>>>(a, M, hh, gaa, gab, gbb, gc);
  return cudaGetLastError();
}

}  // namespace scft
