// grad.h -- arguments of the geometric-derivative kernel.
#pragma once

#include <cuda_runtime.h>

namespace scft {

// per plate, for g in (theta_z, c_x, c_y, c_z):
//   sum d rho_p/dg * Re w+, sum d rho_p/dg * Im w+, sum d rho_p/dg,
//   sum d rho_big/dg * Re rho_A, sum d rho_p/dg * Re rho_A
// (the last two only with the shell potential; rho_big is the enlarged plate)
constexpr int kGradTerms = 5;
constexpr int kGradPerPlate = 4 * kGradTerms;

struct GradArgs {
  int nx, ny, nz, nplates;
  double dx[3], L[3];
  double c[2][3];  // absolute centres
  double u[2][3];  // unit axes
  double len, rad, xi;
  int shell;              // shell potential present
  double len_big, rad_big;  // enlarged plate of the shell
};

cudaError_t launch_geom_grad(const GradArgs &g, const double2 *wpl, const double2 *rhoA, double *part, int blocks,
                             cudaStream_t st);

}  // namespace scft
