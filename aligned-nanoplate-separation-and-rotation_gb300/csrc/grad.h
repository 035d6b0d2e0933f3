// grad.h -- arguments of the geometric-derivative kernel.
#pragma once

#include <cuda_runtime.h>

namespace scft {

// per plate: for g in (theta_z, c_x, c_y, c_z): sum d rho_p/dg * Re w+,
// sum d rho_p/dg * Im w+, sum d rho_p/dg
constexpr int kGradPerPlate = 12;

struct GradArgs {
  int nx, ny, nz, nplates;
  double dx[3], L[3];
  double c[2][3];  // absolute centres
  double u[2][3];  // unit axes
  double len, rad, xi;
};

cudaError_t launch_geom_grad(const GradArgs &g, const double2 *wpl, double *part, int blocks, cudaStream_t st);

}  // namespace scft
