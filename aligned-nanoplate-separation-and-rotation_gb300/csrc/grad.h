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
  int shape;              // SCFT_PLATE_REFERENCE or SCFT_PLATE_CUBOID
  int shell;              // shell potential present
  double len_big, rad_big;  // enlarged plate of the shell
};

cudaError_t launch_geom_grad(const GradArgs &g, const double2 *wpl, const double2 *rhoA, double *part, int blocks,
                             cudaStream_t st);

// Grafted plates (kernels_grad.cu): d rho^big_j / d g_k as a complex field;
// L = masked log q_g[Ng-1]; block sums (4 doubles per block) of the graft
// map's derivative terms for one plate (gd == NULL: of |grad rho_j^big|).
cudaError_t launch_plate_deriv(double2 *out, const GradArgs &g, int j, int k, double len, double rad,
                               cudaStream_t st);
cudaError_t launch_graft_log(double2 *L, const double2 *grafts, const double2 *q64, const float *q32, int K,
                             long long M, cudaStream_t st);
cudaError_t launch_graft_dmap(const double2 *const *gr, const double2 *const *gd, const double2 *L, long long M,
                              double *part, int blocks, cudaStream_t st);

}  // namespace scft
