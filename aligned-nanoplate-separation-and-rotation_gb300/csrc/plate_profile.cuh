// plate_profile.cuh -- the explicit plate's core density and its derivatives
// with respect to the plate's rotation about z and its centre.
//
// Two shapes, both functions of the minimum-image offset dr = r - c and the
// unit axis u (plate normal):
//   SCFT_PLATE_REFERENCE: the reference's particle (code/initialize.cpp:578-612)
//     rho_p = 1/4 erfc((|u.dr| - L/2)/xi) erfc((|u x dr| - R)/xi);
//   SCFT_PLATE_CUBOID (extension, no reference counterpart): a slab of
//     thickness L along u and a 2R x 2R square in the plane,
//     rho_p = 1/8 erfc((|u.dr| - L/2)/xi) erfc((|e1.dr| - R)/xi) erfc((|e2.dr| - R)/xi)
//     with e1 = (u x z)/|u x z| when |u_z| < 0.9, else (u x x)/|u x x|, and
//     e2 = u x e1.
// The derivatives are those of these formulas: a rotation about z moves u by
// du/dtheta = z x u and e1, e2 with it (rigidly on the first branch of e1;
// on the second the normalisation of u x x is differentiated).
#pragma once

#include <cuda_runtime.h>

#include "scft.h"

namespace scft {

__device__ __forceinline__ double plate_derfc(double x) {
  // d/dx erfc(x) = -2/sqrt(pi) exp(-x^2)
  return -1.1283791670955125738961589031215452 * exp(-x * x);
}

__device__ __forceinline__ void cross3(const double a[3], const double b[3], double o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// In-plane axes e1, e2 of the cuboid with axis u; with de1, de2 != NULL also
// their derivatives with respect to a rotation of u about z.
__device__ __forceinline__ void cuboid_frame(const double u[3], double e1[3], double e2[3], double *de1,
                                             double *de2) {
  double t[3], dt[3];
  const bool first = fabs(u[2]) < 0.9;
  if (first) {  // u x z
    t[0] = u[1]; t[1] = -u[0]; t[2] = 0.0;
    dt[0] = u[0]; dt[1] = u[1]; dt[2] = 0.0;
  } else {  // u x x
    t[0] = 0.0; t[1] = u[2]; t[2] = -u[1];
    dt[0] = 0.0; dt[1] = 0.0; dt[2] = -u[0];
  }
  const double n1 = sqrt(dot3(t, t));
  for (int d = 0; d < 3; d++) e1[d] = t[d] / n1;
  cross3(u, e1, e2);
  if (de1 == nullptr) return;
  const double pr = dot3(e1, dt);
  for (int d = 0; d < 3; d++) de1[d] = (dt[d] - e1[d] * pr) / n1;
  const double du[3] = {-u[1], u[0], 0.0};
  double a[3], b[3];
  cross3(du, e1, a);
  cross3(u, de1, b);
  for (int d = 0; d < 3; d++) de2[d] = a[d] + b[d];
}

// rho_p at offset dr.
__device__ __forceinline__ double plate_value(int shape, const double dr[3], const double u[3], double len,
                                              double rad, double xi) {
  if (shape == SCFT_PLATE_CUBOID) {
    double e1[3], e2[3];
    cuboid_frame(u, e1, e2, nullptr, nullptr);
    const double p0 = dot3(u, dr), p1 = dot3(e1, dr), p2 = dot3(e2, dr);
    return 0.125 * erfc((fabs(p0) - 0.5 * len) / xi) * erfc((fabs(p1) - rad) / xi) * erfc((fabs(p2) - rad) / xi);
  }
  double c[3];
  cross3(u, dr, c);
  const double udr = dot3(u, dr);
  const double ucr = sqrt(dot3(c, c));
  return 0.25 * erfc((fabs(udr) - 0.5 * len) / xi) * erfc((fabs(ucr) - rad) / xi);
}

// d rho_p/dg at offset dr for g = (theta_z, c_x, c_y, c_z).
__device__ __forceinline__ void plate_derivs(int shape, const double dr[3], const double u[3], double len, double rad,
                                             double xi, double dg[4]) {
  const double du[3] = {-u[1], u[0], 0.0};  // rotation about z: du/dtheta = z x u
  if (shape == SCFT_PLATE_CUBOID) {
    double e[3][3], de[3][3];
    for (int d = 0; d < 3; d++) {
      e[0][d] = u[d];
      de[0][d] = du[d];
    }
    cuboid_frame(u, e[1], e[2], de[1], de[2]);
    const double half[3] = {0.5 * len, rad, rad};
    double F[3], dF[3];  // erfc factors and their derivatives with respect to p_i = e_i.dr
    for (int i = 0; i < 3; i++) {
      const double p = dot3(e[i], dr);
      const double a = (fabs(p) - half[i]) / xi;
      const double sg = p > 0.0 ? 1.0 : (p < 0.0 ? -1.0 : 0.0);
      F[i] = erfc(a);
      dF[i] = sg * plate_derfc(a) / xi;
    }
    const double w[3] = {dF[0] * F[1] * F[2], F[0] * dF[1] * F[2], F[0] * F[1] * dF[2]};
    // dp_i/dtheta = de_i.dr; dp_i/dc_k = -e_i[k]
    dg[0] = 0.125 * (w[0] * dot3(de[0], dr) + w[1] * dot3(de[1], dr) + w[2] * dot3(de[2], dr));
    for (int k = 0; k < 3; k++) dg[1 + k] = -0.125 * (w[0] * e[0][k] + w[1] * e[1][k] + w[2] * e[2][k]);
    return;
  }
  const double ud = dot3(u, dr);
  double c[3];
  cross3(u, dr, c);
  const double uc = sqrt(dot3(c, c));
  const double a = (fabs(ud) - 0.5 * len) / xi, b = (uc - rad) / xi;
  const double Ea = erfc(a), Eb = erfc(b);
  const double dEa = plate_derfc(a) / xi, dEb = plate_derfc(b) / xi;  // d/d|u.dr|, d/d|u x dr|
  const double sg = ud > 0.0 ? 1.0 : (ud < 0.0 ? -1.0 : 0.0);
  const double dudr = dot3(du, dr);
  const double dud_dth = sg * dudr;
  const double duc_dth = uc > 1e-300 ? -ud * dudr / uc : 0.0;
  dg[0] = 0.25 * (dEa * dud_dth * Eb + Ea * dEb * duc_dth);
  // centre: d dr / d c_k = -e_k
  for (int k = 0; k < 3; k++) {
    const double dud_dc = -sg * u[k];
    const double duc_dc = uc > 1e-300 ? -(dr[k] - ud * u[k]) / uc : 0.0;
    dg[1 + k] = 0.25 * (dEa * dud_dc * Eb + Ea * dEb * duc_dc);
  }
}

}  // namespace scft
