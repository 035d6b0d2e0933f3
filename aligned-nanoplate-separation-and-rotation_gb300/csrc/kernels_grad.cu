// kernels_grad.cu -- geometric derivatives of H with respect to the plates.
//
// The plate core density rho_p (code/initialize.cpp:578-612, or the cuboid
// extension; plate_profile.cuh), a function of dr = r - c (minimum image),
// enters H at fixed fields through
//   -i rho0 int (1 - rho_p) w+           (code/calc_h.cpp:66-87)
//   -nD log Qd with nD = rho0 (Vf - V_exp - phiG Vf)/N, V_exp = int rho_p
//                                          (code/initialize.cpp:251-351),
// so dH/dg = i rho0 int (d rho_p/dg) w+ + (rho0/N) log Qd int (d rho_p/dg)
// for g = a rotation angle of the plate axis u about z (du/dtheta = z x u) or
// a centre coordinate.  With the shell potential U_A = Lambda (rho_big -
// rho_p) on A segments (an extension), -nD log Qd depends on the plate
// through U_A as well: its derivative with respect to U_A(r) is rho_A(r), so
// dH/dg gains Lambda int rho_A d(rho_big - rho_p)/dg.  This kernel forms, per
// plate, the grid sums of d rho_p/dg * w+, of d rho_p/dg and of the shell
// terms (FP64); the host assembles dH/dg.
#include "fft_core.cuh"
#include "grad.h"
#include "plate_profile.cuh"

namespace scft {

__global__ void k_geom_grad(GradArgs g, const double2 *__restrict__ wpl, const double2 *__restrict__ rhoA,
                            double *__restrict__ part) {
  __shared__ double red[32];
  double acc[kGradPerPlate * 2];
  for (int k = 0; k < kGradPerPlate * 2; k++) acc[k] = 0.0;
  const long long M = (long long)g.nx * g.ny * g.nz;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    const int n[3] = {(int)(i % g.nx), (int)((i / g.nx) % g.ny), (int)(i / ((long long)g.nx * g.ny))};
    const double2 w = wpl[i];
    const double ra = g.shell ? rhoA[i].x : 0.0;
    for (int j = 0; j < g.nplates; j++) {
      double dr[3];
      for (int d = 0; d < 3; d++) {
        double r = double(n[d]) * g.dx[d] - g.c[j][d];
        if (r >= 0.5 * g.L[d]) r -= g.L[d];
        else if (r < -0.5 * g.L[d]) r += g.L[d];
        dr[d] = r;
      }
      double dg[4], db[4];
      plate_derivs(g.shape, dr, g.u[j], g.len, g.rad, g.xi, dg);
      if (g.shell) plate_derivs(g.shape, dr, g.u[j], g.len_big, g.rad_big, g.xi, db);
      for (int k = 0; k < 4; k++) {
        double *a = acc + j * kGradPerPlate + kGradTerms * k;
        a[0] += dg[k] * w.x;
        a[1] += dg[k] * w.y;
        a[2] += dg[k];
        if (g.shell) {
          a[3] += db[k] * ra;
          a[4] += dg[k] * ra;
        }
      }
    }
  }
  const int nv = g.nplates * kGradPerPlate;
  for (int k = 0; k < nv; k++) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int wp = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[wp] = v;
    __syncthreads();
    if (wp == 0) {
      v = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (l == 0) part[(long long)blockIdx.x * nv + k] = v;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Grafted plates: the graft map g = G / S, G = sum_j |grad rho_j^big| (rho_j^big
// the 1.05x-enlarged plate, spectral gradient; code/initialize.cpp:160-200),
// S = int G, enters H through -n_exp_nr ng_per_np Re Qga with
// Qga = int g L, L = log q_g[Ng-1] where Re g > 0 and 0 elsewhere
// (code/grafted_nanoparticle.cpp:82-112; q_g does not depend on the plates
// at fixed fields).  So dQga/dg_k = (int dG_k L - Qga int dG_k) / S with
// dG_k = sum_d (d_d rho_j^big)(d_d drho_j^big/dg_k) / |grad rho_j^big| for the
// plate j that g_k moves.
// ---------------------------------------------------------------------------

// out = d rho^big_j / d g_k (real), g_k = (theta_z, c_x, c_y, c_z)[k], for a
// plate of thickness len and radius rad.
__global__ void k_plate_deriv(double2 *out, GradArgs g, int j, int k, double len, double rad) {
  const long long M = (long long)g.nx * g.ny * g.nz;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    const int n[3] = {(int)(i % g.nx), (int)((i / g.nx) % g.ny), (int)(i / ((long long)g.nx * g.ny))};
    double dr[3];
    for (int d = 0; d < 3; d++) {
      double r = double(n[d]) * g.dx[d] - g.c[j][d];
      if (r >= 0.5 * g.L[d]) r -= g.L[d];
      else if (r < -0.5 * g.L[d]) r += g.L[d];
      dr[d] = r;
    }
    double dg[4];
    plate_derivs(g.shape, dr, g.u[j], len, rad, g.xi, dg);
    out[i] = make_double2(dg[k], 0.0);
  }
}

// L = log q_g[Ng-1] where Re g > 0, else 0; q_g from the FP64 history (q64)
// or the FP32 one (q32, stored scaled by 2^-K).
__global__ void k_graft_log(double2 *L, const double2 *__restrict__ grafts, const double2 *__restrict__ q64,
                            const float *__restrict__ q32, int K, long long M) {
  const double ln2 = 0.69314718055994530941723212145817657;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    double2 v = make_double2(0.0, 0.0);
    if (grafts[i].x > 0.0) {
      if (q64) {
        const double2 q = q64[i];
        v = make_double2(log(hypot(q.x, q.y)), atan2(q.y, q.x));
      } else {
        v = make_double2(log((double)q32[i]) + K * ln2, 0.0);
      }
    }
    L[i] = v;
  }
}

// Block partial sums for one plate: part[4 b + {0, 1}] = sum dG L (complex),
// part[4 b + {2, 3}] = sum dG (complex) with dG as above from the plate's
// gradient gr[3] and the gradient gd[3] of its derivative field; with
// gd == NULL, part[4 b + {2, 3}] = sum |grad rho_j^big| (for S).
__global__ void k_graft_dmap(const double2 *__restrict__ gr0, const double2 *__restrict__ gr1,
                             const double2 *__restrict__ gr2, const double2 *__restrict__ gd0,
                             const double2 *__restrict__ gd1, const double2 *__restrict__ gd2,
                             const double2 *__restrict__ L, long long M, double *part) {
  __shared__ double red[4][32];
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    const double2 a0 = gr0[i], a1 = gr1[i], a2 = gr2[i];
    const double2 G = csqrt_d(cadd(cadd(cmul(a0, a0), cmul(a1, a1)), cmul(a2, a2)));
    if (!gd0) {
      s[2] += G.x;
      s[3] += G.y;
      continue;
    }
    if (G.x == 0.0 && G.y == 0.0) continue;
    const double2 num = cadd(cadd(cmul(a0, gd0[i]), cmul(a1, gd1[i])), cmul(a2, gd2[i]));
    // num / G (Smith's division)
    double2 dG;
    if (fabs(G.x) >= fabs(G.y)) {
      const double r = G.y / G.x, den = G.x + G.y * r;
      dG = make_double2((num.x + num.y * r) / den, (num.y - num.x * r) / den);
    } else {
      const double r = G.x / G.y, den = G.x * r + G.y;
      dG = make_double2((num.x * r + num.y) / den, (num.y * r - num.x) / den);
    }
    const double2 t = cmul(dG, L[i]);
    s[0] += t.x;
    s[1] += t.y;
    s[2] += dG.x;
    s[3] += dG.y;
  }
  const int wp = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int k = 0; k < 4; k++) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (l == 0) red[k][wp] = v;
  }
  __syncthreads();
  if (wp == 0)
    for (int k = 0; k < 4; k++) {
      double v = l < (int)(blockDim.x >> 5) ? red[k][l] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (l == 0) part[4 * blockIdx.x + k] = v;
    }
}

cudaError_t launch_plate_deriv(double2 *out, const GradArgs &g, int j, int k, double len, double rad,
                               cudaStream_t st) {
  k_plate_deriv<<<1024, 256, 0, st>>>(out, g, j, k, len, rad);
  return cudaGetLastError();
}

cudaError_t launch_graft_log(double2 *L, const double2 *grafts, const double2 *q64, const float *q32, int K,
                             long long M, cudaStream_t st) {
  k_graft_log<<<1024, 256, 0, st>>>(L, grafts, q64, q32, K, M);
  return cudaGetLastError();
}

cudaError_t launch_graft_dmap(const double2 *const *gr, const double2 *const *gd, const double2 *L, long long M,
                              double *part, int blocks, cudaStream_t st) {
  k_graft_dmap<<<blocks, 256, 0, st>>>(gr[0], gr[1], gr[2], gd ? gd[0] : nullptr, gd ? gd[1] : nullptr,
                                       gd ? gd[2] : nullptr, L, M, part);
  return cudaGetLastError();
}

cudaError_t launch_geom_grad(const GradArgs &g, const double2 *wpl, const double2 *rhoA, double *part, int blocks,
                             cudaStream_t st) {
  k_geom_grad<<<blocks, 256, 0, st>>>(g, wpl, rhoA, part);
  return cudaGetLastError();
}

}  // namespace scft
