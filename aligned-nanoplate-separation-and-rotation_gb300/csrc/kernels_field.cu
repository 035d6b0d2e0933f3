// kernels_field.cu -- pointwise and reduction kernels of the plain FP64 method.
//
// All kernels take an array of FieldInst views and a 2-D grid: blockIdx.y is
// the instance, blockIdx.x strides over its M grid points.  Complex
// arithmetic follows the reference's std::complex<double> expressions term by
// term; where the reference divides by a complex number whose imaginary part
// is exactly zero (the 1S denominators), the division is done per component,
// which is what the complex division reduces to in that case.
#include "fft_core.cuh"
#include "inst.h"
#include "launch.h"
#include "prop_launch.h"

namespace scft {

__device__ __forceinline__ double2 cexp_d(double2 z) {
  double s, c;
  sincos(z.y, &s, &c);
  const double e = exp(z.x);
  return make_double2(e * c, e * s);
}

// Smith's algorithm for a / b.
__device__ __host__ __forceinline__ double2 cdiv_d(double2 a, double2 b) {
  if (fabs(b.x) < fabs(b.y)) {
    const double r = b.x / b.y, d = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
  const double r = b.y / b.x, d = b.y * r + b.x;
  return make_double2((a.y * r + a.x) / d, (a.y - a.x * r) / d);
}

#define FOR_POINTS(FI)                                                              \
  const FieldInst &FI = fi[blockIdx.y];                                             \
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < FI.M; \
       i += (long long)gridDim.x * blockDim.x)

// code/calc_poly_density.cpp:42-54: w_A, w_B, w_G from the seven fields
// (linear, so it applies equally to real-space values and to transforms).
__device__ __forceinline__ void assemble_point(const FieldInst &F, const double2 *w, double2 &wa, double2 &wb,
                                               double2 &wg) {
  {
    const double2 pl = w[0], abp = w[1], abm = w[2];
    const double2 bcp = w[3], bcm = w[4], acp = w[5], acm = w[6];
    // I*x = (-x.y, x.x)
    const double2 Ipl = make_double2(-pl.y, pl.x);
    double2 ab_a, ab_b, ac_a, bc_b, ac_g, bc_g;
    if (F.neg_ab) {  // I*wabm - wabp ; -I*wabm - wabp
      ab_a = make_double2(-abm.y - abp.x, abm.x - abp.y);
      ab_b = make_double2(abm.y - abp.x, -abm.x - abp.y);
    } else {  // I*wabp - wabm ; I*wabp + wabm
      ab_a = make_double2(-abp.y - abm.x, abp.x - abm.y);
      ab_b = make_double2(-abp.y + abm.x, abp.x + abm.y);
    }
    if (F.neg_ac) {  // I*wacm - wacp ; -I*wacm - wacp
      ac_a = make_double2(-acm.y - acp.x, acm.x - acp.y);
      ac_g = make_double2(acm.y - acp.x, -acm.x - acp.y);
    } else {  // I*wacp - wacm ; I*wacp + wacm
      ac_a = make_double2(-acp.y - acm.x, acp.x - acm.y);
      ac_g = make_double2(-acp.y + acm.x, acp.x + acm.y);
    }
    if (F.neg_bc) {  // I*wbcm - wbcp ; -I*wbcm - wbcp
      bc_b = make_double2(-bcm.y - bcp.x, bcm.x - bcp.y);
      bc_g = make_double2(bcm.y - bcp.x, -bcm.x - bcp.y);
    } else {  // I*wbcp - wbcm ; I*wbcp + wbcm
      bc_b = make_double2(-bcp.y - bcm.x, bcp.x - bcm.y);
      bc_g = make_double2(-bcp.y + bcm.x, bcp.x + bcm.y);
    }
    wa = cadd(cadd(Ipl, ab_a), ac_a);
    wb = cadd(cadd(Ipl, ab_b), bc_b);
    wg = cadd(cadd(Ipl, ac_g), bc_g);
  }
}

__global__ void k_assemble(const FieldInst *__restrict__ fi) {
  FOR_POINTS(F) {
    double2 w[7];
    for (int f = 0; f < 7; f++) w[f] = F.w[f][i];
    double2 wa, wb, wg;
    assemble_point(F, w, wa, wb, wg);
    F.sm[0][i] = wa;
    F.sm[1][i] = wb;
    if (F.graft) F.sm[2][i] = wg;
  }
}

// e^{-smw} for the propagators (code/diblock_discrete.cpp:21-28,54,79).
__global__ void k_boltzmann(const FieldInst *__restrict__ fi) {
  FOR_POINTS(F) {
    const int nf = F.graft ? 3 : 2;
    for (int f = 0; f < nf; f++) {
      double2 s = F.sm[f][i];
      if (f == 0 && F.shellU) s.x += F.shellU[i];
      F.expw[f][i] = cexp_d(make_double2(-s.x, -s.y));
    }
  }
}

// Q = integ_trapPBC(q[N-1]) / V and factor = nD / Q / V, one thread per instance.
__global__ void k_q_finalize(const FieldInst *__restrict__ fi, int ninst) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ninst) return;
  const FieldInst &F = fi[t];
  double2 s = make_double2(0.0, 0.0);
  for (int z = 0; z < F.nz; z++) s = cadd(s, F.qpart[z]);
  for (int d = 0; d < 3; d++) s = make_double2(s.x * F.dx[d], s.y * F.dx[d]);
  const double2 Q = make_double2(s.x / F.V, s.y / F.V);
  double2 f = cdiv_d(make_double2(F.nD, 0.0), Q);
  f = make_double2(f.x / F.V, f.y / F.V);
  F.scal[kQd] = Q;
  F.scal[kFactor] = f;
}

// code/calc_poly_density.cpp:187-188: rho *= exp(w) * factor
__global__ void k_density(const FieldInst *__restrict__ fi) {
  FOR_POINTS(F) {
    const double2 fac = F.scal[kFactor];
    double2 a = F.acc[0][0][i], b = F.acc[0][1][i];
    if (!F.single) {
      a = cadd(a, F.acc[1][0][i]);
      b = cadd(b, F.acc[1][1][i]);
    }
    double2 sa = F.sm[0][i];
    if (F.shellU) sa.x += F.shellU[i];
    F.rho[0][i] = cmul(a, cmul(cexp_d(sa), fac));
    F.rho[1][i] = cmul(b, cmul(cexp_d(F.sm[1][i]), fac));
  }
}

__device__ __forceinline__ double2 clog_d(double2 z) {
  return make_double2(log(hypot(z.x, z.y)), atan2(z.y, z.x));
}

// Graft density and the Qga integrand (code/grafted_nanoparticle.cpp:100-117):
//   rhog = acc * (ng_per_np * n_exp * exp(+smwg)),
//   tmp  = Re(grafts) <= 0 ? 0 : grafts * log(q_g[Ng-1]).
// part[(inst*gridDim.x + blk)*2 + {0,1}] = (sum of tmp, (count of Re q <= 0, 0)).
__global__ void k_graft_finalize(const FieldInst *__restrict__ fi, double2 *__restrict__ part) {
  __shared__ double2 red[32];
  __shared__ double redc[32];
  const FieldInst &F = fi[blockIdx.y];
  if (!F.graft) return;
  const double s = F.ng_per_np * F.n_exp_nr;
  double2 acc = make_double2(0.0, 0.0);
  double cnt = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < F.M;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 e = cexp_d(F.sm[2][i]);
    F.rho[2][i] = cmul(F.gacc[i], make_double2(s * e.x, s * e.y));
    const double2 gr = F.grafts[i];
    const double2 ql = F.ghist_last[i];
    if (gr.x > 0.0) acc = cadd(acc, cmul(gr, clog_d(ql)));
    if (ql.x <= 0.0) cnt += 1.0;
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { red[w] = acc; redc[w] = cnt; }
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    acc = l < nw ? red[l] : make_double2(0.0, 0.0);
    cnt = l < nw ? redc[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
      cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if (l == 0) {
      const long long b = (long long)blockIdx.y * gridDim.x + blockIdx.x;
      part[2 * b] = acc;
      part[2 * b + 1] = make_double2(cnt, 0.0);
    }
  }
}

// Qga = integ_trapPBC(tmp) (code/grafted_nanoparticle.cpp:112), one thread per instance.
__global__ void k_qga_finalize(const FieldInst *__restrict__ fi, int ninst, int blocks,
                               const double2 *__restrict__ part) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ninst) return;
  const FieldInst &F = fi[t];
  if (!F.graft) return;
  double2 s = make_double2(0.0, 0.0);
  double cnt = 0.0;
  for (int b = 0; b < blocks; b++) {
    s = cadd(s, part[2 * ((long long)t * blocks + b)]);
    cnt += part[2 * ((long long)t * blocks + b) + 1].x;
  }
  for (int d = 0; d < 3; d++) s = make_double2(s.x * F.dx[d], s.y * F.dx[d]);
  F.scal[kQga] = s;
  F.scal[kQg] = make_double2(cnt, 0.0);
}

// Complex-Langevin noise of field f at k-space point i (zero without).
__device__ __forceinline__ double2 cl_noise(const FieldInst &F, int f, long long i) {
  return F.eta[f] ? F.eta[f][i] : make_double2(0.0, 0.0);
}

// code/1s_update.cpp:58-329 at one k-space point (mean-field: no noise, no
// film/channel, no field nanoparticles, no homopolymer).  ra, rb, rg are the
// forward transforms (1/M scaled) of rhoda, rhodb, rhog_exp at this point and
// w[0..6] the transformed fields (wpl, wabp, wabm, wbcp, wbcm, wacp, wacm),
// updated in place.
__device__ __forceinline__ void update_1s_point(const FieldInst &F, long long i, double2 ra, double2 rb,
                                                double2 rg, double2 *w) {
  const double rho0 = F.rho0, N = (double)F.N, Ng = (double)F.Ng;
  const double li = F.lam_pl, lr = F.lam_mi;
  const double hh = F.hhat[i];
  const double hh2 = hh * hh;
  const double gaa = F.gaa[i], gab = F.gab[i], gbb = F.gbb[i], gc = F.gc[i];
  const double2 enh = F.exp_nrH[i];
  // w+  (:58-84)
  {
    const double evar = (i == 0) ? 1.0 : 0.0;
    const double2 s = cadd(cadd(ra, rg), rb);  // rhoha + rhoda + rhog + rhog_exp + rhodb
    // I*rho0*(exp_nrH - evar) + I*hhat*s
    const double2 u = make_double2(enh.x - evar, enh.y);
    const double2 F1 = make_double2(-rho0 * u.y - hh * s.y, rho0 * u.x + hh * s.x);
    const double A = rho0 / F.kappa + F.phiD * rho0 * N * hh2 * (gaa + 2.0 * gab + gbb) +
                     (F.phiG * Ng * gc) * rho0 * hh2;
    const double B = A - rho0 / F.kappa;
    const double2 wv = w[0];
    const double2 e0 = cl_noise(F, 0, i);
    const double2 num = make_double2(wv.x - li * (F1.x - B * wv.x) + e0.x, wv.y - li * (F1.y - B * wv.y) + e0.y);
    const double den = 1.0 + li * A;
    w[0] = make_double2(num.x / den, num.y / den);
  }
  // AB (:87-166)
  if (F.cab != 0.0) {
    const double c = F.cab;
    double2 wp = w[1], wm = w[2];
    const double2 ep = cl_noise(F, 1, i), em = cl_noise(F, 2, i);
    if (!F.neg_ab) {
      double2 F1 = make_double2(-hh * (ra.y + rb.y), hh * (ra.x + rb.x));  // I*hhat*(ra+rb)
      if (F.np_chem == 1) F1 = make_double2(F1.x - rho0 * enh.x, F1.y - rho0 * enh.y);
      const double A = 2.0 * rho0 / c + F.phiD * rho0 * N * hh2 * (gaa + 2.0 * gab + gbb);
      const double B = A - 2.0 * rho0 / c;
      const double den = 1.0 + li * A;
      wp = make_double2((wp.x - li * (F1.x - B * wp.x) + ep.x) / den, (wp.y - li * (F1.y - B * wp.y) + ep.y) / den);
      double2 F2 = make_double2(hh * (rb.x - ra.x), hh * (rb.y - ra.y));
      if (F.np_chem == 1) F2 = make_double2(F2.x - rho0 * enh.y, F2.y + rho0 * enh.x);
      const double den2 = 1.0 + lr * 2.0 * rho0 / c;
      wm = make_double2((wm.x - lr * F2.x + em.x) / den2, (wm.y - lr * F2.y + em.y) / den2);
    } else {
      const double2 F1 = make_double2(-hh * (ra.x + rb.x), -hh * (ra.y + rb.y));
      const double den1 = 1.0 + lr * 2.0 * rho0 / c;
      wp = make_double2((wp.x - lr * F1.x + ep.x) / den1, (wp.y - lr * F1.y + ep.y) / den1);
      double2 F2 = make_double2(-hh * (ra.y - rb.y), hh * (ra.x - rb.x));  // I*hhat*(ra-rb)
      if (F.np_chem == 1) F2 = make_double2(F2.x - rho0 * enh.x, F2.y - rho0 * enh.y);
      const double A = 2.0 * rho0 / c + F.phiD * rho0 * N * hh2 * (gaa - gbb);
      const double B = A - 2.0 * rho0 / c;
      const double den = 1.0 + li * A;
      wm = make_double2((wm.x - li * (F2.x - B * wm.x) + em.x) / den, (wm.y - li * (F2.y - B * wm.y) + em.y) / den);
    }
    w[1] = wp;
    w[2] = wm;
  } else {
    w[1] = make_double2(0.0, 0.0);
    w[2] = make_double2(0.0, 0.0);
  }
  // BC (:168-247)
  if (F.cbc != 0.0) {
    const double c = F.cbc;
    double2 wp = w[3], wm = w[4];
    const double2 ep = cl_noise(F, 3, i), em = cl_noise(F, 4, i);
    if (!F.neg_bc) {
      const double2 F1 = make_double2(-hh * (rg.y + rb.y), hh * (rg.x + rb.x));
      const double A = 2.0 * rho0 / c + F.phiD * rho0 * N * hh2 * (+gbb) + F.phiG * rho0 * Ng * hh2 * gc;
      const double B = A - 2.0 * rho0 / c;
      const double den = 1.0 + li * A;
      wp = make_double2((wp.x - li * (F1.x - B * wp.x) + ep.x) / den, (wp.y - li * (F1.y - B * wp.y) + ep.y) / den);
      double2 F2 = make_double2(hh * (rg.x - rb.x), hh * (rg.y - rb.y));
      if (F.np_chem == 1) F2 = make_double2(F2.x - rho0 * enh.y, F2.y + rho0 * enh.x);
      const double den2 = 1.0 + lr * 2.0 * rho0 / c;
      wm = make_double2((wm.x - lr * F2.x + em.x) / den2, (wm.y - lr * F2.y + em.y) / den2);
    } else {
      const double2 F1 = make_double2(-hh * (rb.x + rg.x), -hh * (rb.y + rg.y));
      const double den1 = 1.0 + lr * 2.0 * rho0 / c;
      wp = make_double2((wp.x - lr * F1.x + ep.x) / den1, (wp.y - lr * F1.y + ep.y) / den1);
      // -I*hhat*(rg - rb) = (hh*(rg-rb).y, -hh*(rg-rb).x)
      double2 F2 = make_double2(hh * (rg.y - rb.y), -hh * (rg.x - rb.x));
      if (F.np_chem == 1) F2 = make_double2(F2.x - rho0 * enh.x, F2.y - rho0 * enh.y);
      const double A = 2.0 * rho0 / c + F.phiD * rho0 * N * hh2 * gbb - F.phiG * Ng * hh2 * rho0 * gc;
      const double B = A - 2.0 * rho0 / c;
      const double den = 1.0 + li * A;
      wm = make_double2((wm.x - li * (F2.x - B * wm.x) + em.x) / den, (wm.y - li * (F2.y - B * wm.y) + em.y) / den);
    }
    w[3] = wp;
    w[4] = wm;
  } else {
    w[3] = make_double2(0.0, 0.0);
    w[4] = make_double2(0.0, 0.0);
  }
  // AC (:250-329)
  if (F.cac != 0.0) {
    const double c = F.cac;
    double2 wp = w[5], wm = w[6];
    const double2 ep = cl_noise(F, 5, i), em = cl_noise(F, 6, i);
    if (!F.neg_ac) {
      const double2 F1 = make_double2(-hh * (rg.y + ra.y), hh * (rg.x + ra.x));
      const double A = 2.0 * rho0 / c + F.phiD * rho0 * N * hh2 * gaa + F.phiG * Ng * hh2 * rho0 * gc;
      const double B = A - 2.0 * rho0 / c;
      const double den = 1.0 + li * A;
      wp = make_double2((wp.x - li * (F1.x - B * wp.x) + ep.x) / den, (wp.y - li * (F1.y - B * wp.y) + ep.y) / den);
      double2 F2 = make_double2(hh * (rg.x - ra.x), hh * (rg.y - ra.y));
      if (F.np_chem == 1) F2 = make_double2(F2.x - rho0 * enh.y, F2.y + rho0 * enh.x);
      const double den2 = 1.0 + lr * 2.0 * rho0 / c;
      wm = make_double2((wm.x - lr * F2.x + em.x) / den2, (wm.y - lr * F2.y + em.y) / den2);
    } else {
      const double2 F1 = make_double2(-hh * (ra.x + rg.x), -hh * (ra.y + rg.y));
      const double den1 = 1.0 + lr * 2.0 * rho0 / c;
      wp = make_double2((wp.x - lr * F1.x + ep.x) / den1, (wp.y - lr * F1.y + ep.y) / den1);
      double2 F2 = make_double2(hh * (rg.y - ra.y), -hh * (rg.x - ra.x));
      if (F.np_chem == 1) F2 = make_double2(F2.x - rho0 * enh.x, F2.y - rho0 * enh.y);
      const double A = 2.0 * rho0 / c + F.phiD * rho0 * N * hh2 * gaa - F.phiG * Ng * hh2 * rho0 * gc;
      const double B = A - 2.0 * rho0 / c;
      const double den = 1.0 + li * A;
      wm = make_double2((wm.x - li * (F2.x - B * wm.x) + em.x) / den, (wm.y - li * (F2.y - B * wm.y) + em.y) / den);
    }
    w[5] = wp;
    w[6] = wm;
  } else {
    w[5] = make_double2(0.0, 0.0);
    w[6] = make_double2(0.0, 0.0);
  }
}

// Explicit Euler step of the fields at one k point (code/Euler_update.cpp:54-179,
// mean field): w <- w - lam dH/dw with lam_pl for w+ and the + fields, lam_mi
// for the - fields, no Debye terms and no np_chem terms.  Arguments as
// update_1s_point.
__device__ __forceinline__ void euler_pair(const FieldInst &F, double c, int neg, double2 X, double2 Y, double hh,
                                           double2 ep, double2 em, double2 &wp, double2 &wm) {
  const double rho0 = F.rho0, li = F.lam_pl, lr = F.lam_mi;
  const double2 s = cadd(X, Y), d = csub(X, Y);
  // + : 2 rho0 wp / c + hhat (X + Y) (neg ? -1 : I)
  const double2 Fp = neg ? make_double2(2.0 * rho0 * wp.x / c - hh * s.x, 2.0 * rho0 * wp.y / c - hh * s.y)
                         : make_double2(2.0 * rho0 * wp.x / c - hh * s.y, 2.0 * rho0 * wp.y / c + hh * s.x);
  // - : 2 rho0 wm / c + (neg ? I hhat (X - Y) : hhat (Y - X))
  const double2 Fm = neg ? make_double2(2.0 * rho0 * wm.x / c - hh * d.y, 2.0 * rho0 * wm.y / c + hh * d.x)
                         : make_double2(2.0 * rho0 * wm.x / c - hh * d.x, 2.0 * rho0 * wm.y / c - hh * d.y);
  wp = make_double2(wp.x - li * Fp.x + ep.x, wp.y - li * Fp.y + ep.y);
  wm = make_double2(wm.x - lr * Fm.x + em.x, wm.y - lr * Fm.y + em.y);
}

__device__ __forceinline__ void euler_point(const FieldInst &F, long long i, double2 ra, double2 rb, double2 rg,
                                            double2 *w) {
  const double rho0 = F.rho0;
  const double hh = F.hhat[i];
  const double2 enh = F.exp_nrH[i];
  {
    const double evar = (i == 0) ? 1.0 : 0.0;
    const double2 s = cadd(cadd(ra, rg), rb);
    const double2 wv = w[0];
    // rho0 w+ / kappa + I rho0 (exp_nrH - evar) + I hhat s
    const double2 Fv = make_double2(rho0 * F.ikappa * wv.x - rho0 * enh.y - hh * s.y,
                                    rho0 * F.ikappa * wv.y + rho0 * (enh.x - evar) + hh * s.x);
    const double2 e0 = cl_noise(F, 0, i);
    w[0] = make_double2(wv.x - F.lam_pl * Fv.x + e0.x, wv.y - F.lam_pl * Fv.y + e0.y);
  }
  const double2 z = make_double2(0.0, 0.0);
  if (F.cab != 0.0) euler_pair(F, F.cab, F.neg_ab, ra, rb, hh, cl_noise(F, 1, i), cl_noise(F, 2, i), w[1], w[2]);
  else w[1] = w[2] = z;
  if (F.cbc != 0.0) euler_pair(F, F.cbc, F.neg_bc, rb, rg, hh, cl_noise(F, 3, i), cl_noise(F, 4, i), w[3], w[4]);
  else w[3] = w[4] = z;
  if (F.cac != 0.0) euler_pair(F, F.cac, F.neg_ac, ra, rg, hh, cl_noise(F, 5, i), cl_noise(F, 6, i), w[5], w[6]);
  else w[5] = w[6] = z;
}

__global__ void k_update_1s(const FieldInst *__restrict__ fi) {
  FOR_POINTS(F) {
    double2 w[7];
    for (int f = 0; f < 7; f++) w[f] = F.w[f][i];
    const double2 rg = F.graft ? F.rho[2][i] : make_double2(0.0, 0.0);
    if (F.euler)
      euler_point(F, i, F.rho[0][i], F.rho[1][i], rg, w);
    else
      update_1s_point(F, i, F.rho[0][i], F.rho[1][i], rg, w);
    for (int f = 0; f < 7; f++) F.w[f][i] = w[f];
  }
}

// Partial sums for calc_H (code/calc_h.cpp:66-132).  out[(inst*4 + part)*nblk + blk],
// part 0: wpl^2 rho0/kappa/2 - I rho0 (1 - rho_exp_nr) wpl; parts 1-3: (w+^2 + w-^2)
// rho0/chi (+-1) for the BC, AC and AB pairs.
__global__ void k_h_partials(const FieldInst *__restrict__ fi, double2 *__restrict__ out) {
  __shared__ double2 red[32];
  const FieldInst &F = fi[blockIdx.y];
  double2 s[4];
  for (int k = 0; k < 4; k++) s[k] = make_double2(0.0, 0.0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < F.M;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 w = F.w[0][i];
    const double2 w2 = cmul(w, w);
    const double2 t1 = make_double2(w2.x * F.rho0 * F.ikappa / 2.0, w2.y * F.rho0 * F.ikappa / 2.0);
    const double c = F.rho0 * (1.0 - 0.0 - F.rho_exp_nr[i]);
    // I*c*w = (-c*w.y, c*w.x)
    s[0] = cadd(s[0], make_double2(t1.x + c * w.y, t1.y - c * w.x));
    const double chis[3] = {F.cbc, F.cac, F.cab};
    const int negs[3] = {F.neg_bc, F.neg_ac, F.neg_ab};
    const int idx[3] = {3, 5, 1};
    for (int k = 0; k < 3; k++) {
      if (chis[k] == 0.0) continue;
      const double2 p = F.w[idx[k]][i], m = F.w[idx[k] + 1][i];
      const double2 q = cadd(cmul(p, p), cmul(m, m));
      const double f = F.rho0 / chis[k] * (negs[k] ? -1.0 : 1.0);
      s[k + 1] = cadd(s[k + 1], make_double2(q.x * f, q.y * f));
    }
  }
  for (int k = 0; k < 4; k++) {
    double2 v = s[k];
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, o);
      v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
      const int nw = (blockDim.x + 31) >> 5;
      v = l < nw ? red[l] : make_double2(0.0, 0.0);
      for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
      }
      if (l == 0) out[((long long)blockIdx.y * 4 + k) * gridDim.x + blockIdx.x] = v;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// mixed precision: fields in k-space, packed transforms of real pairs
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long neg_k(const FieldInst &F, long long i) {
  const int nx = F.nx, ny = F.ny;
  const long long ix = i % nx, iy = (i / nx) % ny, iz = i / ((long long)nx * ny);
  const long long jx = ix ? nx - ix : 0, jy = iy ? ny - iy : 0, jz = iz ? F.nz - iz : 0;
  return jx + (long long)nx * (jy + (long long)ny * jz);
}

// zg = hhat * w_G, the transform of the smeared graft field.
__device__ __forceinline__ double2 smear_graft(const FieldInst &F, long long i, const double2 *w) {
  double2 wa, wb, wg;
  assemble_point(F, w, wa, wb, wg);
  const double hh = F.hhat[i];
  return make_double2(hh * wg.x, hh * wg.y);
}

// zs = hhat * (w_A + i w_B), the packed transform of the two smeared fields.
__device__ __forceinline__ double2 smear_pack(const FieldInst &F, long long i, const double2 *w) {
  double2 wa, wb, wg;
  assemble_point(F, w, wa, wb, wg);
  const double hh = F.hhat[i];
  return make_double2(hh * (wa.x - wb.y), hh * (wa.y + wb.x));
}

// Stores zs(k) = hhat (w_A + i w_B) for the FP32 inverse transform: the
// k = 0 term (the means of smwa and smwb, which can be large) goes to
// scal[kSmean] in FP64 and is added back by the Boltzmann kernel, so the
// FP32 transform carries only the fluctuating part.
__device__ __forceinline__ void store_zs(const FieldInst &F, long long i, double2 zs) {
  if (i == 0) {
    F.scal[kSmean] = zs;
    // the two-float pairs the Boltzmann kernel needs, formed once here
    const float ah = (float)zs.x, bh = (float)zs.y;
    *reinterpret_cast<float4 *>(&F.scal[kSmean32]) =
        make_float4(ah, (float)(zs.x - (double)ah), bh, (float)(zs.y - (double)bh));
    F.z32[0] = make_float2(0.0f, 0.0f);
  } else {
    F.z32[i] = make_float2((float)zs.x, (float)zs.y);
  }
}

__global__ void k_mix_smear(const FieldInst *__restrict__ fi) {
  FOR_POINTS(F) {
    double2 w[7];
    for (int f = 0; f < 7; f++) w[f] = F.w[f][i];
    store_zs(F, i, smear_pack(F, i, w));
    if (F.graft) F.zg[i] = smear_graft(F, i, w);
  }
}

// 1S update on the k-space fields, with the k-only coefficients tabulated at
// set-up: for every field and sign branch of code/1s_update.cpp:58-329 the step is
// w <- (w - lam (F - B w)) / (1 + lam A) = alpha w - beta F, alpha, beta
// functions of k alone.  No division per iteration; only fields with
// nonzero chi are read and written.
// Sign s_f with w_f(-k) = s_f conj(w_f(k)) under the mean-field phase
// convention (the one scft_set_fields checks): -1 for the fields that are
// imaginary in real space (w+, and the + field of a pair with positive chi or
// the - field of a pair with negative chi), +1 for the real ones.
__device__ __forceinline__ double field_parity(const FieldInst &F, int f) {
  if (f == 0) return -1.0;
  const int neg = (f <= 2) ? F.neg_ab : (f <= 4 ? F.neg_bc : F.neg_ac);
  return (f & 1) ? (neg ? 1.0 : -1.0) : (neg ? -1.0 : 1.0);
}

// The two density transforms come from one packed FP32 transform Z of
// rho_A + i rho_B:
//   rho_A(k) = (Z(k) + conj Z(-k)) / 2,  rho_B(k) = (Z(k) - conj Z(-k)) / (2i),
// and zs(k) is written back into the same array (each thread reads and writes
// only its own pair).
// One thread per pair (k, -k): every field and density is Hermitian or
// anti-Hermitian in k-space, so the update at -k follows from the one at k by
// conjugation; this halves the FP64 work, which bounds this kernel on GB300.
// Threads run over the planes z = 0..nz/2; within the self-conjugate planes
// (z = 0 and, for even nz, nz/2) only the member with the smaller index of
// each pair works.
__global__ void k_mix_update_tab(const FieldInst *__restrict__ fi) {
  const FieldInst &F = fi[blockIdx.y];
  const long long plane = (long long)F.nx * F.ny;
  const long long Mh = plane * (F.nz / 2 + 1);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < Mh;
       i += (long long)gridDim.x * blockDim.x) {
    const long long j = neg_k(F, i);
    if (j < i) continue;
    const float2 Zf = F.z32[i], Zmf = F.z32[j];
    const double2 Z = make_double2(Zf.x, Zf.y), Zm = make_double2(Zmf.x, Zmf.y);
    const double2 ra = make_double2(0.5 * (Z.x + Zm.x), 0.5 * (Z.y - Zm.y));
    const double2 rb = make_double2(0.5 * (Z.y + Zm.y), 0.5 * (Zm.x - Z.x));
    const double rho0 = F.rho0, hh = F.hhat[i];
    const double2 enh = F.exp_nrH[i];
    const double2 rg = F.graft ? F.zg[i] : make_double2(0.0, 0.0);
    double2 w[7];
    for (int f = 0; f < 7; f++) w[f] = F.alpha[f] ? F.w[f][i] : make_double2(0.0, 0.0);
    auto step = [&](int f, double2 Fv) {
      const double a = F.alpha[f][i], b = F.beta[f][i];
      w[f] = make_double2(a * w[f].x - b * Fv.x, a * w[f].y - b * Fv.y);
    };
    // w+ : I rho0 (exp_nrH - evar) + I hhat (rhoda + rhodb)
    {
      const double evar = (i == 0) ? 1.0 : 0.0;
      const double2 sr = cadd(cadd(ra, rb), rg);
      const double2 u = make_double2(enh.x - evar, enh.y);
      step(0, make_double2(-rho0 * u.y - hh * sr.y, rho0 * u.x + hh * sr.x));
    }
    if (F.alpha[1]) {  // AB pair
      if (!F.neg_ab) {
        double2 F1 = make_double2(-hh * (ra.y + rb.y), hh * (ra.x + rb.x));
        if (F.np_chem == 1 && !F.euler) F1 = make_double2(F1.x - rho0 * enh.x, F1.y - rho0 * enh.y);
        double2 F2 = make_double2(hh * (rb.x - ra.x), hh * (rb.y - ra.y));
        if (F.np_chem == 1 && !F.euler) F2 = make_double2(F2.x - rho0 * enh.y, F2.y + rho0 * enh.x);
        step(1, F1);
        step(2, F2);
      } else {
        const double2 F1 = make_double2(-hh * (ra.x + rb.x), -hh * (ra.y + rb.y));
        double2 F2 = make_double2(-hh * (ra.y - rb.y), hh * (ra.x - rb.x));
        if (F.np_chem == 1 && !F.euler) F2 = make_double2(F2.x - rho0 * enh.x, F2.y - rho0 * enh.y);
        step(1, F1);
        step(2, F2);
      }
    }
    // BC and AC pairs: graft density transform rg
    if (F.alpha[3]) {
      if (!F.neg_bc) {
        const double2 F1 = make_double2(-hh * (rg.y + rb.y), hh * (rg.x + rb.x));
        double2 F2 = make_double2(hh * (rg.x - rb.x), hh * (rg.y - rb.y));
        if (F.np_chem == 1 && !F.euler) F2 = make_double2(F2.x - rho0 * enh.y, F2.y + rho0 * enh.x);
        step(3, F1);
        step(4, F2);
      } else {
        const double2 F1 = make_double2(-hh * (rb.x + rg.x), -hh * (rb.y + rg.y));
        double2 F2 = make_double2(hh * (rg.y - rb.y), -hh * (rg.x - rb.x));
        if (F.np_chem == 1 && !F.euler) F2 = make_double2(F2.x - rho0 * enh.x, F2.y - rho0 * enh.y);
        step(3, F1);
        step(4, F2);
      }
    }
    if (F.alpha[5]) {
      if (!F.neg_ac) {
        const double2 F1 = make_double2(-hh * (rg.y + ra.y), hh * (rg.x + ra.x));
        double2 F2 = make_double2(hh * (rg.x - ra.x), hh * (rg.y - ra.y));
        if (F.np_chem == 1 && !F.euler) F2 = make_double2(F2.x - rho0 * enh.y, F2.y + rho0 * enh.x);
        step(5, F1);
        step(6, F2);
      } else {
        const double2 F1 = make_double2(-hh * (ra.x + rg.x), -hh * (ra.y + rg.y));
        double2 F2 = make_double2(hh * (rg.y - ra.y), -hh * (rg.x - ra.x));
        if (F.np_chem == 1 && !F.euler) F2 = make_double2(F2.x - rho0 * enh.x, F2.y - rho0 * enh.y);
        step(5, F1);
        step(6, F2);
      }
    }
    const bool pair = (j != i);
    for (int f = 0; f < 7; f++)
      if (F.alpha[f]) {
        F.w[f][i] = w[f];
        if (pair) {
          const double sf = field_parity(F, f);
          F.w[f][j] = make_double2(sf * w[f].x, -sf * w[f].y);
        }
      }
    double2 wa, wb, wg;
    assemble_point(F, w, wa, wb, wg);
    // zs = hhat (w_A + i w_B) at k and, with w_A(-k) = conj w_A(k), at -k
    store_zs(F, i, make_double2(hh * (wa.x - wb.y), hh * (wa.y + wb.x)));
    if (pair) F.z32[j] = make_float2((float)(hh * (wa.x + wb.y)), (float)(hh * (wb.x - wa.y)));
    if (F.graft) {
      F.zg[i] = make_double2(hh * wg.x, hh * wg.y);
      if (pair) F.zg[j] = make_double2(hh * wg.x, -hh * wg.y);
    }
  }
}

// After the inverse transform z32 = smwa + i smwb minus their means (real
// space): Boltzmann factors for the FP32 sweep.  s = mean + d with the mean
// as a two-float (m_hi, m_lo) and d the FP32 transform value:
// t = fl(m_hi + d) with its rounding error e (two-sum), and
// exp(-s) = expf(-t) (1 - (m_lo + e)), the neglected term being
// O((m_lo + e)^2) ~ 1e-14 relative, so the result carries expf's accuracy
// without an FP64 exponential however large the mean is.
__device__ __forceinline__ float boltz_two_float(float mh, float ml, float d) {
  const float t = mh + d, v = t - mh;
  const float e = (mh - (t - v)) + (d - v);
  return expf(-t) * (1.0f - (ml + e));
}

__global__ void k_mix_boltzmann(const FieldInst *__restrict__ fi) {
  // the means as two-float pairs, split once by the kernel that formed them:
  // GB300 runs FP64 (conversions included) at a small fraction of the FP32
  // rate, so no per-point or per-block FP64 work here
  const float4 m = *reinterpret_cast<const float4 *>(&fi[blockIdx.y].scal[kSmean32]);
  const float ah = m.x, al = m.y, bh = m.z, bl = m.w;
  FOR_POINTS(F) {
    if (F.graft) {
      const double sg = F.zg[i].x;
      const float gh = (float)sg, gl = (float)(sg - (double)gh);
      F.Eg32[i] = expf(-gh) * (1.0f - gl);
      F.sm[2][i] = make_double2(sg, F.zg[i].y);
    }
    const float2 d = F.z32[i];
    const float da = F.shellU ? d.x + (float)F.shellU[i] : d.x;
    F.E32[i] = make_float2(boltz_two_float(ah, al, da), boltz_two_float(bh, bl, d.y));
  }
}

// Q from the plane sums of q_{N-1} and its exponent; factor = nD / Q / V.
__global__ void k_mix_q_finalize(const FieldInst *__restrict__ fi, int ninst) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ninst) return;
  const FieldInst &F = fi[t];
  double s = 0.0;
  const double *pq = F.part64 + (long long)(F.N - 1) * F.nz;  // plane sums of q_{N-1}
  for (int z = 0; z < F.nz; z++) s += pq[z];
  s = ldexp(s, F.K[F.N - 1]);
  for (int d = 0; d < 3; d++) s *= F.dx[d];
  const double Q = s / F.V;
  F.scal[kQd] = make_double2(Q, 0.0);
  F.scal[kFactor] = make_double2(F.nD / Q / F.V, 0.0);
  int fe;
  const float fm = (float)frexp(ldexp(F.nD / Q / F.V, F.K[2 * F.N]), &fe);
  *reinterpret_cast<float2 *>(&F.scal[kFactor32]) = make_float2(fm, __int_as_float(fe));
}

// rho_A, rho_B = acc * e^{+smw} * factor, packed into z32 for the FP32
// forward transform (keep = 0) or stored as FP64 complex arrays for
// scft_get_density and the gradient (keep = 1).  The factor carries the
// accumulators' exponent and can lie outside the FP32 range: it is applied as
// an FP32 mantissa and an ldexpf.
__global__ void k_mix_rho_pack(const FieldInst *__restrict__ fi, int keep) {
  // the factor (accumulators are scaled by 2^-Kref): FP32 mantissa and
  // exponent from k_mix_q_finalize; FP64 (formed here) only for keep
  const float2 fx = *reinterpret_cast<const float2 *>(&fi[blockIdx.y].scal[kFactor32]);
  const float fm = fx.x;
  const int fe = __float_as_int(fx.y);
  double f = 0.0;
  if (keep) {
    const FieldInst &F0 = fi[blockIdx.y];
    f = ldexp(F0.scal[kFactor].x, F0.K[2 * F0.N]);
  }
  FOR_POINTS(F) {
    // e^{+smw} = 1 / e^{-smw}: the FP32 reciprocal of the Boltzmann factor
    const float2 E = F.E32[i];
    const float xa = F.acc32[0][i] * __frcp_rn(E.x), xb = F.acc32[1][i] * __frcp_rn(E.y);
    if (keep) {
      F.rho[0][i] = make_double2((double)xa * f, 0.0);
      F.rho[1][i] = make_double2((double)xb * f, 0.0);
    } else {
      F.z32[i] = make_float2(ldexpf(xa * fm, fe), ldexpf(xb * fm, fe));
    }
  }
}

// Mixed form, grafted instances (code/grafted_nanoparticle.cpp:100-117):
//   rhog = ng_per_np n_exp e^{+smwg} sum_j q_g qdag_g   (FP64, into zg and rho[2])
//   Qga integrand: Re(grafts) <= 0 ? 0 : grafts log(q_g[Ng-1]) with the stored
//   q_g[Ng-1] times 2^K.  part as k_graft_finalize.
__global__ void k_mix_graft_finalize(const FieldInst *__restrict__ fi, double2 *__restrict__ part) {
  __shared__ double2 red[32];
  __shared__ double redc[32];
  const FieldInst &F = fi[blockIdx.y];
  if (!F.graft) return;
  const double s = F.ng_per_np * F.n_exp_nr;
  const double lk = (double)F.gK[F.Ng - 1] * 0.693147180559945309417232121458176568;
  double2 acc = make_double2(0.0, 0.0);
  double cnt = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < F.M;
       i += (long long)gridDim.x * blockDim.x) {
    const double rg = (double)F.gacc32[i] * (s * exp(F.zg[i].x));
    F.zg[i] = make_double2(rg, 0.0);
    F.rho[2][i] = make_double2(rg, 0.0);
    const double2 gr = F.grafts[i];
    const double ql = (double)F.ghist32_last[i];
    if (gr.x > 0.0) {
      const double2 lg = make_double2(log(fabs(ql)) + lk, ql < 0.0 ? 3.14159265358979323846 : 0.0);
      acc = cadd(acc, cmul(gr, lg));
    }
    if (ql <= 0.0) cnt += 1.0;
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { red[w] = acc; redc[w] = cnt; }
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    acc = l < nw ? red[l] : make_double2(0.0, 0.0);
    cnt = l < nw ? redc[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
      cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if (l == 0) {
      const long long b = (long long)blockIdx.y * gridDim.x + blockIdx.x;
      part[2 * b] = acc;
      part[2 * b + 1] = make_double2(cnt, 0.0);
    }
  }
}

// calc_H field terms by Parseval on the k-space fields:
//   int f g dr = V sum_k f(k) g(-k)  (transforms scaled by 1/M).
// out[(inst*4 + part)*gridDim.x + blk]; the host multiplies by V.
__global__ void k_mix_h_partials(const FieldInst *__restrict__ fi, double2 *__restrict__ out) {
  __shared__ double2 red[32];
  const FieldInst &F = fi[blockIdx.y];
  double2 s[4];
  for (int k = 0; k < 4; k++) s[k] = make_double2(0.0, 0.0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < F.M;
       i += (long long)gridDim.x * blockDim.x) {
    const long long mi = neg_k(F, i);
    const double2 w = F.w[0][i], wm = F.w[0][mi];
    const double2 ww = cmul(w, wm);
    // rho0/(2 kappa) w w  + I rho0 rho_exp(-k) w  (- I rho0 w(0) at k = 0)
    const double2 re = F.exp_nrH[mi];
    const double2 rw = cmul(re, w);
    double2 t = make_double2(ww.x * F.rho0 * F.ikappa / 2.0 - F.rho0 * rw.y,
                             ww.y * F.rho0 * F.ikappa / 2.0 + F.rho0 * rw.x);
    if (i == 0) t = make_double2(t.x + F.rho0 * w.y, t.y - F.rho0 * w.x);
    s[0] = cadd(s[0], t);
    const double chis[3] = {F.cbc, F.cac, F.cab};
    const int negs[3] = {F.neg_bc, F.neg_ac, F.neg_ab};
    const int idx[3] = {3, 5, 1};
    for (int k = 0; k < 3; k++) {
      if (chis[k] == 0.0) continue;
      const double2 q = cadd(cmul(F.w[idx[k]][i], F.w[idx[k]][mi]), cmul(F.w[idx[k] + 1][i], F.w[idx[k] + 1][mi]));
      const double f = F.rho0 / chis[k] * (negs[k] ? -1.0 : 1.0);
      s[k + 1] = cadd(s[k + 1], make_double2(q.x * f, q.y * f));
    }
  }
  for (int k = 0; k < 4; k++) {
    double2 v = s[k];
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, o);
      v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
      const int nw = (blockDim.x + 31) >> 5;
      v = l < nw ? red[l] : make_double2(0.0, 0.0);
      for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
      }
      if (l == 0) out[((long long)blockIdx.y * 4 + k) * gridDim.x + blockIdx.x] = v;
    }
    __syncthreads();
  }
}

cudaError_t launch_mix_smear(const FieldInst *fi, int ninst, int blocks, cudaStream_t st) {
  k_mix_smear<<<dim3(blocks, ninst), 256, 0, st>>>(fi);
  return cudaGetLastError();
}
cudaError_t launch_mix_graft_finalize(const FieldInst *fi, int ninst, int blocks, double2 *part, cudaStream_t st) {
  k_mix_graft_finalize<<<dim3(blocks, ninst), 256, 0, st>>>(fi, part);
  return cudaGetLastError();
}
cudaError_t launch_mix_update(const FieldInst *fi, int ninst, int blocks, cudaStream_t st) {
  k_mix_update_tab<<<dim3(blocks, ninst), 256, 0, st>>>(fi);
  return cudaGetLastError();
}
cudaError_t launch_mix_boltzmann(const FieldInst *fi, int ninst, int blocks, cudaStream_t st) {
  k_mix_boltzmann<<<dim3(blocks, ninst), 256, 0, st>>>(fi);
  return cudaGetLastError();
}
cudaError_t launch_mix_q_finalize(const FieldInst *fi, int ninst, cudaStream_t st) {
  k_mix_q_finalize<<<(ninst + 63) / 64, 64, 0, st>>>(fi, ninst);
  return cudaGetLastError();
}
cudaError_t launch_mix_rho_pack(const FieldInst *fi, int ninst, int blocks, int keep, cudaStream_t st) {
  k_mix_rho_pack<<<dim3(blocks, ninst), 256, 0, st>>>(fi, keep);
  return cudaGetLastError();
}
cudaError_t launch_mix_h_partials(const FieldInst *fi, int ninst, int blocks, double2 *out, cudaStream_t st) {
  k_mix_h_partials<<<dim3(blocks, ninst), 256, 0, st>>>(fi, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
cudaError_t launch_assemble(const FieldInst *fi, int ninst, int blocks, cudaStream_t st) {
  k_assemble<<<dim3(blocks, ninst), 256, 0, st>>>(fi);
  return cudaGetLastError();
}
cudaError_t launch_boltzmann(const FieldInst *fi, int ninst, int blocks, cudaStream_t st) {
  k_boltzmann<<<dim3(blocks, ninst), 256, 0, st>>>(fi);
  return cudaGetLastError();
}
cudaError_t launch_q_finalize(const FieldInst *fi, int ninst, cudaStream_t st) {
  k_q_finalize<<<(ninst + 63) / 64, 64, 0, st>>>(fi, ninst);
  return cudaGetLastError();
}
cudaError_t launch_density(const FieldInst *fi, int ninst, int blocks, cudaStream_t st) {
  k_density<<<dim3(blocks, ninst), 256, 0, st>>>(fi);
  return cudaGetLastError();
}
cudaError_t launch_update_1s(const FieldInst *fi, int ninst, int blocks, cudaStream_t st) {
  k_update_1s<<<dim3(blocks, ninst), 256, 0, st>>>(fi);
  return cudaGetLastError();
}
cudaError_t launch_graft_finalize(const FieldInst *fi, int ninst, int blocks, double2 *part, cudaStream_t st) {
  k_graft_finalize<<<dim3(blocks, ninst), 256, 0, st>>>(fi, part);
  return cudaGetLastError();
}
cudaError_t launch_qga_finalize(const FieldInst *fi, int ninst, int blocks, const double2 *part, cudaStream_t st) {
  k_qga_finalize<<<(ninst + 63) / 64, 64, 0, st>>>(fi, ninst, blocks, part);
  return cudaGetLastError();
}
cudaError_t launch_h_partials(const FieldInst *fi, int ninst, int blocks, double2 *out, cudaStream_t st) {
  k_h_partials<<<dim3(blocks, ninst), 256, 0, st>>>(fi, out);
  return cudaGetLastError();
}

}  // namespace scft
