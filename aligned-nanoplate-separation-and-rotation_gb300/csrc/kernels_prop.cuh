// kernels_prop.cuh -- the chain-propagator sweep of the plain FP64 method.
//
// Kernels only: the diblock and graft plane passes are launched from their
// own translation units (kernels_prop_f64.cu, kernels_graft_f64.cu) so that
// the library's units compile in parallel.
//
// Reference: diblock_discrete (code/diblock_discrete.cpp:4-95) computes
//   q_0 = e^{-W},  q_n = e^{-w(n)} * IFFT[ g(k) * FFT[q_{n-1}] ] / M,
// for q (A end first) and q-dagger (B end first), stores all 2N propagators,
// and integrate_diblock_discrete (code/calc_poly_density.cpp:167-191) then
// forms rho_A, rho_B = e^{+W} nD/(Q V) sum_j q_j qdag_{N-1-j}.
//
// Here one step n is two launches over all instances and both propagators:
//   z-column pass (kernels_fft.cuh, mode 2): forward-z, * g(k)/M, inverse-z;
//   xy-plane pass (k_prop_plane below): inverse-xy, * e^{-w(n)} -> q_n, then
//     - q_n kept only for n <= (N-1)/2 (half history);
//     - for n > (N-1)/2 the density terms j = n and j = N-1-n are added
//       from the current propagator and the stored half of the other one
//       (each propagator has its own accumulators, so the two CTAs of a plane
//       never write the same array); for odd N the middle term j = (N-1)/2 is
//       added at step (N-1)/2 + 1 from the two stored copies;
//     - at n = N-1 the plane sums of q_{N-1} (for Q) are written;
//     - forward-xy for the next step.
// Step 0 starts from e^{-W}.
#pragma once
#include "fft_core.cuh"
#include "inst.h"
#include "launch.h"
#include "prop_launch.h"

namespace scft {

__device__ __forceinline__ double2 block_sum_d2(double2 v, double2 *red) {
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
  }
  return v;
}

// GM: the plane is worked on in place in the working array in global memory
// (planes too large for shared memory, see LaunchShape).
template <int MAXV, bool GM>
__global__ void __launch_bounds__(512) k_prop_plane_f64(const PropJob *__restrict__ jobs, const PropInst *__restrict__ insts,
                                 const DevGeom *__restrict__ geoms, const double2 *__restrict__ twbuf, int n) {
  typedef double2 C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PropJob jb = jobs[blockIdx.x];
  const PropInst &P = insts[jb.inst];
  const DevGeom g = geoms[P.geom];
  const int E = g.nx * g.ny;
  const int N = P.N, Na = P.Na, p = jb.p;
  if (n >= N) return;
  const long long zoff = (long long)jb.z * E;
  const long long M = g.M;
  C *work = reinterpret_cast<C *>(P.work[p]) + zoff;
  C *plane = GM ? work : reinterpret_cast<C *>(smem_raw);
  C *twx = GM ? reinterpret_cast<C *>(smem_raw) : plane + E;
  C *twy = twx + g.nx;
  C *red = twy + g.ny;
  // field switch: code/diblock_discrete.cpp:20-28,38-41,62-65
  const bool useA = (p == 0) ? (Na > 0 && n < Na) : !(n <= N - Na - 1);
  const C *Ew = P.expw[useA ? 0 : 1] + zoff;
  load_tw<double>(twx, twbuf, g.ax[0]);
  load_tw<double>(twy, twbuf, g.ax[1]);
  if (n == 0) {
    for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = Ew[e];
  } else {
    if (!GM)
      for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = work[e];
    __syncthreads();
    fft_plane<double, +1, MAXV>(plane, g, twx, twy);
    for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = cmul(plane[e], Ew[e]);
  }
  // plane now holds q_n (p = 0) or qdag_n (p = 1); each thread touches only
  // its own elements until the next transform.
  C *histp = reinterpret_cast<C *>(P.hist[p]);
  if (n <= P.hmax) {
    C *h = histp + (long long)n * M + zoff;
    for (int e = threadIdx.x; e < E; e += blockDim.x) h[e] = plane[e];
  }
  const int m2 = N - 1 - n;
  if (!P.single) {
    if (m2 < n) {
      if (p == 0) {  // term j = n: q_n * qdag_{N-1-n}
        const C *o = reinterpret_cast<const C *>(P.hist[1]) + (long long)m2 * M + zoff;
        C *acc = P.acc[0][n < Na ? 0 : 1] + zoff;
        for (int e = threadIdx.x; e < E; e += blockDim.x) acc[e] = cadd(acc[e], cmul(plane[e], o[e]));
      } else {  // term j = N-1-n: q_{N-1-n} * qdag_n
        const C *o = reinterpret_cast<const C *>(P.hist[0]) + (long long)m2 * M + zoff;
        C *acc = P.acc[1][m2 < Na ? 0 : 1] + zoff;
        for (int e = threadIdx.x; e < E; e += blockDim.x) acc[e] = cadd(acc[e], cmul(o[e], plane[e]));
      }
    }
    const int mid = (N - 1) / 2;
    if ((N & 1) && p == 0 && n == mid + 1) {
      const C *a = reinterpret_cast<const C *>(P.hist[0]) + (long long)mid * M + zoff;
      const C *b = reinterpret_cast<const C *>(P.hist[1]) + (long long)mid * M + zoff;
      C *acc = P.acc[0][mid < Na ? 0 : 1] + zoff;
      for (int e = threadIdx.x; e < E; e += blockDim.x) acc[e] = cadd(acc[e], cmul(a[e], b[e]));
    }
  } else if (p == 0) {
    if (m2 < n) {  // terms j = n and j = N-1-n are the same product
      const C *o = histp + (long long)m2 * M + zoff;
      C *acc = P.acc[0][n < Na ? 0 : 1] + zoff;
      for (int e = threadIdx.x; e < E; e += blockDim.x) {
        const C t = cmul(plane[e], o[e]);
        acc[e] = cadd(acc[e], cadd(t, t));
      }
    } else if (m2 == n) {
      C *acc = P.acc[0][n < Na ? 0 : 1] + zoff;
      for (int e = threadIdx.x; e < E; e += blockDim.x) acc[e] = cadd(acc[e], cmul(plane[e], plane[e]));
    }
  }
  if (n == N - 1) {
    if (p == 0) {
      C s = make_double2(0.0, 0.0);
      for (int e = threadIdx.x; e < E; e += blockDim.x) s = cadd(s, plane[e]);
      s = block_sum_d2(s, red);
      if (threadIdx.x == 0) P.qpart[jb.z] = s;
    }
    return;
  }
  __syncthreads();
  fft_plane<double, -1, MAXV>(plane, g, twx, twy);
  if (!GM)
    for (int e = threadIdx.x; e < E; e += blockDim.x) work[e] = plane[e];
}

// Graft sweeps (code/grafted_nanoparticle.cpp:15-42 and :44-100), one CTA per
// (instance, z) for instances with grafted plates.
//   sweep 0: q_g[0] = e^{-w_G}; q_g[n] = e^{-w_G} * IFFT[g(k) FFT[q_g[n-1]]]/M,
//            every step kept (the density needs all of them);
//   sweep 1: qdag_g[0] = grafts * e^{-w_G} / q_g[Ng-1]; same recurrence, and
//            the density term q_g[Ng-1-n] * qdag_g[n] is added at step n.
template <int MAXV, bool GM>
__global__ void __launch_bounds__(512) k_graft_plane_f64(const PropJob *__restrict__ jobs,
                                                        const PropInst *__restrict__ insts,
                                                        const DevGeom *__restrict__ geoms,
                                                        const double2 *__restrict__ twbuf, int sweep, int n) {
  typedef double2 C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PropJob jb = jobs[blockIdx.x];
  const PropInst &P = insts[jb.inst];
  const DevGeom g = geoms[P.geom];
  const int Ng = P.Ng;
  if (n >= Ng) return;
  const int E = g.nx * g.ny;
  const long long zoff = (long long)jb.z * E;
  const long long M = g.M;
  const C *Ew = P.gexpw + zoff;
  C *work = reinterpret_cast<C *>(P.gwork) + zoff;
  C *plane = GM ? work : reinterpret_cast<C *>(smem_raw);
  C *twx = GM ? reinterpret_cast<C *>(smem_raw) : plane + E;
  C *twy = twx + g.nx;
  const C *hist = reinterpret_cast<const C *>(P.ghist);
  load_tw<double>(twx, twbuf, g.ax[0]);
  load_tw<double>(twy, twbuf, g.ax[1]);
  if (n == 0) {
    if (sweep == 0) {
      for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = Ew[e];
    } else {
      const C *last = hist + (long long)(Ng - 1) * M + zoff;
      const C *gr = P.grafts + zoff;
      for (int e = threadIdx.x; e < E; e += blockDim.x) {
        // expl_grafts * exp(-smwg) / q[Ng-1]
        const C a = cmul(gr[e], Ew[e]);
        const C b = last[e];
        C r;
        if (fabs(b.x) < fabs(b.y)) {
          const double q = b.x / b.y, d = b.x * q + b.y;
          r = make_double2((a.x * q + a.y) / d, (a.y * q - a.x) / d);
        } else {
          const double q = b.y / b.x, d = b.y * q + b.x;
          r = make_double2((a.y * q + a.x) / d, (a.y - a.x * q) / d);
        }
        plane[e] = r;
      }
    }
  } else {
    if (!GM)
      for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = work[e];
    __syncthreads();
    fft_plane<double, +1, MAXV>(plane, g, twx, twy);
    for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = cmul(plane[e], Ew[e]);
  }
  if (sweep == 0) {
    C *h = reinterpret_cast<C *>(P.ghist) + (long long)n * M + zoff;
    for (int e = threadIdx.x; e < E; e += blockDim.x) h[e] = plane[e];
  } else {
    const C *o = hist + (long long)(Ng - 1 - n) * M + zoff;
    C *acc = P.gacc + zoff;
    for (int e = threadIdx.x; e < E; e += blockDim.x) acc[e] = cadd(acc[e], cmul(o[e], plane[e]));
  }
  if (n == Ng - 1) return;
  __syncthreads();
  fft_plane<double, -1, MAXV>(plane, g, twx, twy);
  if (!GM)
    for (int e = threadIdx.x; e < E; e += blockDim.x) work[e] = plane[e];
}

}  // namespace scft
