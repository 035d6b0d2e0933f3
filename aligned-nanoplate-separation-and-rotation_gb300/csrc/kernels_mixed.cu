// kernels_mixed.cu -- propagator sweep of the mixed-precision form.
//
// Mean-field fields are real, so q_n and qdag_n are real and the bond kernel
// g(k) = exp(-k^2/6) is real and even: the convolution maps real arrays to
// real arrays.  One FP32 complex array z = q + i*qdag therefore carries both
// propagators through a single transform per step (the recurrence of
// code/diblock_discrete.cpp:31-85, for q and qdag at once).  The xy-plane pass
// applies e^{-w} separately to the real part (q, field of step n for q) and
// the imaginary part (qdag), which is exact for real fields.
//
// Mean in FP64: the plane pass writes exact (FP64) plane sums of what it
// stores; the next step's column pass drops the FP32 k = 0 coefficient and the
// plane pass adds the FP64 mean back, as a two-float constant, before the
// Boltzmann factor.  Rounding of the mean mode would otherwise be one
// coherent error per step that does not average over the grid.
//
// Range: each step is rescaled by a power of two chosen from that mean (lag 1,
// so no extra synchronisation), which is exact in floating point.  Integer
// exponents K[p][n] (q_true = q_stored * 2^K) are kept per instance.  The
// density terms q_j qdag_{N-1-j} all have about the same magnitude, so they
// are accumulated in FP32 relative to one reference exponent K[2N] fixed at
// the first accumulating step; Q and the finalised densities are FP64.  No
// FP64 arithmetic runs per grid point here: GB300 issues FP64 at a small
// fraction of its FP32 rate.
//
// Density terms are accumulated as in the FP64 kernel: for n > (N-1)/2 the
// terms j = n and j = N-1-n pair the current step with the stored half of
// the history; the middle term of odd N is formed in place at n = (N-1)/2.
#include "async_copy.cuh"
#include "fft_core.cuh"
#include "inst.h"
#include "launch.h"
#include "prop_launch.h"

namespace scft {

// PP: the transforms run out of place between two plane buffers
// (fft_plane_pp), which needs E * 8 bytes more shared memory but keeps the
// registers free of the in-place form's per-thread value arrays.
// STAGE: the plane arrives by bulk copy (cp.async.bulk) into shared memory,
// and so do the Boltzmann plane (issued at kernel start, so that its latency
// overlaps the inverse transforms) and, on a paired step, the stored partner
// plane (issued into the Boltzmann buffer once that is consumed, overlapping
// the history store).  It needs E * 8 bytes more shared memory and 16-byte
// aligned planes (E even); the host picks it when every plane of the batch
// qualifies and the total fits.  Waits are bounded and set *err when they
// run out.
// Launch bounds: the out-of-place form runs up to 512 threads, two CTAs per
// SM (64 registers); the in-place form keeps a thread's MAXV values live
// across its barriers and runs one CTA per SM (its plane fills shared
// memory), with MAXV = 16 on up to 1024 threads for planes too large for a
// second buffer (128 x 128).
template <int MAXV, bool STAGE, bool PP>
__global__ void __launch_bounds__(PP ? 512 : (MAXV == 16 ? 1024 : 512), PP ? 2 : 1) k_mix_prop_plane(const PropJob *__restrict__ jobs,
                                                       const MixInst *__restrict__ insts,
                                                       const DevGeom *__restrict__ geoms,
                                                       const float2 *__restrict__ twbuf, int n, int *err) {
  typedef float2 C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_red[2][32];
  __shared__ int s_exp[2];
  __shared__ __align__(8) uint64_t s_bar[2];  // [0] working plane, [1] Boltzmann then partner plane
  const PropJob jb = jobs[blockIdx.x];
  const MixInst &P = insts[jb.inst];
  const int N = P.N, Na = P.Na;
  if (n >= N) return;
  const DevGeom g = geoms[P.geom];
  const int E = g.nx * g.ny;
  const int nz = g.nz;
  const int nbuf = PP ? 2 : 1;
  C *plane = reinterpret_cast<C *>(smem_raw);
  C *plane2 = plane + E;  // second buffer (PP)
  C *twx = plane + nbuf * E;
  C *twy = twx + g.nx;
  C *Es = reinterpret_cast<C *>(smem_raw + (((size_t)(nbuf * E + g.nx + g.ny) * sizeof(C) + 15) & ~(size_t)15));
  const long long zoff = (long long)jb.z * E;
  const long long M = g.M;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m2 = N - 1 - n;
  C *cur = plane;  // buffer holding the plane
  const uint32_t pbytes = (uint32_t)E * (uint32_t)sizeof(C);
  if (STAGE && threadIdx.x == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    const uint64_t pol = l2_policy_last();
    if (n > 0) {
      mbar_expect_tx(&s_bar[0], pbytes);
      bulk_load_1d(plane, P.work + zoff, pbytes, &s_bar[0], pol);
    }
    mbar_expect_tx(&s_bar[1], pbytes);
    bulk_load_1d(Es, P.E + zoff, pbytes, &s_bar[1], pol);
  }
  // bounded wait on stage barrier b, phase ph (all threads)
  // (err[1] is the poll limit of the first try: kWaitPolls unless lowered
  // with scft_set_wait_limit)
  const int first_polls = STAGE ? err[1] : 0;
  auto stage_wait = [&](int b, uint32_t ph) {
    if (!mbar_wait(&s_bar[b], ph, first_polls)) {
      atomicExch(err, 1);
      mbar_wait(&s_bar[b], ph, kWaitPolls);  // let copies in flight land before the CTA moves on
    }
  };
  // previous step's means (FP64, same summation order in every CTA) and the
  // power-of-two exponents chosen from them
  __shared__ float s_mh[2], s_ml[2];  // the step means as two-float pairs (split once)
  if (warp == 0) {
    double a = 0.0, b = 0.0;
    if (n > 0) {
      const double *pq = P.part + (long long)(n - 1) * nz;
      const double *pd = P.part + (long long)(N + n - 1) * nz;
      for (int z = lane; z < nz; z += 32) {
        a += pq[z];
        b += pd[z];
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      const double ma = a / (double)M, mb = b / (double)M;
      int ea = 0, eb = 0;
      if (n > 0 && isfinite(ma) && ma > 0.0) frexp(ma, &ea);
      if (n > 0 && isfinite(mb) && mb > 0.0) frexp(mb, &eb);
      s_exp[0] = ea;
      s_exp[1] = eb;
      s_mh[0] = (float)ma;
      s_ml[0] = (float)(ma - (double)s_mh[0]);
      s_mh[1] = (float)mb;
      s_ml[1] = (float)(mb - (double)s_mh[1]);
    }
  }
  load_tw<float>(twx, twbuf, g.ax[0]);
  load_tw<float>(twy, twbuf, g.ax[1]);
  const C *Ew = STAGE ? Es : P.E + zoff;
  C *work = P.work + zoff;
  const bool useA_q = (Na > 0 && n < Na);
  const bool useA_d = !(n <= N - Na - 1);
  if (STAGE) __syncthreads();  // barriers initialised
  if (n == 0) {
    if (STAGE) stage_wait(1, 0);
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const C v = Ew[e];
      plane[e] = make_float2(useA_q ? v.x : v.y, useA_d ? v.x : v.y);
    }
    __syncthreads();
  } else {
    if (STAGE) {
      stage_wait(0, 0);
    } else {
      // four independent loads in flight per thread and round
      for (int e0 = threadIdx.x; e0 < E; e0 += 4 * blockDim.x) {
        C w4[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = e0 + u * blockDim.x;
          if (e < E) w4[u] = work[e];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = e0 + u * blockDim.x;
          if (e < E) plane[e] = w4[u];
        }
      }
    }
    __syncthreads();
    if (PP)
      cur = fft_plane_pp<float, +1>(plane, plane2, g, twx, twy);
    else
      fft_plane<float, +1, MAXV>(plane, g, twx, twy);
    if (STAGE) stage_wait(1, 0);
  }
  const int eq = s_exp[0], ed = s_exp[1];
  const int Kq = (n == 0) ? 0 : P.K[n - 1] + eq;
  const int Kd = (n == 0) ? 0 : P.K[N + n - 1] + ed;
  if (n > 0) {
    // q = (conv + mean) * e^{-w} * 2^{-e}, the mean as a two-float constant
    const float sq = ldexpf(1.0f, -eq), sd = ldexpf(1.0f, -ed);
    const float mq_hi = s_mh[0], mq_lo = s_ml[0];
    const float md_hi = s_mh[1], md_lo = s_ml[1];
    for (int e0 = threadIdx.x; e0 < E; e0 += 4 * blockDim.x) {
      C v4[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int e = e0 + u * blockDim.x;
        if (e < E) v4[u] = Ew[e];
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int e = e0 + u * blockDim.x;
        if (e >= E) break;
        const C v = v4[u];
        const C z = cur[e];
        const float eq_ = useA_q ? v.x : v.y, ed_ = useA_d ? v.x : v.y;
        const float uq = fmaf(z.x, eq_, fmaf(mq_hi, eq_, mq_lo * eq_));
        const float ud = fmaf(z.y, ed_, fmaf(md_hi, ed_, md_lo * ed_));
        cur[e] = make_float2(uq * sq, ud * sd);
      }
    }
  }
  if (jb.z == 0 && threadIdx.x == 0) {
    P.K[n] = Kq;
    P.K[N + n] = Kd;
  }
  if (STAGE && m2 < n) {
    // every thread is done with the Boltzmann buffer: reuse it for the
    // stored partner plane, which arrives while the history is stored
    __syncthreads();
    if (threadIdx.x == 0) {
      fence_proxy_async_smem();
      mbar_expect_tx(&s_bar[1], pbytes);
      bulk_load_1d(Es, P.hist + (long long)m2 * M + zoff, pbytes, &s_bar[1], l2_policy_first());
    }
  }
  // history (first half) and plane sums (mean of the next step, Q): each
  // thread sums its few values in FP32, the warp with error-free FP32
  // two-sums, the block in FP64 (one value per warp: GB300 runs FP64 at a
  // small fraction of the FP32 rate)
  float aqf = 0.f, adf = 0.f;
  C *hst = P.hist + (long long)n * M + zoff;
  const bool keep = (n <= P.hmax);
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    const C z = cur[e];
    aqf += z.x;
    adf += z.y;
    if (keep) hst[e] = z;
  }
  // density terms, relative to the reference exponent Kref
  const int n0 = N / 2;  // first step that adds a term
  if (m2 <= n) {
    const int Kref = (n == n0) ? Kq + (m2 == n ? Kd : P.K[N + m2]) : P.K[2 * N];
    if (n == n0 && jb.z == 0 && threadIdx.x == 0) P.K[2 * N] = Kref;
    if (m2 < n) {
      if (STAGE) stage_wait(1, 1);
      const C *o = STAGE ? Es : P.hist + (long long)m2 * M + zoff;
      const float f1 = ldexpf(1.0f, Kq + P.K[N + m2] - Kref);  // q_n * qdag_{m2}
      const float f2 = ldexpf(1.0f, P.K[m2] + Kd - Kref);      // q_{m2} * qdag_n
      float *a1 = P.acc[n < Na ? 0 : 1] + zoff;
      float *a2 = P.acc[m2 < Na ? 0 : 1] + zoff;
      const bool same = (a1 == a2);
      for (int e0 = threadIdx.x; e0 < E; e0 += 4 * blockDim.x) {
        C h4[4];
        float b1[4], b2[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = e0 + u * blockDim.x;
          if (e < E) {
            h4[u] = o[e];
            b1[u] = a1[e];
            if (!same) b2[u] = a2[e];
          }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = e0 + u * blockDim.x;
          if (e >= E) break;
          const C z = cur[e], h = h4[u];
          if (same) {
            a1[e] = b1[u] + fmaf(z.x * h.y, f1, (h.x * z.y) * f2);
          } else {
            a1[e] = b1[u] + (z.x * h.y) * f1;
            a2[e] = b2[u] + (h.x * z.y) * f2;
          }
        }
      }
    } else {
      const float f = ldexpf(1.0f, Kq + Kd - Kref);
      float *a1 = P.acc[n < Na ? 0 : 1] + zoff;
      for (int e = threadIdx.x; e < E; e += blockDim.x) {
        const C z = cur[e];
        a1[e] += (z.x * z.y) * f;
      }
    }
  }
  {
    float cq = 0.f, cd = 0.f;
    for (int o = 16; o > 0; o >>= 1) {
      const float s2 = __shfl_down_sync(0xffffffffu, aqf, o), c2 = __shfl_down_sync(0xffffffffu, cq, o);
      const float t2 = __shfl_down_sync(0xffffffffu, adf, o), d2 = __shfl_down_sync(0xffffffffu, cd, o);
      float sa = aqf + s2, va = sa - aqf;
      cq += c2 + ((aqf - (sa - va)) + (s2 - va));
      aqf = sa;
      float sb = adf + t2, vb = sb - adf;
      cd += d2 + ((adf - (sb - vb)) + (t2 - vb));
      adf = sb;
    }
    if (lane == 0) {
      s_red[0][warp] = (double)aqf + (double)cq;
      s_red[1][warp] = (double)adf + (double)cd;
    }
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    double aq = lane < nw ? s_red[0][lane] : 0.0;
    double ad = lane < nw ? s_red[1][lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      aq += __shfl_down_sync(0xffffffffu, aq, o);
      ad += __shfl_down_sync(0xffffffffu, ad, o);
    }
    if (lane == 0) {
      P.part[(long long)n * nz + jb.z] = aq;
      P.part[(long long)(N + n) * nz + jb.z] = ad;
    }
  }
  if (n == N - 1) return;
  __syncthreads();
  if (PP) {
    cur = fft_plane_pp<float, -1>(cur, cur == plane ? plane2 : plane, g, twx, twy);
  } else {
    fft_plane<float, -1, MAXV>(plane, g, twx, twy);
  }
  for (int e = threadIdx.x; e < E; e += blockDim.x) work[e] = cur[e];
}

// Graft sweeps of the mixed form (code/grafted_nanoparticle.cpp:15-117), one
// real propagator through the complex FP32 transform (imaginary part zero):
// sweep 0 advances q_g from the free end, q_g[0] = e^{-smwg}, and stores
// every step; sweep 1 advances qdag_g from qdag_g[0] = grafts e^{-smwg} /
// q_g[Ng-1] and accumulates qdag_g[n] q_g[Ng-1-n].  Mean in FP64 and
// power-of-two rescaling exactly as in the diblock sweep; with qdag_g[0]
// scaled by 2^-K[0][Ng-1] the products need no reference exponent.
template <int MAXV>
__global__ void __launch_bounds__(MAXV == 16 ? 1024 : 512, 1) k_mix_graft_plane(const PropJob *__restrict__ jobs,
                                                        const GraftMixInst *__restrict__ insts,
                                                        const DevGeom *__restrict__ geoms,
                                                        const float2 *__restrict__ twbuf, int sweep, int n) {
  typedef float2 C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_red[32];
  __shared__ float s_mh, s_ml;
  __shared__ int s_exp;
  const PropJob jb = jobs[blockIdx.x];
  const GraftMixInst &P = insts[jb.inst];
  const int Ng = P.Ng;
  if (n >= Ng) return;
  const DevGeom g = geoms[P.geom];
  const int E = g.nx * g.ny;
  const int nz = g.nz;
  C *plane = reinterpret_cast<C *>(smem_raw);
  C *twx = plane + E;
  C *twy = twx + g.nx;
  const long long zoff = (long long)jb.z * E;
  const long long M = g.M;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *part = P.part + (long long)sweep * Ng * nz;
  int *K = P.K + sweep * Ng;
  if (warp == 0) {
    double a = 0.0;
    if (n > 0)
      for (int z = lane; z < nz; z += 32) a += part[(long long)(n - 1) * nz + z];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) {
      const double ma = a / (double)M;
      int ea = 0;
      if (n > 0 && isfinite(ma) && ma > 0.0) frexp(ma, &ea);
      s_exp = ea;
      s_mh = (float)ma;
      s_ml = (float)(ma - (double)s_mh);
    }
  }
  load_tw<float>(twx, twbuf, g.ax[0]);
  load_tw<float>(twy, twbuf, g.ax[1]);
  const float *Eg = P.Eg + zoff;
  C *work = P.work + zoff;
  if (n == 0) {
    if (sweep == 0) {
      for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = make_float2(Eg[e], 0.f);
    } else {
      const float *last = P.hist + (long long)(Ng - 1) * M + zoff;
      const double2 *gr = P.grafts + zoff;
      for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = make_float2((float)gr[e].x * Eg[e] / last[e], 0.f);
    }
    __syncthreads();
  } else {
    for (int e = threadIdx.x; e < E; e += blockDim.x) plane[e] = work[e];
    __syncthreads();
    fft_plane<float, +1, MAXV>(plane, g, twx, twy);
  }
  const int ex = s_exp;
  const int Kn = (n > 0) ? K[n - 1] + ex : (sweep == 0 ? 0 : -P.K[Ng - 1]);
  if (n > 0) {
    const float sc = ldexpf(1.0f, -ex);
    const float m_hi = s_mh, m_lo = s_ml;
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const float eg = Eg[e];
      plane[e] = make_float2(fmaf(plane[e].x, eg, fmaf(m_hi, eg, m_lo * eg)) * sc, 0.f);
    }
  }
  if (jb.z == 0 && threadIdx.x == 0) K[n] = Kn;
  float af = 0.f;
  if (sweep == 0) {
    float *h = P.hist + (long long)n * M + zoff;
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const float v = plane[e].x;
      af += v;
      h[e] = v;
    }
  } else {
    const float *o = P.hist + (long long)(Ng - 1 - n) * M + zoff;
    const float f = ldexpf(1.0f, Kn + P.K[Ng - 1 - n]);
    float *acc = P.acc + zoff;
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const float v = plane[e].x;
      af += v;
      acc[e] += (v * o[e]) * f;
    }
  }
  double a = (double)af;
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if (lane == 0) s_red[warp] = a;
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    a = lane < nw ? s_red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) part[(long long)n * nz + jb.z] = a;
  }
  if (n == Ng - 1) return;
  __syncthreads();
  fft_plane<float, -1, MAXV>(plane, g, twx, twy);
  for (int e = threadIdx.x; e < E; e += blockDim.x) work[e] = plane[e];
}

template <int MAXV>
static cudaError_t launch_mix_graft_t(const LaunchShape &ls, const PropJob *jobs, int njobs,
                                      const GraftMixInst *insts, const DevGeom *geoms, const void *tw, int sweep,
                                      int n, cudaStream_t st) {
  auto kfn = k_mix_graft_plane<MAXV>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, ls.smem);
  if (e != cudaSuccess) return e;
  kfn<<<njobs, ls.threads, ls.smem, st>>>(jobs, insts, geoms, reinterpret_cast<const float2 *>(tw), sweep, n);
  return cudaGetLastError();
}

cudaError_t launch_mix_graft_plane(const LaunchShape &ls, const PropJob *jobs, int njobs, const GraftMixInst *insts,
                                   const DevGeom *geoms, const void *tw, int sweep, int n, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (ls.maxv <= 8) return launch_mix_graft_t<8>(ls, jobs, njobs, insts, geoms, tw, sweep, n, st);
  if (ls.maxv <= 16) return launch_mix_graft_t<16>(ls, jobs, njobs, insts, geoms, tw, sweep, n, st);
  return launch_mix_graft_t<32>(ls, jobs, njobs, insts, geoms, tw, sweep, n, st);
}

template <int MAXV, bool STAGE, bool PP>
static cudaError_t launch_mix_t(const LaunchShape &ls, const PropJob *jobs, int njobs, const MixInst *insts,
                                const DevGeom *geoms, const void *tw, int n, int *err, cudaStream_t st) {
  auto kfn = k_mix_prop_plane<MAXV, STAGE, PP>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, ls.smem);
  if (e != cudaSuccess) return e;
  kfn<<<njobs, ls.threads, ls.smem, st>>>(jobs, insts, geoms, reinterpret_cast<const float2 *>(tw), n, err);
  return cudaGetLastError();
}

cudaError_t launch_mix_prop_plane(const LaunchShape &ls, const PropJob *jobs, int njobs, const MixInst *insts,
                                  const DevGeom *geoms, const void *tw, int n, int *err, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (ls.pp) {  // the value bound does not apply out of place
    if (ls.stage) {
      if (!err) return cudaErrorInvalidValue;
      return launch_mix_t<8, true, true>(ls, jobs, njobs, insts, geoms, tw, n, err, st);
    }
    return launch_mix_t<8, false, true>(ls, jobs, njobs, insts, geoms, tw, n, err, st);
  }
  if (ls.stage) return cudaErrorInvalidValue;  // staging is laid out for the out-of-place form
  if (ls.maxv <= 8) return launch_mix_t<8, false, false>(ls, jobs, njobs, insts, geoms, tw, n, err, st);
  if (ls.maxv <= 16) return launch_mix_t<16, false, false>(ls, jobs, njobs, insts, geoms, tw, n, err, st);
  return launch_mix_t<32, false, false>(ls, jobs, njobs, insts, geoms, tw, n, err, st);
}

}  // namespace scft
