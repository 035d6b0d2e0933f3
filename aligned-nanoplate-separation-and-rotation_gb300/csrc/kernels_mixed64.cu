// kernels_mixed64.cu -- the mixed-form propagator step specialised for 64-point
// axes (the 64^3 workloads), same arithmetic contract as kernels_mixed.cu and
// the generic column pass (mode 3).
//
// A 64-point transform is done by a group of 8 threads, thread t holding the
// 8 values x[t + 8a], a = 0..7 ("four-step", 64 = 8 x 8):
//   Y[t][c]  = sum_a x[8a + t] w8^(a c)          (DFT8 in registers)
//   Y[t][c] *= w64^(t c)                          (twiddle)
//   exchange through shared memory so that thread t holds Y[b][t], b = 0..7
//   X[t + 8d] = sum_b Y[b][t] w8^(b d)            (DFT8 in registers)
// so the output comes back in the same "t + 8j" order as the input.  Shared
// layouts are padded so that every exchange is free of bank conflicts, and no
// index needs a runtime division.
#include "fft_core.cuh"
#include "inst.h"
#include "launch.h"
#include "prop_launch.h"

namespace scft {

namespace {

constexpr int kRowPad = 72;  // padded row stride (float2) of the 64 x 64 plane buffer

template <int SIGN> __device__ __forceinline__ void dft8f(float2 *v) { Dft<8, SIGN, float2>::run(v); }

// twiddle multiply by w64^(t c) (SIGN < 0) or its conjugate
template <int SIGN> __device__ __forceinline__ void tw64(float2 *v, int t, const float2 *tw) {
#pragma unroll
  for (int c = 1; c < 8; c++) v[c] = ctw<SIGN>(v[c], tw[t * c]);
}

// 64-point transform of a group of 8 threads.  Thread t of the group holds
// v[a] = x[t + 8a]; the exchange goes through xch with element (b, c) of the
// group at xch[b * sb + c * sc] (strides chosen by the caller so that a warp's
// accesses spread over the banks).  On return v[d] = X[t + 8d].
template <int SIGN>
__device__ __forceinline__ void fft64_group(float2 *v, int t, float2 *xch, int sb, int sc, const float2 *tw) {
  dft8f<SIGN>(v);
  tw64<SIGN>(v, t, tw);
#pragma unroll
  for (int c = 0; c < 8; c++) xch[t * sb + c * sc] = v[c];
  __syncthreads();
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = xch[b * sb + t * sc];
  __syncthreads();
  dft8f<SIGN>(v);
}

}  // namespace

// Plane pass of step n for 64 x 64 xy planes, 512 threads: column phase
// (thread = column x, part t) for the y transforms, row phase (thread = row y,
// part t) for the x transforms and all pointwise work.
__global__ void __launch_bounds__(512, 2) k_mix_plane64(const PropJob *__restrict__ jobs,
                                                        const MixInst *__restrict__ insts,
                                                        const float2 *__restrict__ tw_g, int n) {
  __shared__ __align__(16) float2 buf[64 * kRowPad];
  __shared__ float2 tw[64];
  __shared__ double s_red[2][16];
  __shared__ double s_mu[2];
  __shared__ int s_exp[2];
  const PropJob jb = jobs[blockIdx.x];
  const MixInst &P = insts[jb.inst];
  const int N = P.N, Na = P.Na;
  if (n >= N) return;
  const int nz = 64;
  const long long M = 64LL * 64 * 64;
  const long long zoff = (long long)jb.z * 4096;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  if (tid < 64) tw[tid] = tw_g[tid];
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
      s_mu[0] = ma;
      s_mu[1] = mb;
    }
  }
  // row-phase coordinates: this thread owns (y = row, x = t + 8d)
  const int row = tid >> 3, tr = tid & 7;
  // column-phase coordinates: this thread owns (y = tc + 8d, x = col)
  const int col = tid & 63, tc = tid >> 6;
  float2 v[8];
  const float2 *Ew = P.E + zoff;
  float2 *work = P.work + zoff;
  const bool useA_q = (Na > 0 && n < Na);
  const bool useA_d = !(n <= N - Na - 1);
  __syncthreads();  // tw, s_mu, s_exp
  if (n == 0) {
#pragma unroll
    for (int d = 0; d < 8; d++) {
      const float2 e = Ew[row * 64 + tr + 8 * d];
      v[d] = make_float2(useA_q ? e.x : e.y, useA_d ? e.x : e.y);
    }
  } else {
    // inverse y transform (column phase)
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = work[(tc + 8 * a) * 64 + col];
    fft64_group<+1>(v, tc, buf + col, 8 * 64, 64, tw);
    // to the row phase through the padded plane
#pragma unroll
    for (int d = 0; d < 8; d++) buf[(tc + 8 * d) * kRowPad + col] = v[d];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = buf[row * kRowPad + tr + 8 * a];
    __syncthreads();
    // inverse x transform (row phase)
    fft64_group<+1>(v, tr, buf + row * kRowPad, 9, 1, tw);
    // q = (conv + mean) * e^{-w} * 2^{-e}, the mean as a two-float constant
    const int eq = s_exp[0], ed = s_exp[1];
    const float sq = ldexpf(1.0f, -eq), sd = ldexpf(1.0f, -ed);
    const double mq = s_mu[0], md = s_mu[1];
    const float mq_hi = (float)mq, mq_lo = (float)(mq - (double)mq_hi);
    const float md_hi = (float)md, md_lo = (float)(md - (double)md_hi);
#pragma unroll
    for (int d = 0; d < 8; d++) {
      const float2 e = Ew[row * 64 + tr + 8 * d];
      const float eq_ = useA_q ? e.x : e.y, ed_ = useA_d ? e.x : e.y;
      const float uq = fmaf(v[d].x, eq_, fmaf(mq_hi, eq_, mq_lo * eq_));
      const float ud = fmaf(v[d].y, ed_, fmaf(md_hi, ed_, md_lo * ed_));
      v[d] = make_float2(uq * sq, ud * sd);
    }
  }
  const int Kq = (n == 0) ? 0 : P.K[n - 1] + s_exp[0];
  const int Kd = (n == 0) ? 0 : P.K[N + n - 1] + s_exp[1];
  if (jb.z == 0 && tid == 0) {
    P.K[n] = Kq;
    P.K[N + n] = Kd;
  }
  // history, plane sums, density terms (row phase ownership)
  float aqf = 0.f, adf = 0.f;
  const bool keep = (n <= P.hmax);
  float2 *hst = P.hist + (long long)n * M + zoff;
#pragma unroll
  for (int d = 0; d < 8; d++) {
    aqf += v[d].x;
    adf += v[d].y;
    if (keep) hst[row * 64 + tr + 8 * d] = v[d];
  }
  const int m2 = N - 1 - n;
  const int n0 = N / 2;
  if (m2 <= n) {
    const int Kref = (n == n0) ? Kq + (m2 == n ? Kd : P.K[N + m2]) : P.K[2 * N];
    if (n == n0 && jb.z == 0 && tid == 0) P.K[2 * N] = Kref;
    if (m2 < n) {
      const float2 *o = P.hist + (long long)m2 * M + zoff;
      const float f1 = ldexpf(1.0f, Kq + P.K[N + m2] - Kref);
      const float f2 = ldexpf(1.0f, P.K[m2] + Kd - Kref);
      float *a1 = P.acc[n < Na ? 0 : 1] + zoff;
      float *a2 = P.acc[m2 < Na ? 0 : 1] + zoff;
#pragma unroll
      for (int d = 0; d < 8; d++) {
        const int i = row * 64 + tr + 8 * d;
        const float2 h = o[i];
        if (a1 == a2) {
          a1[i] += fmaf(v[d].x * h.y, f1, (h.x * v[d].y) * f2);
        } else {
          a1[i] += (v[d].x * h.y) * f1;
          a2[i] += (h.x * v[d].y) * f2;
        }
      }
    } else {
      const float f = ldexpf(1.0f, Kq + Kd - Kref);
      float *a1 = P.acc[n < Na ? 0 : 1] + zoff;
#pragma unroll
      for (int d = 0; d < 8; d++) {
        const int i = row * 64 + tr + 8 * d;
        a1[i] += (v[d].x * v[d].y) * f;
      }
    }
  }
  double aq = (double)aqf, ad = (double)adf;
  for (int o = 16; o > 0; o >>= 1) {
    aq += __shfl_down_sync(0xffffffffu, aq, o);
    ad += __shfl_down_sync(0xffffffffu, ad, o);
  }
  if (lane == 0) {
    s_red[0][warp] = aq;
    s_red[1][warp] = ad;
  }
  __syncthreads();
  if (warp == 0) {
    aq = lane < 16 ? s_red[0][lane] : 0.0;
    ad = lane < 16 ? s_red[1][lane] : 0.0;
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
  // forward x transform (row phase), then to the column phase, forward y
  fft64_group<-1>(v, tr, buf + row * kRowPad, 9, 1, tw);
#pragma unroll
  for (int d = 0; d < 8; d++) buf[row * kRowPad + tr + 8 * d] = v[d];
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 8; a++) v[a] = buf[(tc + 8 * a) * kRowPad + col];
  __syncthreads();
  fft64_group<-1>(v, tc, buf + col, 8 * 64, 64, tw);
#pragma unroll
  for (int d = 0; d < 8; d++) work[(tc + 8 * d) * 64 + col] = v[d];
}

// z pass for nz = 64, mode 3 of the generic column pass: tile of TX x columns
// at one y, 8 threads per column.
template <int TX>
__global__ void __launch_bounds__(8 * TX) k_mix_col64(const ColJob *__restrict__ jobs,
                                                      const float2 *__restrict__ tw_g, int nx, int ny) {
  __shared__ __align__(16) float2 buf[64 * TX];
  __shared__ float2 tw[64];
  const ColJob jb = jobs[blockIdx.x];
  const int tid = threadIdx.x;
  const int col = tid % TX, t = tid / TX;
  if (tid < 64) tw[tid] = tw_g[tid];
  const long long plane = (long long)nx * ny;
  const long long base = (long long)jb.y * nx + jb.x0 + col;
  float2 *a = reinterpret_cast<float2 *>(jb.ptr);
  const float *h = reinterpret_cast<const float *>(jb.kern);
  float2 v[8];
#pragma unroll
  for (int j = 0; j < 8; j++) v[j] = a[(t + 8 * j) * plane + base];
  __syncthreads();  // tw
  fft64_group<-1>(v, t, buf + col, 8 * TX, TX, tw);
  const double sdbl = 1.0 / (double)(plane * 64);
  const float s_hi = (float)sdbl, s_lo = (float)(sdbl - (double)s_hi);
#pragma unroll
  for (int d = 0; d < 8; d++) {
    const int kz = t + 8 * d;
    const float hv = h[kz * plane + base];
    float2 u = make_float2(fmaf(v[d].x, s_hi, v[d].x * s_lo), fmaf(v[d].y, s_hi, v[d].y * s_lo));
    u = make_float2(fmaf(-hv, u.x, u.x), fmaf(-hv, u.y, u.y));
    if (kz == 0 && jb.y == 0 && jb.x0 + col == 0) u = make_float2(0.f, 0.f);
    v[d] = u;
  }
  fft64_group<+1>(v, t, buf + col, 8 * TX, TX, tw);
#pragma unroll
  for (int j = 0; j < 8; j++) a[(t + 8 * j) * plane + base] = v[j];
}

cudaError_t launch_mix_plane64(const PropJob *jobs, int njobs, const MixInst *insts, const void *tw64,
                               int n, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  k_mix_plane64<<<njobs, 512, 0, st>>>(jobs, insts, reinterpret_cast<const float2 *>(tw64), n);
  return cudaGetLastError();
}

cudaError_t launch_mix_col64(const ColJob *jobs, int njobs, const void *tw64, int nx, int ny, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  k_mix_col64<16><<<njobs, 128, 0, st>>>(jobs, reinterpret_cast<const float2 *>(tw64), nx, ny);
  return cudaGetLastError();
}

}  // namespace scft
