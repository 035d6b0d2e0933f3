// kernels_mixed48.cu -- the mixed-form propagator step for 48 x 48 x 48 grids
// (the 48^3 instances of the mixed-size sweep), same arithmetic contract as
// kernels_mixed.cu and kernels_mixed64.cu.
//
// A 48-point transform is done by a group of 4 threads, thread t holding the
// 12 values x[t + 4a] (fft48_group, mix_core.cuh: DFT12 in registers,
// twiddle, one exchange, three DFT4), so a 48 x 48 plane is 192 threads x 12
// values in one CTA: the plane pass is the 64-point pass's structure (column
// phase, padded transpose, row phase inside one warp, pointwise step, back)
// with that transform; the z pass runs 4 threads per z column.
#include "inst.h"
#include "launch.h"
#include "mix_core.cuh"
#include "prop_launch.h"

#include <string.h>

namespace scft {

namespace {

// Padded row stride (float2) of a 48 x 48 plane: the row exchange area
// (4 threads x 12 values at stride 13) fits a row, and a half-warp's four
// rows x four threads fall on distinct 8-byte slots.
constexpr int kRP48 = 52;

// Element (row, x) of a 48-row plane staged by three 48 x 128 B boxes with
// the 128-byte swizzle: box x / 16, 16-byte chunk ((x % 16) / 2) ^ (row % 8).
__device__ __forceinline__ float2 swz48(const float2 *plane, int row, int x) {
  return plane[(x >> 4) * 768 + row * 16 + ((((x & 15) >> 1) ^ (row & 7)) << 1) + (x & 1)];
}

}  // namespace

struct Plane48Shared {
  float2 tw[48];       // 48-point twiddles
  double red[2][6];    // per-warp plane sums
  float mh[2], ml[2];  // step means as two-float pairs
  int exp[2];          // power-of-two exponents of the step
};

// Plane pass of step n for 48 x 48 xy planes (nz the same for every instance
// of the launch), 192 threads, one CTA per (instance, z plane): CTA b works
// on plane b % nz of T.inst[b / nz].  Dynamic shared memory (1024-byte
// aligned): the TMA-staged Boltzmann and history planes (18 KB each), then
// the padded exchange/transpose plane (19.5 KB).
// T.tmE / T.tmH: E32 and hist32 as rows of 48 float2 (96 floats), boxes of
// 48 rows x 32 floats, 128-byte swizzle.
template <int CAP>
__global__ void __launch_bounds__(192, 3) k_mix_plane48(const __grid_constant__ Mix64TableT<CAP> T,
                                                        const float2 *__restrict__ tw_g, int n) {
  extern __shared__ __align__(16) unsigned char dsm_raw[];
  float2 *Es = reinterpret_cast<float2 *>(dsm_raw + ((1024 - (smem_u32(dsm_raw) & 1023)) & 1023));
  float2 *Hs = Es + 2304;
  float2 *buf = Hs + 2304;
  __shared__ Plane48Shared S;
  __shared__ __align__(8) uint64_t s_bar;
  const int nz = T.nz;
  const int ii = blockIdx.x / nz;
  const int zz = blockIdx.x - ii * nz;
  const MixInst &P = T.inst[ii];
  const int N = P.N, Na = P.Na;
  if (n >= N) return;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const long long M = 2304LL * nz;
  const long long zoff = (long long)zz * 2304;
  // row phase: (y = row, x = tr + 4a); column phase: (y = tc + 4a, x = col)
  const int row = tid >> 2, tr = tid & 3;
  const int col = tid % 48, tc = tid / 48;
  if (tid == 0) mbar_init(&s_bar, 1);
  if (tid < 48) S.tw[tid] = tw_g[tid];
  float2 v[12];
  float2 *work = P.work + zoff;
  if (n > 0) {
#pragma unroll
    for (int a = 0; a < 12; a++) v[a] = work[(tc + 4 * a) * 48 + col];
  }
  const int m2 = N - 1 - n;
  const bool pair = (m2 < n);
  const uint64_t pol_first = l2_policy_first();
  __syncthreads();  // barrier initialised
  if (tid == 0) {
    mbar_expect_tx(&s_bar, pair ? 36864u : 18432u);
    const uint64_t pol_last = l2_policy_last();
    for (int b = 0; b < 3; b++) tma_load_2d(Es + b * 768, &T.tmE[ii], 32 * b, zz * 48, &s_bar, pol_last);
    if (pair)
      for (int b = 0; b < 3; b++) tma_load_2d(Hs + b * 768, &T.tmH[ii], 32 * b, (m2 * nz + zz) * 48, &s_bar, pol_first);
  }
  const int gi = row * 48 + tr;  // plane index of element a = 0 (row phase)
  float *a1 = P.acc[n < Na ? 0 : 1] + zoff + gi;
  float *a2 = P.acc[m2 < Na ? 0 : 1] + zoff + gi;
  const bool same_acc = (a1 == a2);
  if (warp < 2) {
    // warp 0: mean of q_{n-1}; warp 1: mean of qdag_{n-1}
    double a = 0.0;
    if (n > 0) {
      const double *pp = P.part + (long long)(warp * N + n - 1) * nz;
      for (int z = lane; z < nz; z += 32) a += pp[z];
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) {
      const double ma = a / (double)M;
      int ea = 0;
      if (n > 0 && isfinite(ma) && ma > 0.0) frexp(ma, &ea);
      S.exp[warp] = ea;
      const float hi = (float)ma;
      S.mh[warp] = hi;
      S.ml[warp] = (float)(ma - (double)hi);
    }
  }
  const bool useA_q = (Na > 0 && n < Na);
  const bool useA_d = !(n <= N - Na - 1);
  __syncthreads();  // means, exponents, twiddles
  if (n > 0) {
    // inverse y (column phase), transpose, inverse x (row phase, in one warp)
    fft48_group<+1, false>(v, tc, buf + col, 12 * 48, 48, S.tw);
#pragma unroll
    for (int d = 0; d < 12; d++) buf[(tc + 4 * d) * kRP48 + col] = v[d];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 12; a++) v[a] = buf[row * kRP48 + tr + 4 * a];
    // a row's exchange area lies inside its padded row, and a warp owns whole
    // rows: a warp barrier suffices
    __syncwarp();
    fft48_group<+1, true>(v, tr, buf + row * kRP48, 13, 1, S.tw);
  }
  if (!mbar_wait(&s_bar, 0, T.err[1])) {
    atomicExch(T.err, 1);
    mbar_wait(&s_bar, 0, kWaitPolls);  // let copies in flight land before the CTA moves on
  }
  if (n == 0) {
#pragma unroll
    for (int a = 0; a < 12; a++) {
      const float2 e = swz48(Es, row, tr + 4 * a);
      v[a] = make_float2(useA_q ? e.x : e.y, useA_d ? e.x : e.y);
    }
  } else {
    const int eq = S.exp[0], ed = S.exp[1];
    const float sq = ldexpf(1.0f, -eq), sd = ldexpf(1.0f, -ed);
    const float mq_hi = S.mh[0], mq_lo = S.ml[0];
    const float md_hi = S.mh[1], md_lo = S.ml[1];
#pragma unroll
    for (int a = 0; a < 12; a++) {
      const float2 e = swz48(Es, row, tr + 4 * a);
      const float eq_ = useA_q ? e.x : e.y, ed_ = useA_d ? e.x : e.y;
      const float uq = fmaf(v[a].x, eq_, fmaf(mq_hi, eq_, mq_lo * eq_));
      const float ud = fmaf(v[a].y, ed_, fmaf(md_hi, ed_, md_lo * ed_));
      v[a] = make_float2(uq * sq, ud * sd);
    }
  }
  const int Kq = (n == 0) ? 0 : P.K[n - 1] + S.exp[0];
  const int Kd = (n == 0) ? 0 : P.K[N + n - 1] + S.exp[1];
  if (zz == 0 && tid == 0) {
    P.K[n] = Kq;
    P.K[N + n] = Kd;
  }
  if (n <= P.hmax) {
    float2 *hst = P.hist + (long long)n * M + zoff + gi;
#pragma unroll
    for (int a = 0; a < 12; a++) st_stream(hst + 4 * a, v[a], pol_first);
  }
  const int n0 = N / 2;
  if (m2 <= n) {
    const int Kref = (n == n0) ? Kq + (m2 == n ? Kd : P.K[N + m2]) : P.K[2 * N];
    if (n == n0 && zz == 0 && tid == 0) P.K[2 * N] = Kref;
    if (pair) {
      const float f1 = ldexpf(1.0f, Kq + P.K[N + m2] - Kref);
      const float f2 = ldexpf(1.0f, P.K[m2] + Kd - Kref);
      if (same_acc) {
#pragma unroll
        for (int a = 0; a < 12; a++) {
          const float2 h = swz48(Hs, row, tr + 4 * a);
          a1[4 * a] += fmaf(v[a].x * h.y, f1, (h.x * v[a].y) * f2);
        }
      } else {
#pragma unroll
        for (int a = 0; a < 12; a++) {
          const float2 h = swz48(Hs, row, tr + 4 * a);
          a1[4 * a] += (v[a].x * h.y) * f1;
          a2[4 * a] += (h.x * v[a].y) * f2;
        }
      }
    } else {
      const float f = ldexpf(1.0f, Kq + Kd - Kref);
#pragma unroll
      for (int a = 0; a < 12; a++) a1[4 * a] += (v[a].x * v[a].y) * f;
    }
  }
  // plane sums: error-free FP32 two-sums within the thread and the warp
  float sq_ = 0.f, cq = 0.f, sd_ = 0.f, cd = 0.f;
#pragma unroll
  for (int a = 0; a < 12; a++) {
    float e;
    two_sum(sq_, v[a].x, sq_, e);
    cq += e;
    two_sum(sd_, v[a].y, sd_, e);
    cd += e;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_down_sync(0xffffffffu, sq_, o), c2 = __shfl_down_sync(0xffffffffu, cq, o);
    const float t2 = __shfl_down_sync(0xffffffffu, sd_, o), d2 = __shfl_down_sync(0xffffffffu, cd, o);
    float e;
    two_sum(sq_, s2, sq_, e);
    cq += c2 + e;
    two_sum(sd_, t2, sd_, e);
    cd += d2 + e;
  }
  if (lane == 0) {
    S.red[0][warp] = (double)sq_ + (double)cq;
    S.red[1][warp] = (double)sd_ + (double)cd;
  }
  // warp 0 sums the warp results after the next block barrier: the forward
  // transpose's (the forward row transform only touches the warp's own rows
  // of buf), or on the last step a barrier of its own
  const bool last = (n == N - 1);
  if (!last) {
    fft48_group<-1, true>(v, tr, buf + row * kRP48, 13, 1, S.tw);
#pragma unroll
    for (int a = 0; a < 12; a++) buf[row * kRP48 + tr + 4 * a] = v[a];
  }
  __syncthreads();  // also: every read of Es, Hs and every write of S.red is done
  if (warp == 0) {
    double aq = lane < 6 ? S.red[0][lane] : 0.0;
    double ad = lane < 6 ? S.red[1][lane] : 0.0;
    for (int o = 4; o > 0; o >>= 1) {
      aq += __shfl_down_sync(0xffffffffu, aq, o);
      ad += __shfl_down_sync(0xffffffffu, ad, o);
    }
    if (lane == 0) {
      P.part[(long long)n * nz + zz] = aq;
      P.part[(long long)(N + n) * nz + zz] = ad;
    }
  }
  if (last) return;
  // to the column phase, forward y (the exchange goes through the consumed
  // Boltzmann plane Es, so no barrier between the transposed reads and it)
#pragma unroll
  for (int a = 0; a < 12; a++) v[a] = buf[(tc + 4 * a) * kRP48 + col];
  fft48_group<-1, false>(v, tc, Es + col, 12 * 48, 48, S.tw);
#pragma unroll
  for (int d = 0; d < 12; d++) work[(tc + 4 * d) * 48 + col] = v[d];
}

// z pass for nz = 48, the contract of k_mix_col64: tile of 16 x columns at
// one y, 4 threads per column.
__global__ void __launch_bounds__(64) k_mix_col48(const ColJob *__restrict__ jobs, const float2 *__restrict__ tw_g,
                                                  int nx, int ny, float s_hi, float s_lo) {
  constexpr int TX = 16;
  __shared__ __align__(16) float2 buf[48 * TX];
  __shared__ float2 tw[48];
  const ColJob jb = jobs[blockIdx.x];
  const int tid = threadIdx.x;
  const int col = tid % TX, t = tid / TX;
  if (tid < 48) tw[tid] = tw_g[tid];
  const long long plane = (long long)nx * ny;
  const long long base = (long long)jb.y * nx + jb.x0 + col;
  float2 *a = reinterpret_cast<float2 *>(jb.ptr);
  const float *ht = reinterpret_cast<const float *>(jb.kern);
  const float hx = ht[jb.x0 + col], hy = ht[nx + jb.y];
  const float hxy = fmaf(-hx, hy, hx + hy);
  float2 v[12];
#pragma unroll
  for (int j = 0; j < 12; j++) v[j] = a[(t + 4 * j) * plane + base];
  __syncthreads();  // tw
  fft48_group<-1, false>(v, t, buf + col, 12 * TX, TX, tw);
#pragma unroll
  for (int d = 0; d < 12; d++) {
    const int kz = t + 4 * d;
    const float hz = ht[nx + ny + kz];
    const float hv = fmaf(-hxy, hz, hxy + hz);
    float2 u = make_float2(fmaf(v[d].x, s_hi, v[d].x * s_lo), fmaf(v[d].y, s_hi, v[d].y * s_lo));
    u = make_float2(fmaf(-hv, u.x, u.x), fmaf(-hv, u.y, u.y));
    if (kz == 0 && jb.y == 0 && jb.x0 + col == 0) u = make_float2(0.f, 0.f);
    v[d] = u;
  }
  fft48_group<+1, false>(v, t, buf + col, 12 * TX, TX, tw);
#pragma unroll
  for (int j = 0; j < 12; j++) a[(t + 4 * j) * plane + base] = v[j];
}

cudaError_t launch_mix_col48(const ColJob *jobs, int njobs, const void *tw48, int nx, int ny, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  const double s = 1.0 / ((double)nx * ny * 48.0);
  const float s_hi = (float)s, s_lo = (float)(s - (double)s_hi);
  k_mix_col48<<<njobs, 64, 0, st>>>(jobs, reinterpret_cast<const float2 *>(tw48), nx, ny, s_hi, s_lo);
  return cudaGetLastError();
}

template <int CAP>
static cudaError_t launch_plane48_chunks(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH,
                                         int ninst, int nz, const void *tw48, int n, int *err, cudaStream_t st) {
  const int smem = 1024 + 2 * 2304 * (int)sizeof(float2) + 48 * kRP48 * (int)sizeof(float2);
  auto kfn = k_mix_plane48<CAP>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  for (int i0 = 0; i0 < ninst; i0 += CAP) {
    const int cnt = ninst - i0 < CAP ? ninst - i0 : CAP;
    Mix64TableT<CAP> T;
    memset(&T, 0, sizeof T);
    for (int k = 0; k < cnt; k++) {
      T.inst[k] = insts[i0 + k];
      T.tmE[k] = tmE[i0 + k];
      T.tmH[k] = tmH[i0 + k];
    }
    T.err = err;
    T.nz = nz;
    kfn<<<nz * cnt, 192, smem, st>>>(T, reinterpret_cast<const float2 *>(tw48), n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_mix_plane48(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                               int nz, const void *tw48, int n, int *err, cudaStream_t st) {
  if (ninst <= 0) return cudaSuccess;
  if (ninst <= 4) return launch_plane48_chunks<4>(insts, tmE, tmH, ninst, nz, tw48, n, err, st);
  return launch_plane48_chunks<16>(insts, tmE, tmH, ninst, nz, tw48, n, err, st);
}

}  // namespace scft
