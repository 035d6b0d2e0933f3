// kernels_mixed128.cu -- the mixed-form propagator step for 128 x 128 xy planes
// (the large grafted workload: 128 x 128 x 256), same arithmetic contract as
// kernels_mixed.cu and kernels_mixed64.cu.
//
// Plane pass: a cluster of four CTAs per plane, each holding one 64 x 64
// quadrant, so that every CTA runs the 64-point machinery of the 64^3 kernels
// (8 values per thread, 512 threads, two CTAs per SM) and the 128-point
// transforms close with one radix-2 butterfly between partner CTAs, read
// through distributed shared memory.
//
// k-space layout.  A 128-point axis is stored parity-major: wavenumber k at
// position P(k) = (k % 2) 64 + k / 2, on both x and y of every plane of the
// working array between the plane pass and the z pass.  CTA q = rx + 2 ry of a
// plane's cluster then owns the stored quadrant px in [64 rx, 64 rx + 64),
// py in [64 ry, 64 ry + 64): the wavenumbers kx = 2 jx + rx, ky = 2 jy + ry.
// The z pass multiplies by per-axis factor tables stored in the same order,
// and the zero mode (kx = ky = 0) sits at position 0 as in natural order.
//
// Inverse transform of a plane (sign +, W = exp(2 pi i / 128)):
//   y: A_ry[m][jx] = IDFT64 over jy of the quadrant; partners ry = 0, 1 (same
//      rx) combine  y[m] = A_0[m] + W^m A_1[m],  y[m + 64] = A_0[m] - W^m A_1[m];
//      CTA ry keeps rows 64 ry + m;
//   x: B_rx[m][p] = IDFT64 over jx; partners rx = 0, 1 combine the same way;
//      CTA rx keeps columns 64 rx + p.
// Each CTA then holds the real-space quadrant x in [64 rx, +64),
// y in [64 ry, +64) in natural order: the Boltzmann factors, the history, the
// density accumulators and the plane sums are those of the 64^3 kernel on a
// quadrant (row stride 128).  The forward transform splits by decimation in
// frequency:  a[p] = x[p] + x[p + 64] -> DFT64 -> even k;
// b[p] = (x[p] - x[p + 64]) W^-p -> DFT64 -> odd k; first along x, then y.
//
// Cluster barriers: every thread of the four CTAs runs the same sequence
// (it depends only on n and the instance's N, common to the cluster).  A
// CTA's shared buffers are read by its partners only between two barriers,
// and no CTA leaves while a partner may still read them.
//
// z pass for nz = 256 (k_mix_col256): 16 threads per column, thread t holding
// the 16 values x[t + 16a]; 256 = 16 x 16:
//   Y[t][c]  = sum_a x[t + 16a] w16^(a c)         (DFT16 in registers)
//   Y[t][c] *= w256^(t c)
//   exchange through shared memory: thread t takes c = t
//   X[t + 16d] = sum_b Y[b][t] w16^(b d)           (DFT16 in registers)
// so the output returns in the input order.
#include "inst.h"
#include "launch.h"
#include "mix_core.cuh"
#include "prop_launch.h"

#include <string.h>

namespace scft {

namespace {

// Element (row, x) of a 64 x 64 exchange quadrant: rows of 64 float2 with
// bit 3 of x flipped on odd rows.  Each half-warp's access is then free of
// bank conflicts in both phases: two rows x 8 consecutive x (row phase) take
// the two 8-slot halves of the 16 eight-byte slots, and 16 consecutive x of
// one row (column phase) take all 16.
__device__ __forceinline__ int xl_idx(int row, int x) { return row * 64 + (x ^ ((row & 1) << 3)); }

template <int SIGN>
__device__ __forceinline__ void fft256_group(float2 *v, int t, float2 *xch, int sb, int sc, const float2 *tw) {
  dft16f<SIGN, 16>(v, tw);
#pragma unroll
  for (int c = 1; c < 16; c++) v[c] = ctw<SIGN>(v[c], tw[t * c]);
#pragma unroll
  for (int c = 0; c < 16; c++) xch[t * sb + c * sc] = v[c];
  __syncthreads();
#pragma unroll
  for (int b = 0; b < 16; b++) v[b] = xch[b * sb + t * sc];
  __syncthreads();
  dft16f<SIGN, 16>(v, tw);
}

}  // namespace

// z pass for nz = 256, the contract of k_mix_col64: tile of TX x columns at
// one y (8 or 16: the tile and its exchange area take 4 KB per column of
// static shared memory), 16 threads per column.
template <int TX>
__global__ void __launch_bounds__(16 * TX) k_mix_col256(const ColJob *__restrict__ jobs,
                                                        const float2 *__restrict__ tw_g, int nx, int ny, float s_hi,
                                                        float s_lo) {
  __shared__ __align__(16) float2 buf[256 * TX];
  __shared__ float2 tw[256];
  const ColJob jb = jobs[blockIdx.x];
  const int tid = threadIdx.x;
  const int col = tid % TX, t = tid / TX;
  for (int k = tid; k < 256; k += 16 * TX) tw[k] = tw_g[k];
  const long long plane = (long long)nx * ny;
  const long long base = (long long)jb.y * nx + jb.x0 + col;
  float2 *a = reinterpret_cast<float2 *>(jb.ptr);
  const float *ht = reinterpret_cast<const float *>(jb.kern);
  const float hx = ht[jb.x0 + col], hy = ht[nx + jb.y];
  const float hxy = fmaf(-hx, hy, hx + hy);
  float2 v[16];
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = a[(t + 16 * j) * plane + base];
  __syncthreads();  // tw
  fft256_group<-1>(v, t, buf + col, 16 * TX, TX, tw);
#pragma unroll
  for (int d = 0; d < 16; d++) {
    const int kz = t + 16 * d;
    const float hz = ht[nx + ny + kz];
    const float hv = fmaf(-hxy, hz, hxy + hz);
    float2 u = make_float2(fmaf(v[d].x, s_hi, v[d].x * s_lo), fmaf(v[d].y, s_hi, v[d].y * s_lo));
    u = make_float2(fmaf(-hv, u.x, u.x), fmaf(-hv, u.y, u.y));
    if (kz == 0 && jb.y == 0 && jb.x0 + col == 0) u = make_float2(0.f, 0.f);
    v[d] = u;
  }
  fft256_group<+1>(v, t, buf + col, 16 * TX, TX, tw);
#pragma unroll
  for (int j = 0; j < 16; j++) a[(t + 16 * j) * plane + base] = v[j];
}

cudaError_t launch_mix_col256(const ColJob *jobs, int njobs, const void *tw, int nx, int ny, int tx, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  const double s = 1.0 / ((double)nx * ny * 256.0);
  const float s_hi = (float)s, s_lo = (float)(s - (double)s_hi);
  const float2 *t2 = reinterpret_cast<const float2 *>(tw);
  switch (tx) {
    case 8: k_mix_col256<8><<<njobs, 128, 0, st>>>(jobs, t2, nx, ny, s_hi, s_lo); break;
    case 16: k_mix_col256<16><<<njobs, 256, 0, st>>>(jobs, t2, nx, ny, s_hi, s_lo); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Static shared scratch of one quadrant task.
struct Plane128Shared {
  float2 tw[64];       // 64-point twiddles
  float2 w128[64];     // exp(-2 pi i m / 128), m < 64: the radix-2 twiddles
  double red[2][16];   // per-warp sums of the quadrant
  double qs[2];        // quadrant sums, read by CTA 0 of the cluster
  float mh[2], ml[2];  // step means as two-float pairs
  int exp[2];          // power-of-two exponents of the step
};

// Thread roles in a quadrant task (512 threads): row phase (y = row,
// x = tr + 8d), column phase (y = tc + 8d, x = col); q = rx + 2 ry the CTA's
// rank in the cluster.
struct Quad {
  int q, rx, ry, row, tr, col, tc;
};

__device__ __forceinline__ Quad quad_roles() {
  Quad Z;
  Z.q = (int)cl_rank();
  Z.rx = Z.q & 1;
  Z.ry = Z.q >> 1;
  const int tid = threadIdx.x;
  Z.row = tid >> 3;
  Z.tr = tid & 7;
  Z.col = tid & 63;
  Z.tc = tid >> 6;
  return Z;
}

// Inverse transform of a plane: on entry v holds the CTA's k-space quadrant
// in column ownership (jy = tc + 8a, jx = col); on return the real-space
// quadrant in row ownership (x = tr + 8d of row `row`).  Two cluster
// barriers plus one split one; buf is free for the caller afterwards, but a
// partner may read it until it passes its next cluster barrier.
__device__ __forceinline__ void quad_inverse(float2 *v, float2 *buf, const Plane128Shared &S, const Quad &Z) {
  fft64_colhalf<+1, 1>(v, Z.tc, buf + Z.col, S.tw);
#pragma unroll
  for (int d = 0; d < 8; d++) buf[(Z.tc + 8 * d) * kRowPad + Z.col] = v[d];
  cl_sync();
  {
    const uint32_t rb = cl_map(buf + Z.row * kRowPad + Z.tr, (uint32_t)(Z.q ^ 2));
    const float2 w = S.w128[Z.row];
#pragma unroll
    for (int a = 0; a < 8; a++) {
      const float2 own = buf[Z.row * kRowPad + Z.tr + 8 * a];
      const float2 oth = ld_cl(rb + 8u * (uint32_t)(8 * a));
      v[a] = Z.ry == 0 ? cadd(own, ctw<+1>(oth, w)) : csub(oth, ctw<+1>(own, w));
    }
  }
  cl_arrive();  // done reading the partner's buffer
  cl_wait();    // and every partner done reading this one: buf may be overwritten
  fft64_group<+1, true>(v, Z.tr, buf + Z.row * kRowPad, 9, 1, S.tw);
#pragma unroll
  for (int d = 0; d < 8; d++) buf[Z.row * kRowPad + Z.tr + 8 * d] = v[d];
  cl_sync();
  {
    const uint32_t rb = cl_map(buf + Z.row * kRowPad + Z.tr, (uint32_t)(Z.q ^ 1));
#pragma unroll
    for (int d = 0; d < 8; d++) {
      const float2 oth = ld_cl(rb + 8u * (uint32_t)(8 * d));
      const float2 w = S.w128[Z.tr + 8 * d];
      v[d] = Z.rx == 0 ? cadd(v[d], ctw<+1>(oth, w)) : csub(oth, ctw<+1>(v[d], w));
    }
  }
}

// First half of the forward transform: the real-space quadrant v (row
// ownership) into X (xl_idx layout), for the x partner.  X must be free
// in this CTA; the caller then passes a cluster barrier (cl_sync) before
// quad_forward.
__device__ __forceinline__ void quad_forward_publish(const float2 *v, float2 *X, const Quad &Z) {
#pragma unroll
  for (int d = 0; d < 8; d++) X[xl_idx(Z.row, Z.tr + 8 * d)] = v[d];
}

// Rest of the forward transform after that barrier: x radix-2 with the x
// partner's X, DFT64 over x, y radix-2 through Y (free in this CTA) with the
// y partner, DFT64 over y; on return v holds the k-space quadrant in column
// ownership.  Ends with a cluster arrive: the caller stores v and then calls
// cl_wait() before leaving, so that no CTA leaves while a partner may still
// read its X or Y.
__device__ __forceinline__ void quad_forward(float2 *v, const float2 *X, float2 *Y, float2 *buf,
                                             const Plane128Shared &S, const Quad &Z) {
  {
    const uint32_t rb = cl_map(X, (uint32_t)(Z.q ^ 1));
#pragma unroll
    for (int d = 0; d < 8; d++) {
      const int x = Z.tr + 8 * d;
      const float2 oth = ld_cl(rb + 8u * (uint32_t)xl_idx(Z.row, x));
      v[d] = Z.rx == 0 ? cadd(v[d], oth) : ctw<-1>(csub(oth, v[d]), S.w128[x]);
    }
  }
  fft64_group<-1, true>(v, Z.tr, buf + Z.row * kRowPad, 9, 1, S.tw);
#pragma unroll
  for (int d = 0; d < 8; d++) Y[xl_idx(Z.row, Z.tr + 8 * d)] = v[d];
  cl_sync();
  {
    const uint32_t rb = cl_map(Y, (uint32_t)(Z.q ^ 2));
#pragma unroll
    for (int a = 0; a < 8; a++) {
      const int m = Z.tc + 8 * a;
      const float2 own = Y[xl_idx(m, Z.col)];
      const float2 oth = ld_cl(rb + 8u * (uint32_t)xl_idx(m, Z.col));
      v[a] = Z.ry == 0 ? cadd(own, oth) : ctw<-1>(csub(oth, own), S.w128[m]);
    }
  }
  cl_arrive();  // done reading the partners' buffers
  fft64_colhalf<-1, 0>(v, Z.tc, buf + Z.col, S.tw);
}

// Plane pass of step n for 128 x 128 xy planes (any nz, the same for every
// instance of the launch): 512 threads per CTA, clusters of four CTAs, one
// cluster per (instance, z plane): cluster b works on plane b % nz of
// T.inst[b / nz].  Dynamic shared memory (1024-byte aligned): the staged
// Boltzmann and history quadrants (32 KB each, reused as the exchange
// buffers of the forward transform once consumed), then the padded
// exchange/transpose quadrant (36.9 KB); 101 KB, two CTAs per SM.
// T.tmE / T.tmH: E32 and hist32 as rows of 128 float2 (256 floats), boxes of
// 64 rows x 32 floats, 128-byte swizzle.
template <int CAP>
__global__ void __cluster_dims__(4, 1, 1) __launch_bounds__(512, 2)
    k_mix_plane128(const __grid_constant__ Mix64TableT<CAP> T, const float2 *__restrict__ tw64_g,
                   const float2 *__restrict__ tw128_g, int n) {
  extern __shared__ __align__(16) unsigned char dsm_raw[];
  float2 *Es = reinterpret_cast<float2 *>(dsm_raw + ((1024 - (smem_u32(dsm_raw) & 1023)) & 1023));
  float2 *Hs = Es + 4096;
  float2 *buf = Hs + 4096;
  __shared__ Plane128Shared S;
  __shared__ __align__(8) uint64_t s_bar;
  const int nz = T.nz;
  const Quad Z = quad_roles();
  const int q = Z.q, rx = Z.rx, ry = Z.ry;
  const int task = blockIdx.x >> 2;
  const int ii = task / nz;
  const int zz = task - ii * nz;
  const MixInst &P = T.inst[ii];
  const int N = P.N, Na = P.Na;
  if (n >= N) return;  // the whole cluster (same instance)
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const long long M = 16384LL * nz;
  const long long qoff = (long long)zz * 16384 + (64 * ry) * 128 + 64 * rx;  // quadrant origin
  const int row = Z.row, tr = Z.tr, col = Z.col, tc = Z.tc;
  if (tid == 0) mbar_init(&s_bar, 1);
  if (tid < 64) {
    S.tw[tid] = tw64_g[tid];
    S.w128[tid] = tw128_g[tid];
  }
  float2 v[8];
  float2 *work = P.work + qoff;
  if (n > 0) {
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = work[(tc + 8 * a) * 128 + col];
  }
  const int m2 = N - 1 - n;
  const bool pair = (m2 < n);
  const uint64_t pol_first = l2_policy_first();
  __syncthreads();  // barrier initialised
  if (tid == 0) {
    mbar_expect_tx(&s_bar, pair ? 65536u : 32768u);
    const uint64_t pol_last = l2_policy_last();
    for (int b = 0; b < 4; b++) tma_load_2d(Es + b * 1024, &T.tmE[ii], 128 * rx + 32 * b, zz * 128 + 64 * ry, &s_bar,
                                            pol_last);
    if (pair)
      for (int b = 0; b < 4; b++)
        tma_load_2d(Hs + b * 1024, &T.tmH[ii], 128 * rx + 32 * b, (m2 * nz + zz) * 128 + 64 * ry, &s_bar, pol_first);
  }
  const int gi = row * 128 + tr;  // quadrant index of element d = 0 (row phase)
  float acc1[8], acc2[8];
  float *a1 = P.acc[n < Na ? 0 : 1] + qoff + gi;
  float *a2 = P.acc[m2 < Na ? 0 : 1] + qoff + gi;
  const bool same_acc = (a1 == a2);
  if (pair) {
#pragma unroll
    for (int d = 0; d < 8; d++) acc1[d] = a1[8 * d];
    if (!same_acc) {
#pragma unroll
      for (int d = 0; d < 8; d++) acc2[d] = a2[8 * d];
    }
  }
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
  if (n > 0) quad_inverse(v, buf, S, Z);
  // (the partners' reads of buf end before they arrive at the next barrier)
  if (!mbar_wait(&s_bar, 0, T.err[1])) {
    atomicExch(T.err, 1);
    mbar_wait(&s_bar, 0, kWaitPolls);  // let copies in flight land before the CTA moves on
  }
  if (n == 0) {
#pragma unroll
    for (int d = 0; d < 8; d++) {
      const float2 e = swz(Es, row, tr + 8 * d);
      v[d] = make_float2(useA_q ? e.x : e.y, useA_d ? e.x : e.y);
    }
  } else {
    const int eq = S.exp[0], ed = S.exp[1];
    const float sq = ldexpf(1.0f, -eq), sd = ldexpf(1.0f, -ed);
    const float mq_hi = S.mh[0], mq_lo = S.ml[0];
    const float md_hi = S.mh[1], md_lo = S.ml[1];
#pragma unroll
    for (int d = 0; d < 8; d++) {
      const float2 e = swz(Es, row, tr + 8 * d);
      const float eq_ = useA_q ? e.x : e.y, ed_ = useA_d ? e.x : e.y;
      const float uq = fmaf(v[d].x, eq_, fmaf(mq_hi, eq_, mq_lo * eq_));
      const float ud = fmaf(v[d].y, ed_, fmaf(md_hi, ed_, md_lo * ed_));
      v[d] = make_float2(uq * sq, ud * sd);
    }
  }
  const int Kq = (n == 0) ? 0 : P.K[n - 1] + S.exp[0];
  const int Kd = (n == 0) ? 0 : P.K[N + n - 1] + S.exp[1];
  if (zz == 0 && q == 0 && tid == 0) {
    P.K[n] = Kq;
    P.K[N + n] = Kd;
  }
  // density terms of a paired step into the accumulator registers (stored
  // after the cluster arrive below)
  const int n0 = N / 2;
  const int Kref = (m2 <= n) ? ((n == n0) ? Kq + (m2 == n ? Kd : P.K[N + m2]) : P.K[2 * N]) : 0;
  if (m2 <= n && n == n0 && zz == 0 && q == 0 && tid == 0) P.K[2 * N] = Kref;
  if (pair) {
    const float f1 = ldexpf(1.0f, Kq + P.K[N + m2] - Kref);
    const float f2 = ldexpf(1.0f, P.K[m2] + Kd - Kref);
    if (same_acc) {
#pragma unroll
      for (int d = 0; d < 8; d++) {
        const float2 h = swz(Hs, row, tr + 8 * d);
        acc1[d] = acc1[d] + fmaf(v[d].x * h.y, f1, (h.x * v[d].y) * f2);
      }
    } else {
#pragma unroll
      for (int d = 0; d < 8; d++) {
        const float2 h = swz(Hs, row, tr + 8 * d);
        acc1[d] = acc1[d] + (v[d].x * h.y) * f1;
        acc2[d] = acc2[d] + (h.x * v[d].y) * f2;
      }
    }
  }
  // quadrant sums: error-free FP32 two-sums within the thread and the warp
  float sq_ = 0.f, cq = 0.f, sd_ = 0.f, cd = 0.f;
#pragma unroll
  for (int d = 0; d < 8; d++) {
    float e;
    two_sum(sq_, v[d].x, sq_, e);
    cq += e;
    two_sum(sd_, v[d].y, sd_, e);
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
  __syncthreads();  // also: every read of the staged quadrants Es, Hs is done
  if (warp == 0) {
    double aq = lane < 16 ? S.red[0][lane] : 0.0;
    double ad = lane < 16 ? S.red[1][lane] : 0.0;
    for (int o = 8; o > 0; o >>= 1) {
      aq += __shfl_down_sync(0xffffffffu, aq, o);
      ad += __shfl_down_sync(0xffffffffu, ad, o);
    }
    if (lane == 0) {
      S.qs[0] = aq;
      S.qs[1] = ad;
    }
  }
  const bool last = (n == N - 1);
  // forward x (decimation in frequency): the x partner's real-space values
  // through Es (its staged factors are consumed)
  if (!last) quad_forward_publish(v, Es, Z);
  cl_arrive();  // quadrant sums and the exchange values released to the cluster
  // this step's global writes, issued after the arrive so that its release
  // does not wait for them (the new accumulator values were formed above,
  // while the staged partner plane Hs was still this CTA's)
  if (n <= P.hmax) {
    float2 *hst = P.hist + (long long)n * M + qoff + gi;
#pragma unroll
    for (int d = 0; d < 8; d++) st_stream(hst + 8 * d, v[d], pol_first);
  }
  if (pair) {
#pragma unroll
    for (int d = 0; d < 8; d++) a1[8 * d] = acc1[d];
    if (!same_acc) {
#pragma unroll
      for (int d = 0; d < 8; d++) a2[8 * d] = acc2[d];
    }
  } else if (m2 == n) {
    const float f = ldexpf(1.0f, Kq + Kd - Kref);
#pragma unroll
    for (int d = 0; d < 8; d++) a1[8 * d] += (v[d].x * v[d].y) * f;
  }
  cl_wait();
  if (q == 0 && tid == 0) {
    // plane sums over the four quadrants, in rank order
    double sqv = 0.0, sdv = 0.0;
    for (int r = 0; r < 4; r++) {
      sqv += ld_cl_d(cl_map(&S.qs[0], (uint32_t)r));
      sdv += ld_cl_d(cl_map(&S.qs[1], (uint32_t)r));
    }
    P.part[(long long)n * nz + zz] = sqv;
    P.part[(long long)(N + n) * nz + zz] = sdv;
  }
  if (last) {
    cl_sync();  // CTA 0 has read every quadrant sum
    return;
  }
  quad_forward(v, Es, Hs, buf, S, Z);
#pragma unroll
  for (int d = 0; d < 8; d++) work[(tc + 8 * d) * 128 + col] = v[d];
  cl_wait();  // no CTA leaves while a partner may still read its buffers
}

// Graft sweep plane pass of step n for 128 x 128 xy planes (sweep 0: q_g from
// the free end, stored; sweep 1: qdag_g from the grafting surface, paired
// with the stored steps into the graft density), the contract of
// k_mix_graft_plane (kernels_mixed.cu) with the k-space layout of
// k_mix_plane128.  The field is real: it rides in the real part of the
// complex transform.  Cluster b works on plane b % nz of T.inst[b / nz].
// Dynamic shared memory: two 32 KB exchange quadrants and the padded
// exchange/transpose quadrant, as k_mix_plane128.
template <int CAP>
__global__ void __cluster_dims__(4, 1, 1) __launch_bounds__(512, 2)
    k_mix_graft_plane128(const __grid_constant__ Graft128TableT<CAP> T, const float2 *__restrict__ tw64_g,
                         const float2 *__restrict__ tw128_g, int sweep, int n) {
  extern __shared__ __align__(16) unsigned char dsm_raw[];
  float2 *Xs = reinterpret_cast<float2 *>(dsm_raw + ((1024 - (smem_u32(dsm_raw) & 1023)) & 1023));
  float2 *Ys = Xs + 4096;
  float2 *buf = Ys + 4096;
  __shared__ Plane128Shared S;
  const int nz = T.nz;
  const Quad Z = quad_roles();
  const int task = blockIdx.x >> 2;
  const int ii = task / nz;
  const int zz = task - ii * nz;
  const GraftMixInst &P = T.inst[ii];
  const int Ng = P.Ng;
  if (n >= Ng) return;  // the whole cluster (same instance)
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const long long M = 16384LL * nz;
  const long long qoff = (long long)zz * 16384 + (64 * Z.ry) * 128 + 64 * Z.rx;  // quadrant origin
  const int gi = Z.row * 128 + Z.tr;  // quadrant index of element d = 0 (row phase)
  if (tid < 64) {
    S.tw[tid] = tw64_g[tid];
    S.w128[tid] = tw128_g[tid];
  }
  double *part = P.part + (long long)sweep * Ng * nz;
  int *K = P.K + sweep * Ng;
  float2 v[8];
  float2 *work = P.work + qoff;
  if (n > 0) {
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = work[(Z.tc + 8 * a) * 128 + Z.col];
  }
  float eg[8];
  const float *Eg = P.Eg + qoff + gi;
#pragma unroll
  for (int d = 0; d < 8; d++) eg[d] = Eg[8 * d];
  if (warp == 0) {
    double a = 0.0;
    if (n > 0)
      for (int z = lane; z < nz; z += 32) a += part[(long long)(n - 1) * nz + z];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) {
      const double ma = a / (double)M;
      int ea = 0;
      if (n > 0 && isfinite(ma) && ma > 0.0) frexp(ma, &ea);
      S.exp[0] = ea;
      const float hi = (float)ma;
      S.mh[0] = hi;
      S.ml[0] = (float)(ma - (double)hi);
    }
  }
  __syncthreads();  // mean, exponent, twiddles
  if (n > 0) quad_inverse(v, buf, S, Z);
  const int ex = S.exp[0];
  const int Kn = (n > 0) ? K[n - 1] + ex : (sweep == 0 ? 0 : -P.K[Ng - 1]);
  if (n == 0) {
    if (sweep == 0) {
#pragma unroll
      for (int d = 0; d < 8; d++) v[d] = make_float2(eg[d], 0.f);
    } else {
      const float *last = P.hist + (long long)(Ng - 1) * M + qoff + gi;
      const double2 *gr = P.grafts + qoff + gi;
#pragma unroll
      for (int d = 0; d < 8; d++) v[d] = make_float2((float)gr[8 * d].x * eg[d] / last[8 * d], 0.f);
    }
  } else {
    const float sc = ldexpf(1.0f, -ex);
    const float m_hi = S.mh[0], m_lo = S.ml[0];
#pragma unroll
    for (int d = 0; d < 8; d++) v[d] = make_float2(fmaf(v[d].x, eg[d], fmaf(m_hi, eg[d], m_lo * eg[d])) * sc, 0.f);
  }
  if (zz == 0 && Z.q == 0 && tid == 0) K[n] = Kn;
  // quadrant sum: error-free FP32 two-sums within the thread and the warp
  float sa = 0.f, ca = 0.f;
#pragma unroll
  for (int d = 0; d < 8; d++) {
    float e;
    two_sum(sa, v[d].x, sa, e);
    ca += e;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_down_sync(0xffffffffu, sa, o), c2 = __shfl_down_sync(0xffffffffu, ca, o);
    float e;
    two_sum(sa, s2, sa, e);
    ca += c2 + e;
  }
  if (lane == 0) S.red[0][warp] = (double)sa + (double)ca;
  __syncthreads();
  if (warp == 0) {
    double aq = lane < 16 ? S.red[0][lane] : 0.0;
    for (int o = 8; o > 0; o >>= 1) aq += __shfl_down_sync(0xffffffffu, aq, o);
    if (lane == 0) S.qs[0] = aq;
  }
  const bool last = (n == Ng - 1);
  if (!last) quad_forward_publish(v, Xs, Z);
  cl_arrive();  // quadrant sums and the exchange values released to the cluster
  // this step's global writes after the arrive (its release does not wait for them)
  if (sweep == 0) {
    float *h = P.hist + (long long)n * M + qoff + gi;
#pragma unroll
    for (int d = 0; d < 8; d++) h[8 * d] = v[d].x;
  } else {
    const float *o = P.hist + (long long)(Ng - 1 - n) * M + qoff + gi;
    const float f = ldexpf(1.0f, Kn + P.K[Ng - 1 - n]);
    float *acc = P.acc + qoff + gi;
#pragma unroll
    for (int d = 0; d < 8; d++) acc[8 * d] += (v[d].x * o[8 * d]) * f;
  }
  cl_wait();
  if (Z.q == 0 && tid == 0) {
    double sv = 0.0;
    for (int r = 0; r < 4; r++) sv += ld_cl_d(cl_map(&S.qs[0], (uint32_t)r));
    part[(long long)n * nz + zz] = sv;
  }
  if (last) {
    cl_sync();  // CTA 0 has read every quadrant sum
    return;
  }
  quad_forward(v, Xs, Ys, buf, S, Z);
#pragma unroll
  for (int d = 0; d < 8; d++) work[(Z.tc + 8 * d) * 128 + Z.col] = v[d];
  cl_wait();  // no CTA leaves while a partner may still read its buffers
}

template <int CAP>
static cudaError_t launch_graft128_chunks(const GraftMixInst *insts, int ninst, int nz, const void *tw64,
                                          const void *tw128, int sweep, int n, cudaStream_t st) {
  const int smem = 1024 + 2 * 4096 * (int)sizeof(float2) + kPlanePad * (int)sizeof(float2);
  auto kfn = k_mix_graft_plane128<CAP>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  for (int i0 = 0; i0 < ninst; i0 += CAP) {
    const int cnt = ninst - i0 < CAP ? ninst - i0 : CAP;
    Graft128TableT<CAP> T;
    memset(&T, 0, sizeof T);
    for (int k = 0; k < cnt; k++) T.inst[k] = insts[i0 + k];
    T.nz = nz;
    kfn<<<4 * nz * cnt, 512, smem, st>>>(T, reinterpret_cast<const float2 *>(tw64),
                                          reinterpret_cast<const float2 *>(tw128), sweep, n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_mix_graft_plane128(const GraftMixInst *insts, int ninst, int nz, const void *tw64,
                                      const void *tw128, int sweep, int n, cudaStream_t st) {
  if (ninst <= 0) return cudaSuccess;
  if (ninst <= 4) return launch_graft128_chunks<4>(insts, ninst, nz, tw64, tw128, sweep, n, st);
  return launch_graft128_chunks<16>(insts, ninst, nz, tw64, tw128, sweep, n, st);
}

// One plane-pass launch per chunk of at most CAP instances (4 CTAs per plane).
template <int CAP>
static cudaError_t launch_plane128_chunks(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH,
                                          int ninst, int nz, const void *tw64, const void *tw128, int n, int *err,
                                          cudaStream_t st) {
  const int smem = 1024 + 2 * 4096 * (int)sizeof(float2) + kPlanePad * (int)sizeof(float2);
  auto kfn = k_mix_plane128<CAP>;
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
    kfn<<<4 * nz * cnt, 512, smem, st>>>(T, reinterpret_cast<const float2 *>(tw64),
                                          reinterpret_cast<const float2 *>(tw128), n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_mix_plane128(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                                int nz, const void *tw64, const void *tw128, int n, int *err, cudaStream_t st) {
  if (ninst <= 0) return cudaSuccess;
  if (ninst <= 4) return launch_plane128_chunks<4>(insts, tmE, tmH, ninst, nz, tw64, tw128, n, err, st);
  return launch_plane128_chunks<16>(insts, tmE, tmH, ninst, nz, tw64, tw128, n, err, st);
}

}  // namespace scft
