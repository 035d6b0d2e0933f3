// kernels_mixed96.cu -- the mixed-form plane pass for 96 x 64 xy planes (the
// 96 x 64 x 64 instances of the mixed-size sweep), same arithmetic contract
// as kernels_mixed.cu and kernels_mixed64.cu.
//
// A cluster of three CTAs per plane, each holding a 32-column slab of all 64
// rows (2048 values: 256 threads x 8).  The 64-point y transforms are local
// (the 64-point machinery); the 96-point x transforms are a local 32-point
// transform (four threads per row) closed by one radix-3 step between the
// three CTAs, read through distributed shared memory:
//   inverse: C_q[n'] = IDFT32 over m of X[3m + q];
//            x[32 i + n'] = sum_q W96^-((32 i + n') q) C_q[n'] in CTA i;
//   forward: D_q[n'] = sum_i x[32 i + n'] W96^((32 i + n') q) in CTA q;
//            X[3m + q] = DFT32 over n' of D_q.
// So CTA i holds real-space columns [32 i, 32 i + 32) in natural order, and
// in k-space the wavenumbers kx = 3m + i, stored residue-major (kx at
// position (kx % 3) 32 + kx / 3), which is again the column range
// [32 i, 32 i + 32).  The z pass reads its x factor table in that order.
//
// Cluster barriers: every thread of the three CTAs runs the same sequence (it
// depends only on n and the instance's N); a CTA's buffers are read by its
// partners only between two barriers, and no CTA leaves while a partner may
// still read them.
#include "inst.h"
#include "launch.h"
#include "mix_core.cuh"
#include "prop_launch.h"

#include <string.h>

namespace scft {

namespace {

constexpr int kRP96 = 36;  // padded row stride (float2) of a 64 x 32 slab

// Element (row, x) of an unpadded 64 x 32 exchange slab with bits 2-3 of x
// flipped by row % 4: free of bank conflicts for a half-warp's four rows x
// four threads (row phase) and for 16 consecutive x of one row (column
// phase).
__device__ __forceinline__ int xl96(int row, int x) { return row * 32 + (x ^ ((row & 3) << 2)); }

}  // namespace

struct Plane96Shared {
  float2 tw64[64];     // 64-point twiddles
  float2 tw32[32];     // 32-point twiddles
  float2 w96[96];      // exp(-2 pi i t / 96): the radix-3 twiddles
  double red[2][8];    // per-warp sums of the slab
  double qs[2];        // slab sums, read by CTA 0 of the cluster
  float mh[2], ml[2];  // step means as two-float pairs
  int exp[2];          // power-of-two exponents of the step
};

// Plane pass of step n for 96 x 64 xy planes (nz the same for every instance
// of the launch): 256 threads per CTA, clusters of three CTAs, one cluster
// per (instance, z plane): cluster b works on plane b % nz of T.inst[b / nz].
// Dynamic shared memory (1024-byte aligned): the staged Boltzmann and history
// slabs (16 KB each, as two 64-row x 128-byte boxes with the 128-byte
// swizzle; reused as exchange buffers once consumed), then the padded
// exchange/transpose slab (18 KB): 51 KB, four CTAs per SM.
// T.tmE / T.tmH: E32 and hist32 as rows of 96 float2 (192 floats).
template <int CAP>
__global__ void __cluster_dims__(3, 1, 1) __launch_bounds__(256, 4)
    k_mix_plane96(const __grid_constant__ Mix64TableT<CAP> T, const float2 *__restrict__ tw64_g,
                  const float2 *__restrict__ tw32_g, const float2 *__restrict__ tw96_g, int n) {
  extern __shared__ __align__(16) unsigned char dsm_raw[];
  float2 *Es = reinterpret_cast<float2 *>(dsm_raw + ((1024 - (smem_u32(dsm_raw) & 1023)) & 1023));
  float2 *Hs = Es + 2048;
  float2 *buf = Hs + 2048;
  __shared__ Plane96Shared S;
  __shared__ __align__(8) uint64_t s_bar;
  const int nz = T.nz;
  const int q = (int)cl_rank();  // 0, 1, 2
  const int ra = q == 2 ? 0 : q + 1, rb = q == 0 ? 2 : q - 1;  // the two partners
  const int task = blockIdx.x / 3;
  const int ii = task / nz;
  const int zz = task - ii * nz;
  const MixInst &P = T.inst[ii];
  const int N = P.N, Na = P.Na;
  if (n >= N) return;  // the whole cluster (same instance)
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const long long M = 6144LL * nz;
  const long long soff = (long long)zz * 6144 + 32 * q;  // slab origin (row stride 96)
  // row phase: (y = row, x = tr + 4j); column phase: (y = tc + 8d, x = col)
  const int row = tid >> 2, tr = tid & 3;
  const int col = tid & 31, tc = tid >> 5;
  if (tid == 0) mbar_init(&s_bar, 1);
  if (tid < 64) S.tw64[tid] = tw64_g[tid];
  if (tid < 32) S.tw32[tid] = tw32_g[tid];
  if (tid < 96) S.w96[tid] = tw96_g[tid];
  float2 v[8];
  float2 *work = P.work + soff;
  if (n > 0) {
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = work[(tc + 8 * a) * 96 + col];
  }
  const int m2 = N - 1 - n;
  const bool pair = (m2 < n);
  const uint64_t pol_first = l2_policy_first();
  __syncthreads();  // barrier initialised
  if (tid == 0) {
    mbar_expect_tx(&s_bar, pair ? 32768u : 16384u);
    const uint64_t pol_last = l2_policy_last();
    for (int b = 0; b < 2; b++) tma_load_2d(Es + b * 1024, &T.tmE[ii], 64 * q + 32 * b, zz * 64, &s_bar, pol_last);
    if (pair)
      for (int b = 0; b < 2; b++)
        tma_load_2d(Hs + b * 1024, &T.tmH[ii], 64 * q + 32 * b, (m2 * nz + zz) * 64, &s_bar, pol_first);
  }
  const int gi = row * 96 + tr;  // slab index of element j = 0 (row phase)
  float acc1[8], acc2[8];
  float *a1 = P.acc[n < Na ? 0 : 1] + soff + gi;
  float *a2 = P.acc[m2 < Na ? 0 : 1] + soff + gi;
  const bool same_acc = (a1 == a2);
  if (pair) {
#pragma unroll
    for (int j = 0; j < 8; j++) acc1[j] = a1[4 * j];
    if (!same_acc) {
#pragma unroll
      for (int j = 0; j < 8; j++) acc2[j] = a2[4 * j];
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
  if (n > 0) {
    // inverse y (local), transpose, inverse 32-point x over this CTA's m
    fft64_group<+1, false>(v, tc, buf + col, 8 * 32, 32, S.tw64);
#pragma unroll
    for (int d = 0; d < 8; d++) buf[(tc + 8 * d) * kRP96 + col] = v[d];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = buf[row * kRP96 + tr + 4 * a];
    // a row's exchange area lies inside its padded row, and a warp owns
    // whole rows: a warp barrier suffices
    __syncwarp();
    fft32_group<+1, true>(v, tr, buf + row * kRP96, 9, 1, S.tw32);
#pragma unroll
    for (int j = 0; j < 8; j++) buf[row * kRP96 + tr + 4 * j] = v[j];
    cl_sync();
    // radix-3 step: x[32 q + n'] = sum_r W96^-((32 q + n') r) C_r[n']
    {
      const uint32_t pa = cl_map(buf + row * kRP96 + tr, (uint32_t)ra);
      const uint32_t pb = cl_map(buf + row * kRP96 + tr, (uint32_t)rb);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int nn = 32 * q + tr + 4 * j;
        const float2 ca = ld_cl(pa + 8u * (uint32_t)(4 * j));
        const float2 cb = ld_cl(pb + 8u * (uint32_t)(4 * j));
        const float2 own = ctw<+1>(v[j], S.w96[(nn * q) % 96]);
        const float2 ta = ctw<+1>(ca, S.w96[(nn * ra) % 96]);
        const float2 tb = ctw<+1>(cb, S.w96[(nn * rb) % 96]);
        v[j] = cadd(own, cadd(ta, tb));
      }
    }
    // no barrier here: buf is next rewritten by the forward transform, after
    // the cluster barrier that follows the slab sums, before which every
    // partner has finished these reads
  }
  if (!mbar_wait(&s_bar, 0, T.err[1])) {
    atomicExch(T.err, 1);
    mbar_wait(&s_bar, 0, kWaitPolls);  // let copies in flight land before the CTA moves on
  }
  if (n == 0) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const float2 e = swz(Es, row, tr + 4 * j);
      v[j] = make_float2(useA_q ? e.x : e.y, useA_d ? e.x : e.y);
    }
  } else {
    const int eq = S.exp[0], ed = S.exp[1];
    const float sq = ldexpf(1.0f, -eq), sd = ldexpf(1.0f, -ed);
    const float mq_hi = S.mh[0], mq_lo = S.ml[0];
    const float md_hi = S.mh[1], md_lo = S.ml[1];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const float2 e = swz(Es, row, tr + 4 * j);
      const float eq_ = useA_q ? e.x : e.y, ed_ = useA_d ? e.x : e.y;
      const float uq = fmaf(v[j].x, eq_, fmaf(mq_hi, eq_, mq_lo * eq_));
      const float ud = fmaf(v[j].y, ed_, fmaf(md_hi, ed_, md_lo * ed_));
      v[j] = make_float2(uq * sq, ud * sd);
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
      for (int j = 0; j < 8; j++) {
        const float2 h = swz(Hs, row, tr + 4 * j);
        acc1[j] = acc1[j] + fmaf(v[j].x * h.y, f1, (h.x * v[j].y) * f2);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const float2 h = swz(Hs, row, tr + 4 * j);
        acc1[j] = acc1[j] + (v[j].x * h.y) * f1;
        acc2[j] = acc2[j] + (h.x * v[j].y) * f2;
      }
    }
  }
  // slab sums: error-free FP32 two-sums within the thread and the warp
  float sq_ = 0.f, cq = 0.f, sd_ = 0.f, cd = 0.f;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    float e;
    two_sum(sq_, v[j].x, sq_, e);
    cq += e;
    two_sum(sd_, v[j].y, sd_, e);
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
  __syncthreads();  // also: every read of the staged slabs Es, Hs is done
  if (warp == 0) {
    double aq = lane < 8 ? S.red[0][lane] : 0.0;
    double ad = lane < 8 ? S.red[1][lane] : 0.0;
    for (int o = 4; o > 0; o >>= 1) {
      aq += __shfl_down_sync(0xffffffffu, aq, o);
      ad += __shfl_down_sync(0xffffffffu, ad, o);
    }
    if (lane == 0) {
      S.qs[0] = aq;
      S.qs[1] = ad;
    }
  }
  const bool last = (n == N - 1);
  // forward x, radix-3 step first: the real-space slab through Es
  if (!last) {
#pragma unroll
    for (int j = 0; j < 8; j++) Es[xl96(row, tr + 4 * j)] = v[j];
  }
  cl_arrive();  // slab sums and the exchange values released to the cluster
  // this step's global writes, issued after the arrive so that its release
  // does not wait for them
  if (n <= P.hmax) {
    float2 *hst = P.hist + (long long)n * M + soff + gi;
#pragma unroll
    for (int j = 0; j < 8; j++) st_stream(hst + 4 * j, v[j], pol_first);
  }
  if (pair) {
#pragma unroll
    for (int j = 0; j < 8; j++) a1[4 * j] = acc1[j];
    if (!same_acc) {
#pragma unroll
      for (int j = 0; j < 8; j++) a2[4 * j] = acc2[j];
    }
  } else if (m2 == n) {
    const float f = ldexpf(1.0f, Kq + Kd - Kref);
#pragma unroll
    for (int j = 0; j < 8; j++) a1[4 * j] += (v[j].x * v[j].y) * f;
  }
  cl_wait();
  if (q == 0 && tid == 0) {
    // plane sums over the three slabs, in rank order
    double sqv = 0.0, sdv = 0.0;
    for (int r = 0; r < 3; r++) {
      sqv += ld_cl_d(cl_map(&S.qs[0], (uint32_t)r));
      sdv += ld_cl_d(cl_map(&S.qs[1], (uint32_t)r));
    }
    P.part[(long long)n * nz + zz] = sqv;
    P.part[(long long)(N + n) * nz + zz] = sdv;
  }
  if (last) {
    cl_sync();  // CTA 0 has read every slab sum
    return;
  }
  {
    // D_q[n'] = sum_i x[32 i + n'] W96^((32 i + n') q)
    const uint32_t pa = cl_map(Es, (uint32_t)ra), pb = cl_map(Es, (uint32_t)rb);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int np = tr + 4 * j;
      const uint32_t o = 8u * (uint32_t)xl96(row, np);
      const float2 xa = ld_cl(pa + o), xb = ld_cl(pb + o);
      const float2 own = ctw<-1>(v[j], S.w96[((32 * q + np) * q) % 96]);
      const float2 ta = ctw<-1>(xa, S.w96[((32 * ra + np) * q) % 96]);
      const float2 tb = ctw<-1>(xb, S.w96[((32 * rb + np) * q) % 96]);
      v[j] = cadd(own, cadd(ta, tb));
    }
  }
  cl_arrive();  // done reading the partners' buffers
  fft32_group<-1, true>(v, tr, buf + row * kRP96, 9, 1, S.tw32);
  // to the column phase through Hs (its staged plane is consumed), forward y
#pragma unroll
  for (int j = 0; j < 8; j++) Hs[xl96(row, tr + 4 * j)] = v[j];
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 8; a++) v[a] = Hs[xl96(tc + 8 * a, col)];
  fft64_group<-1, false>(v, tc, buf + col, 8 * 32, 32, S.tw64);
#pragma unroll
  for (int d = 0; d < 8; d++) work[(tc + 8 * d) * 96 + col] = v[d];
  cl_wait();  // no CTA leaves while a partner may still read its buffers
}

template <int CAP>
static cudaError_t launch_plane96_chunks(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH,
                                         int ninst, int nz, const void *tw64, const void *tw32, const void *tw96,
                                         int n, int *err, cudaStream_t st) {
  const int smem = 1024 + 2 * 2048 * (int)sizeof(float2) + 64 * kRP96 * (int)sizeof(float2);
  auto kfn = k_mix_plane96<CAP>;
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
    kfn<<<3 * nz * cnt, 256, smem, st>>>(T, reinterpret_cast<const float2 *>(tw64),
                                          reinterpret_cast<const float2 *>(tw32),
                                          reinterpret_cast<const float2 *>(tw96), n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_mix_plane96(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                               int nz, const void *tw64, const void *tw32, const void *tw96, int n, int *err,
                               cudaStream_t st) {
  if (ninst <= 0) return cudaSuccess;
  if (ninst <= 4) return launch_plane96_chunks<4>(insts, tmE, tmH, ninst, nz, tw64, tw32, tw96, n, err, st);
  return launch_plane96_chunks<16>(insts, tmE, tmH, ninst, nz, tw64, tw32, tw96, n, err, st);
}

}  // namespace scft
