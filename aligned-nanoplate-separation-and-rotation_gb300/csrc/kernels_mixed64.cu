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
// index needs a runtime division.  Exchanges between the 8 threads of one row
// stay inside a warp (warp barrier); exchanges along y cross warps (block
// barrier).
//
// The plane pass stages the Boltzmann factors and the stored history plane it
// needs after the inverse transforms with TMA tensor loads issued at kernel
// start (cp.async.bulk.tensor, completion on an mbarrier), so that their
// memory latency overlaps the transform work.  Each 64 x 64 float2 plane
// arrives as four 64-row x 128-byte boxes with the 128-byte swizzle (16-byte
// chunk c of row r stored at chunk c ^ (r & 7)), which keeps the row-phase
// reads free of bank conflicts without padding.  The mbarrier wait is
// bounded; a wait that runs out sets the context's error word.
// Plane sums are formed with error-free FP32 two-sums per thread and across
// the warp (FP64 only for the 16 warp results): GB300 issues FP64 at a small
// fraction of its FP32 rate.
#include "inst.h"
#include "launch.h"
#include "mix_core.cuh"
#include "prop_launch.h"

#include <string.h>

namespace scft {


// Static shared scratch of one plane task.
struct Plane64Shared {
  float2 tw[64];      // 64-point twiddles
  double red[2][16];  // per-warp plane sums
  float mh[2], ml[2]; // step means as two-float pairs
  int exp[2];         // power-of-two exponents of the step
};

// Thread 0 of the CTA: TMA loads of the Boltzmann plane zz of instance ii
// and, on a paired step n (partner step m2 = N - 1 - n < n), of the stored
// history plane m2, into Es / Hs, completing on `bar` (E rows z*64 + y of a
// 64 nz-row tensor; history rows (m2*nz + z)*64 + y).
template <class TT>
__device__ __forceinline__ void plane64_stage(const TT &T, int ii, int zz, int nz, int n, float2 *Es,
                                              float2 *Hs, uint64_t *bar) {
  const MixInst &P = T.inst[ii];
  const int m2 = P.N - 1 - n;
  const bool pair = (m2 < n);
  mbar_expect_tx(bar, pair ? 65536u : 32768u);
  const uint64_t pol_last = l2_policy_last(), pol_first = l2_policy_first();
  for (int b = 0; b < 4; b++) tma_load_2d(Es + b * 1024, &T.tmE[ii], 32 * b, zz * 64, bar, pol_last);
  if (pair)
    for (int b = 0; b < 4; b++) tma_load_2d(Hs + b * 1024, &T.tmH[ii], 32 * b, (m2 * nz + zz) * 64, bar, pol_first);
}

// One plane task: plane zz of instance ii at step n (n < N), 512 threads.
// On entry S.tw holds the twiddles and plane64_stage has been issued on
// `bar`, whose phase `parity` completes when the staged planes have landed;
// both are ordered before the first wait by the body's first block barrier.
// The CTA's shared planes Es, Hs (TMA, 128-byte swizzle) and buf (padded
// exchange plane) are free again once the body returns and the caller has
// passed a block barrier.
// STAGE: thread 0 issues plane64_stage itself, right after its working-plane
// loads (the one-launch-per-step kernel); otherwise the caller has issued it.
template <int NZ, bool STAGE, class TT>
__device__ __forceinline__ void plane64_body(const TT &T, int ii, int zz, int n, float2 *Es, float2 *Hs,
                                             float2 *buf, Plane64Shared &S, uint64_t *bar, uint32_t parity) {
  const int nz = NZ ? NZ : T.nz;
  const MixInst &P = T.inst[ii];
  const int N = P.N, Na = P.Na;
  const long long M = 4096LL * nz;
  const long long zoff = (long long)zz * 4096;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  // row-phase ownership: (y = row, x = tr + 8d); column phase: (y = tc + 8d, x = col)
  const int row = tid >> 3, tr = tid & 7;
  const int col = tid & 63, tc = tid >> 6;
  float2 v[8];
  float2 *work = P.work + zoff;
  if (n > 0) {
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = work[(tc + 8 * a) * 64 + col];
  }
  const int m2 = N - 1 - n;
  const bool pair = (m2 < n);  // a stored partner plane is needed
  const uint64_t pol_first = l2_policy_first();
  if (STAGE && tid == 0) plane64_stage(T, ii, zz, nz, n, Es, Hs, bar);
  // accumulators of a paired step, loaded now so that their latency overlaps
  // the inverse transforms (row-phase ownership, as they are used)
  const int gi = row * 64 + tr;  // global index of element d = 0 in this plane
  float acc1[8], acc2[8];
  float *a1 = P.acc[n < Na ? 0 : 1] + zoff + gi;
  float *a2 = P.acc[m2 < Na ? 0 : 1] + zoff + gi;
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
    // warp 0: mean of q_{n-1}; warp 1: mean of qdag_{n-1} (64 FP64 plane sums each)
    double a = 0.0;
    if (n > 0) {
      const double *pp = P.part + (long long)(warp * N + n - 1) * nz;
      for (int z = lane; z < nz; z += 32) a += pp[z];
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) {
      const double ma = NZ ? a * (1.0 / (double)M) : a / (double)M;  // 2^18 when NZ = 64: exact
      int ea = 0;
      if (n > 0 && isfinite(ma) && ma > 0.0) frexp(ma, &ea);
      S.exp[warp] = ea;
      // split once here: GB300 runs FP64 (conversions included) at a small
      // fraction of the FP32 rate, so no thread of the plane does it
      const float hi = (float)ma;
      S.mh[warp] = hi;
      S.ml[warp] = (float)(ma - (double)hi);
    }
  }
  const bool useA_q = (Na > 0 && n < Na);
  const bool useA_d = !(n <= N - Na - 1);
  __syncthreads();  // means, exponents (and, on entry, the twiddles and the barrier's initialisation)
  if (n > 0) {
    // inverse y transform (column phase)
    fft64_colhalf<+1, 1>(v, tc, buf + col, S.tw);
#pragma unroll
    for (int d = 0; d < 8; d++) buf[(tc + 8 * d) * kRowPad + col] = v[d];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = buf[row * kRowPad + tr + 8 * a];
    // a row's exchange area (row * kRowPad + 9b + c < (row + 1) * kRowPad)
    // lies inside the padded row, and a warp owns whole rows: a warp
    // barrier suffices before the exchange overwrites what was just read
    __syncwarp();
    // inverse x transform (row phase, inside one warp)
    fft64_group<+1, true>(v, tr, buf + row * kRowPad, 9, 1, S.tw);
  }
  // every thread waits on the mbarrier itself (acquiring the staged planes),
  // and the shared plane is touched only in the thread's own rows until the
  // barrier of the plane sums: no block barrier here
  if (!mbar_wait(bar, parity, T.err[1])) {
    atomicExch(T.err, 1);
    mbar_wait(bar, parity, kWaitPolls);  // let copies in flight land before the CTA moves on
  }

  if (n == 0) {
#pragma unroll
    for (int d = 0; d < 8; d++) {
      const float2 e = swz(Es, row, tr + 8 * d);
      v[d] = make_float2(useA_q ? e.x : e.y, useA_d ? e.x : e.y);
    }
  } else {
    // q = (conv + mean) * e^{-w} * 2^{-e}, the mean as a two-float constant
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
  if (zz == 0 && tid == 0) {
    P.K[n] = Kq;
    P.K[N + n] = Kd;
  }
  // history, density terms, plane sums (row-phase ownership)
  if (n <= P.hmax) {
    float2 *hst = P.hist + (long long)n * M + zoff + gi;
#pragma unroll
    for (int d = 0; d < 8; d++) st_stream(hst + 8 * d, v[d], pol_first);
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
        for (int d = 0; d < 8; d++) {
          const float2 h = swz(Hs, row, tr + 8 * d);
          a1[8 * d] = acc1[d] + fmaf(v[d].x * h.y, f1, (h.x * v[d].y) * f2);
        }
      } else {
#pragma unroll
        for (int d = 0; d < 8; d++) {
          const float2 h = swz(Hs, row, tr + 8 * d);
          a1[8 * d] = acc1[d] + (v[d].x * h.y) * f1;
          a2[8 * d] = acc2[d] + (h.x * v[d].y) * f2;
        }
      }
    } else {
      const float f = ldexpf(1.0f, Kq + Kd - Kref);
#pragma unroll
      for (int d = 0; d < 8; d++) a1[8 * d] += (v[d].x * v[d].y) * f;
    }
  }
  // plane sums: error-free FP32 two-sums within the thread and the warp
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
  // warp 0 sums the 16 warp results after the next block barrier: the
  // forward transpose's, or on the last step a barrier of its own
  const bool last = (n == N - 1);
  if (!last) {
    // forward x transform (row phase; a warp's own rows of buf), then the
    // transpose to the column phase
    fft64_group<-1, true>(v, tr, buf + row * kRowPad, 9, 1, S.tw);
#pragma unroll
    for (int d = 0; d < 8; d++) buf[row * kRowPad + tr + 8 * d] = v[d];
  }
  __syncthreads();  // also: every read of Es, Hs and every write of S.red is done
  if (warp == 0) {
    double aq = lane < 16 ? S.red[0][lane] : 0.0;
    double ad = lane < 16 ? S.red[1][lane] : 0.0;
    for (int o = 8; o > 0; o >>= 1) {
      aq += __shfl_down_sync(0xffffffffu, aq, o);
      ad += __shfl_down_sync(0xffffffffu, ad, o);
    }
    if (lane == 0) {
      P.part[(long long)n * nz + zz] = aq;
      P.part[(long long)(N + n) * nz + zz] = ad;
    }
  }
  if (last) return;
#pragma unroll
  for (int a = 0; a < 8; a++) v[a] = buf[(tc + 8 * a) * kRowPad + col];
  // the one-launch-per-step kernel exchanges through the consumed Boltzmann
  // plane Es, so no barrier is needed between the transposed reads of buf
  // and the exchange; the persistent sweep keeps buf (Es is a bulk-copy
  // destination of its next task)
  if (!STAGE) __syncthreads();
  fft64_colhalf<-1, 0>(v, tc, (STAGE ? Es : buf) + col, S.tw);
#pragma unroll
  for (int d = 0; d < 8; d++) work[(tc + 8 * d) * 64 + col] = v[d];
}


// Plane pass of step n for 64 x 64 xy planes (any nz, the same for every
// instance of the launch), 512 threads, one CTA per (instance, z plane): CTA b
// works on plane b % nz of T.inst[b / nz].  The
// instance table is a kernel parameter, so the first global loads (the
// working plane, the prefetches) depend on nothing loaded before them.
// Dynamic shared memory (1024-byte aligned for the swizzle): staged Boltzmann
// plane and history plane (32 KB each), then the padded exchange/transpose
// plane (36.9 KB); 101 KB, two CTAs per SM.
// NZ: nz known at compile time (64), or 0 to read it from the table.
template <int NZ, int CAP>
__global__ void __launch_bounds__(512, 2) k_mix_plane64(const __grid_constant__ Mix64TableT<CAP> T,
                                                        const float2 *__restrict__ tw_g, int n) {
  extern __shared__ __align__(16) unsigned char dsm_raw[];
  float2 *Es = reinterpret_cast<float2 *>(dsm_raw + ((1024 - (smem_u32(dsm_raw) & 1023)) & 1023));
  float2 *Hs = Es + 4096;
  float2 *buf = Hs + 4096;
  __shared__ Plane64Shared S;
  __shared__ __align__(8) uint64_t s_bar;
  const int nz = NZ ? NZ : T.nz;
  const int ii = blockIdx.x / nz;
  const int zz = blockIdx.x - ii * nz;
  if (n >= T.inst[ii].N) return;
  if (threadIdx.x == 0) mbar_init(&s_bar, 1);
  if (threadIdx.x < 64) S.tw[threadIdx.x] = tw_g[threadIdx.x];
  plane64_body<NZ, true>(T, ii, zz, n, Es, Hs, buf, S, &s_bar, 0);
}

// z pass for nz = 64 (mode 3 of the generic column pass): tile of TX x columns
// at one y, 8 threads per column.  g(k) = gx gy gz factorises over the axes,
// so h = 1 - g(k) is formed on the fly from per-axis tables h_d = 1 - g_d
// (jb.kern = [hx | hy | hz], each -expm1(-k_d^2/6) rounded once) as
// 1 - (1 - a)(1 - b) = a + b - a b, applied twice: every term is positive, so
// h keeps its relative accuracy where it is small.  The pass moves only the
// propagator itself.
// One z-pass tile: TX columns x0 .. x0 + TX - 1 at row y of the array a, all
// 64 z, 8 * TX threads; tw (64 twiddles) and buf (64 * TX float2) in shared
// memory, the twiddles ready on entry (ordered by the block barrier after
// the loads).
template <int TX>
__device__ __forceinline__ void col64_body(float2 *a, const float *ht, int x0, int y, int nx, int ny,
                                           const float2 *tw, float2 *buf, float s_hi, float s_lo) {
  const int tid = threadIdx.x;
  const int col = tid % TX, t = tid / TX;
  const long long plane = (long long)nx * ny;
  const long long base = (long long)y * nx + x0 + col;
  const float hx = ht[x0 + col], hy = ht[nx + y];
  const float hxy = fmaf(-hx, hy, hx + hy);
  float2 v[8];
#pragma unroll
  for (int j = 0; j < 8; j++) v[j] = a[(t + 8 * j) * plane + base];
  __syncthreads();  // tw
  fft64_group<-1, false>(v, t, buf + col, 8 * TX, TX, tw);
#pragma unroll
  for (int d = 0; d < 8; d++) {
    const int kz = t + 8 * d;
    const float hz = ht[nx + ny + kz];
    const float hv = fmaf(-hxy, hz, hxy + hz);
    float2 u = make_float2(fmaf(v[d].x, s_hi, v[d].x * s_lo), fmaf(v[d].y, s_hi, v[d].y * s_lo));
    u = make_float2(fmaf(-hv, u.x, u.x), fmaf(-hv, u.y, u.y));
    if (kz == 0 && y == 0 && x0 + col == 0) u = make_float2(0.f, 0.f);
    v[d] = u;
  }
  fft64_group<+1, false>(v, t, buf + col, 8 * TX, TX, tw);
#pragma unroll
  for (int j = 0; j < 8; j++) a[(t + 8 * j) * plane + base] = v[j];
}

template <int TX>
__global__ void __launch_bounds__(8 * TX) k_mix_col64(const ColJob *__restrict__ jobs,
                                                      const float2 *__restrict__ tw_g, int nx, int ny, float s_hi,
                                                      float s_lo) {
  __shared__ __align__(16) float2 buf[64 * TX];
  __shared__ float2 tw[64];
  const ColJob jb = jobs[blockIdx.x];
  if (threadIdx.x < 64) tw[threadIdx.x] = tw_g[threadIdx.x];
  col64_body<TX>(reinterpret_cast<float2 *>(jb.ptr), reinterpret_cast<const float *>(jb.kern), jb.x0, jb.y, nx, ny,
                 tw, buf, s_hi, s_lo);
}

// z pass for nz = 128, same contract as k_mix_col64: 8 threads per column,
// thread t holding the 16 values x[t + 8a].  128 = 8 x 16:
//   Y[t][c]  = sum_a x[t + 8a] w16^(a c)          (DFT16 in registers, 4 x 4)
//   Y[t][c] *= w128^(t c)
//   exchange through shared memory: thread t takes c = t and c = t + 8
//   X[c + 16 d] = sum_b Y[b][c] w8^(b d)          (two DFT8)
// which returns X[t + 8m] in v[m], the input order, so the same routine runs
// both directions.
template <int SIGN>
__device__ __forceinline__ void fft128_group(float2 *v, int t, float2 *xch, int sb, int sc, const float2 *tw) {
  dft16f<SIGN>(v, tw);
#pragma unroll
  for (int c = 1; c < 16; c++) v[c] = ctw<SIGN>(v[c], tw[t * c]);
#pragma unroll
  for (int c = 0; c < 16; c++) xch[t * sb + c * sc] = v[c];
  __syncthreads();
  float2 p[8], q[8];
#pragma unroll
  for (int b = 0; b < 8; b++) {
    p[b] = xch[b * sb + t * sc];
    q[b] = xch[b * sb + (t + 8) * sc];
  }
  __syncthreads();
  dft8f<SIGN>(p);
  dft8f<SIGN>(q);
#pragma unroll
  for (int d = 0; d < 8; d++) {
    v[2 * d] = p[d];
    v[2 * d + 1] = q[d];
  }
}

template <int TX>
__global__ void __launch_bounds__(8 * TX) k_mix_col128(const ColJob *__restrict__ jobs,
                                                       const float2 *__restrict__ tw_g, int nx, int ny, float s_hi,
                                                       float s_lo) {
  __shared__ __align__(16) float2 buf[128 * TX];
  __shared__ float2 tw[128];
  const ColJob jb = jobs[blockIdx.x];
  const int tid = threadIdx.x;
  const int col = tid % TX, t = tid / TX;
  for (int k = tid; k < 128; k += 8 * TX) tw[k] = tw_g[k];
  const long long plane = (long long)nx * ny;
  const long long base = (long long)jb.y * nx + jb.x0 + col;
  float2 *a = reinterpret_cast<float2 *>(jb.ptr);
  const float *ht = reinterpret_cast<const float *>(jb.kern);
  const float hx = ht[jb.x0 + col], hy = ht[nx + jb.y];
  const float hxy = fmaf(-hx, hy, hx + hy);
  float2 v[16];
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = a[(t + 8 * j) * plane + base];
  __syncthreads();  // tw
  fft128_group<-1>(v, t, buf + col, 16 * TX, TX, tw);
#pragma unroll
  for (int d = 0; d < 16; d++) {
    const int kz = t + 8 * d;
    const float hz = ht[nx + ny + kz];
    const float hv = fmaf(-hxy, hz, hxy + hz);
    float2 u = make_float2(fmaf(v[d].x, s_hi, v[d].x * s_lo), fmaf(v[d].y, s_hi, v[d].y * s_lo));
    u = make_float2(fmaf(-hv, u.x, u.x), fmaf(-hv, u.y, u.y));
    if (kz == 0 && jb.y == 0 && jb.x0 + col == 0) u = make_float2(0.f, 0.f);
    v[d] = u;
  }
  fft128_group<+1>(v, t, buf + col, 16 * TX, TX, tw);
#pragma unroll
  for (int j = 0; j < 16; j++) a[(t + 8 * j) * plane + base] = v[j];
}

// ---------------------------------------------------------------------------
// Plane pass, second form: warp-local column transforms
// ---------------------------------------------------------------------------
// The same step as plane64_body with fewer block barriers.  The working plane
// arrives by cp.async (16-byte chunks, coalesced) into an unpadded shared
// plane W laid out so that every access of the step is free of bank
// conflicts: element (y, x) at W[y*64 + 2 s_y(x/2) + x%2] with the 16-byte
// chunk permutation s_y(k) = (k & 24) | ((h(y%8) ^ y/8 ^ k ^ k/8) & 7),
// h = [0,4,1,5,2,6,3,7] (a CPU emulation of every access pattern: column
// reads and writes, the in-column exchange, row reads and writes are
// conflict-free; the in-row exchange read, whose 16 lanes share one x
// parity, is two-way).  The 8 threads of a column are 8 lanes of one warp
// (warp w owns columns 4w .. 4w+3; rows 4w .. 4w+3 in the row phase), so the
// column exchanges need only warp barriers; block barriers remain for the
// plane's arrival, the two transposes and the plane sums (4 against 8).
// The arithmetic and its order are those of plane64_body: results are
// bit-identical.
__device__ __forceinline__ int w_idx(int y, int x) {
  const int k = x >> 1, e = y & 7;
  const int hh = (e >> 1) | ((e & 1) << 2);
  return y * 64 + 2 * ((k & 24) | ((hh ^ (y >> 3) ^ k ^ (k >> 3)) & 7)) + (x & 1);
}

// 64-point transform of a column x held by 8 lanes (position t) of one warp:
// thread t holds x[t + 8a]; the exchange goes through the column's own slots
// of W (element (b, c) of the 8 x 8 exchange at row b + 8c).
template <int SIGN>
__device__ __forceinline__ void fft64_col_w(float2 *v, int x, int t, float2 *W, const float2 *tw) {
  dft8f<SIGN>(v);
  tw64<SIGN>(v, t, tw);
  __syncwarp();
#pragma unroll
  for (int c = 0; c < 8; c++) W[w_idx(t + 8 * c, x)] = v[c];
  __syncwarp();
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = W[w_idx(b + 8 * t, x)];
  __syncwarp();
  dft8f<SIGN>(v);
}

// The same for a row (element (b, c) at x = b + 8c of the row).
template <int SIGN>
__device__ __forceinline__ void fft64_row_w(float2 *v, int row, int t, float2 *W, const float2 *tw) {
  dft8f<SIGN>(v);
  tw64<SIGN>(v, t, tw);
  __syncwarp();
#pragma unroll
  for (int c = 0; c < 8; c++) W[w_idx(row, t + 8 * c)] = v[c];
  __syncwarp();
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = W[w_idx(row, b + 8 * t)];
  __syncwarp();
  dft8f<SIGN>(v);
}

template <int NZ, class TT>
__device__ __forceinline__ void plane64w_body(const TT &T, int ii, int zz, int n, float2 *Es, float2 *Hs,
                                              float2 *W, Plane64Shared &S, uint64_t *bar, uint32_t parity) {
  const int nz = NZ ? NZ : T.nz;
  const MixInst &P = T.inst[ii];
  const int N = P.N, Na = P.Na;
  const long long M = 4096LL * nz;
  const long long zoff = (long long)zz * 4096;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  // row phase: (y = row, x = tr + 8d); column phase: (y = ct + 8d, x = cx)
  const int row = tid >> 3, tr = tid & 7;
  const int cx = 4 * warp + (lane >> 3), ct = lane & 7;
  float2 v[8];
  float2 *work = P.work + zoff;
  if (n > 0) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int q = tid + 512 * j, y = q >> 5, k = q & 31;
      cp_async16(W + w_idx(y, 2 * k), work + y * 64 + 2 * k);
    }
    cp_async_commit();
  }
  const int m2 = N - 1 - n;
  const bool pair = (m2 < n);
  const uint64_t pol_first = l2_policy_first();
  if (tid == 0) plane64_stage(T, ii, zz, nz, n, Es, Hs, bar);
  const int gi = row * 64 + tr;
  float acc1[8], acc2[8];
  float *a1 = P.acc[n < Na ? 0 : 1] + zoff + gi;
  float *a2 = P.acc[m2 < Na ? 0 : 1] + zoff + gi;
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
    double a = 0.0;
    if (n > 0) {
      const double *pp = P.part + (long long)(warp * N + n - 1) * nz;
      for (int z = lane; z < nz; z += 32) a += pp[z];
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) {
      const double ma = NZ ? a * (1.0 / (double)M) : a / (double)M;
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
  if (n > 0) cp_async_wait_all();
  __syncthreads();  // W, means, exponents (and, on entry, the twiddles and the barrier's initialisation)
  if (n > 0) {
    // inverse y transform (warp-local column phase), back into the column's slots
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = W[w_idx(ct + 8 * a, cx)];
    fft64_col_w<+1>(v, cx, ct, W, S.tw);
#pragma unroll
    for (int d = 0; d < 8; d++) W[w_idx(ct + 8 * d, cx)] = v[d];
    __syncthreads();
    // inverse x transform (row phase; a warp owns its four rows)
#pragma unroll
    for (int d = 0; d < 8; d++) v[d] = W[w_idx(row, tr + 8 * d)];
    fft64_row_w<+1>(v, row, tr, W, S.tw);
  }
  if (!mbar_wait(bar, parity, T.err[1])) {
    atomicExch(T.err, 1);
    mbar_wait(bar, parity, kWaitPolls);
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
  if (zz == 0 && tid == 0) {
    P.K[n] = Kq;
    P.K[N + n] = Kd;
  }
  if (n <= P.hmax) {
    float2 *hst = P.hist + (long long)n * M + zoff + gi;
#pragma unroll
    for (int d = 0; d < 8; d++) st_stream(hst + 8 * d, v[d], pol_first);
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
        for (int d = 0; d < 8; d++) {
          const float2 h = swz(Hs, row, tr + 8 * d);
          a1[8 * d] = acc1[d] + fmaf(v[d].x * h.y, f1, (h.x * v[d].y) * f2);
        }
      } else {
#pragma unroll
        for (int d = 0; d < 8; d++) {
          const float2 h = swz(Hs, row, tr + 8 * d);
          a1[8 * d] = acc1[d] + (v[d].x * h.y) * f1;
          a2[8 * d] = acc2[d] + (h.x * v[d].y) * f2;
        }
      }
    } else {
      const float f = ldexpf(1.0f, Kq + Kd - Kref);
#pragma unroll
      for (int d = 0; d < 8; d++) a1[8 * d] += (v[d].x * v[d].y) * f;
    }
  }
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
  __syncthreads();
  if (warp == 0) {
    double aq = lane < 16 ? S.red[0][lane] : 0.0;
    double ad = lane < 16 ? S.red[1][lane] : 0.0;
    for (int o = 8; o > 0; o >>= 1) {
      aq += __shfl_down_sync(0xffffffffu, aq, o);
      ad += __shfl_down_sync(0xffffffffu, ad, o);
    }
    if (lane == 0) {
      P.part[(long long)n * nz + zz] = aq;
      P.part[(long long)(N + n) * nz + zz] = ad;
    }
  }
  if (n == N - 1) return;
  // forward x transform (row phase), back into the rows; then the columns
  fft64_row_w<-1>(v, row, tr, W, S.tw);
#pragma unroll
  for (int d = 0; d < 8; d++) W[w_idx(row, tr + 8 * d)] = v[d];
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 8; a++) v[a] = W[w_idx(ct + 8 * a, cx)];
  fft64_col_w<-1>(v, cx, ct, W, S.tw);
#pragma unroll
  for (int d = 0; d < 8; d++) work[(ct + 8 * d) * 64 + cx] = v[d];
}

template <int NZ, int CAP>
__global__ void __launch_bounds__(512, 2) k_mix_plane64w(const __grid_constant__ Mix64TableT<CAP> T,
                                                         const float2 *__restrict__ tw_g, int n) {
  extern __shared__ __align__(16) unsigned char dsm_raw[];
  float2 *Es = reinterpret_cast<float2 *>(dsm_raw + ((1024 - (smem_u32(dsm_raw) & 1023)) & 1023));
  float2 *Hs = Es + 4096;
  float2 *W = Hs + 4096;
  __shared__ Plane64Shared S;
  __shared__ __align__(8) uint64_t s_bar;
  const int nz = NZ ? NZ : T.nz;
  const int ii = blockIdx.x / nz;
  const int zz = blockIdx.x - ii * nz;
  if (n >= T.inst[ii].N) return;
  if (threadIdx.x == 0) mbar_init(&s_bar, 1);
  if (threadIdx.x < 64) S.tw[threadIdx.x] = tw_g[threadIdx.x];
  plane64w_body<NZ>(T, ii, zz, n, Es, Hs, W, S, &s_bar, 0);
}

// ---------------------------------------------------------------------------
// The whole sweep in one persistent launch
// ---------------------------------------------------------------------------
// k_mix_sweep64 runs every step of the propagator sweep of a batch of
// 64 x 64 x 64 instances (the recurrence of code/diblock_discrete.cpp:31-85,
// q and qdag at once) as one launch.  Its CTAs (as many as are resident at
// once, launched cooperatively so that all of them are) take tasks in a fixed
// order from an atomic counter:
//   step n = 0:      plane tasks P(0, i, z)            for every active i, z
//   step n >= 1:     z tasks P'(n, i, y), then P(n, i, z)
// where P(n, i, z) is the plane pass of plane z (plane64_body) and Z(n, i, y)
// the z pass of row y, all 64 columns (col64_body with 64 columns).  Active
// instances at step n are those with N > n, a prefix of the job order.
// Dependencies, per instance, carried by two counters of finished tasks:
//   Z(n, i, .) needs every P(n - 1, i, .)        (plane tasks done >= 64 n)
//   P(n, i, .) needs every Z(n, i, .)            (z tasks done >= 64 n)
//   and, on a paired step, the plane tasks of step m2 = N - 1 - n, which
//   wrote the stored partner plane             (plane tasks done >= 64 (m2 + 1))
// A task depends only on tasks earlier in the order, and every CTA is
// resident, so the task with the smallest unfinished index can always run:
// the sweep cannot deadlock.  A finished task is published by its thread 0
// after a block barrier with a release (fence + atomic add); a waiting task's
// thread 0 acquires the counter before the block barrier that lets its
// threads read.  A plane task stages its Boltzmann plane (constant during the
// sweep) and partner plane by TMA as soon as the partner's step is published,
// before it waits for the z pass of its own step, so the copies overlap that
// wait.  Every wait is bounded (err[2] polls, kSpinPolls by default): one
// that runs out sets the error word to 2 and raises the abort flag, which
// every other waiting CTA checks, so the launch always ends; the host reports
// SCFT_ERR_CUDA and the sweep's results are invalid.
namespace {

enum { kPlaneTask = 0, kZTask = 1 };

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Orders this thread's (acquired) view of global memory before its later
// bulk-copy (async proxy) reads.
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;\n" ::: "memory");
}

// Thread 0 of a CTA: waits until *cnt >= target.  False when the wait ran
// out (it then records the timeout) or another CTA has aborted the sweep.
// On success a GPU-scope fence follows the acquiring load (as after a grid
// barrier), so that the CTA's threads, ordered after thread 0 by a block
// barrier, read what the producing tasks wrote.
__device__ bool wait_count(const unsigned *cnt, unsigned target, unsigned *abort_flag, int *err) {
  const int polls = err[2];  // kSpinPolls unless lowered with scft_set_wait_limit
  for (int k = 0; k < polls; k++) {
    if (ld_acquire(cnt) >= target) {
      __threadfence();
      return true;
    }
    if ((k & 63) == 63 && ld_acquire(abort_flag)) return false;
    __nanosleep(64);
  }
  atomicExch(err, 2);
  atomicExch(abort_flag, 1u);
  return false;
}

// Task t of the order above -> (kind, step n, instance ii, plane or row).
__device__ __forceinline__ void sweep64_decode(const Sweep64Table &T, unsigned t, int &kind, int &n, int &ii,
                                               int &row) {
  unsigned base = 0;
  int s0 = 0;
  for (int a = T.ninst; a >= 1; a--) {
    const int s1 = T.m.inst[a - 1].N;  // steps s0 .. s1 - 1 have `a` active instances
    if (s1 <= s0) continue;
    const unsigned per = 128u * (unsigned)a;  // tasks of a step n >= 1
    const unsigned seg = (s0 == 0 ? 64u * a + per * (unsigned)(s1 - 1) : per * (unsigned)(s1 - s0));
    if (t < base + seg) {
      unsigned r = t - base;
      if (s0 == 0 && r < 64u * a) {
        kind = kPlaneTask;
        n = 0;
      } else {
        if (s0 == 0) {
          r -= 64u * a;
          n = 1 + (int)(r / per);
        } else {
          n = s0 + (int)(r / per);
        }
        r %= per;
        kind = r < 64u * a ? kZTask : kPlaneTask;
        if (kind == kPlaneTask) r -= 64u * a;
      }
      ii = (int)(r >> 6);
      row = (int)(r & 63);
      return;
    }
    base += seg;
    s0 = s1;
  }
  kind = -1;  // past the end (not reached: t < total)
  n = ii = row = 0;
}

}  // namespace

__global__ void __launch_bounds__(512, 2) k_mix_sweep64(const __grid_constant__ Sweep64Table T,
                                                        const float2 *__restrict__ tw_g) {
  extern __shared__ __align__(16) unsigned char dsm_raw[];
  // Es, Hs: staged planes; then buf: padded plane (plane tasks) or 64 x 64
  // z-pass tile (z tasks); formed where used, to keep registers free
#define SWEEP64_ES reinterpret_cast<float2 *>(dsm_raw + ((1024 - (smem_u32(dsm_raw) & 1023)) & 1023))
  __shared__ Plane64Shared S;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ unsigned s_task;
  __shared__ int s_go;
  if (threadIdx.x == 0) mbar_init(&s_bar, 1);
  if (threadIdx.x < 64) S.tw[threadIdx.x] = tw_g[threadIdx.x];
  __syncthreads();
  uint32_t parity = 0;
  for (;;) {
    if (threadIdx.x == 0) s_task = atomicAdd(T.ctr, 1u);
    __syncthreads();
    const unsigned t = s_task;
    if (t >= T.total) break;
    int kind, n, ii, row;
    sweep64_decode(T, t, kind, n, ii, row);
    if (kind < 0) break;  // not reached: every t < total decodes
    if (kind == kPlaneTask) {
      if (threadIdx.x == 0) {
        unsigned *abort_flag = T.ctr + 1, *done_p = T.ctr + 2, *done_z = T.ctr + 2 + T.ninst;
        float2 *Es = SWEEP64_ES;
        const MixInst &P = T.m.inst[ii];
        const int m2 = P.N - 1 - n;
        bool ok = true, issued = false;
        if (m2 < n) ok = wait_count(done_p + ii, 64u * (unsigned)(m2 + 1), abort_flag, T.m.err);
        if (ok) {
          fence_proxy_async_global();
          plane64_stage(T.m, ii, row, 64, n, Es, Es + 4096, &s_bar);
          issued = true;
        }
        if (ok && n > 0) ok = wait_count(done_z + ii, 64u * (unsigned)n, abort_flag, T.m.err);
        if (!ok && issued) mbar_wait(&s_bar, parity, kWaitPolls);  // the copies land before the CTA leaves
        s_go = ok;
      }
      __syncthreads();
      if (!s_go) break;
      {
        float2 *Es = SWEEP64_ES;
        plane64_body<64, false>(T.m, ii, row, n, Es, Es + 4096, Es + 8192, S, &s_bar, parity);
      }
      parity ^= 1u;
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(T.ctr + 2 + ii, 1u);
      }
    } else {
      if (threadIdx.x == 0) s_go = wait_count(T.ctr + 2 + ii, 64u * (unsigned)n, T.ctr + 1, T.m.err);
      __syncthreads();
      if (!s_go) break;
      col64_body<64>(T.m.inst[ii].work, T.ht[ii], 0, row, 64, 64, S.tw, SWEEP64_ES + 8192, T.s_hi, T.s_lo);
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(T.ctr + 2 + T.ninst + ii, 1u);
      }
    }
  }
#undef SWEEP64_ES
}

static int sweep64_smem() { return 1024 + 2 * 4096 * (int)sizeof(float2) + kPlanePad * (int)sizeof(float2); }

cudaError_t sweep64_capacity(int *ctas) {
  const int smem = sweep64_smem();
  cudaError_t e = cudaFuncSetAttribute(k_mix_sweep64, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_mix_sweep64, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mix_sweep64, 512, smem);
  if (e != cudaSuccess) return e;
  *ctas = per_sm * sms;
  return per_sm < 1 ? cudaErrorInvalidConfiguration : cudaSuccess;
}

cudaError_t launch_mix_sweep64(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH,
                               const float *const *ht, int ninst, const void *tw64, unsigned *ctr, int *err,
                               int max_ctas, cudaStream_t st) {
  if (ninst <= 0) return cudaSuccess;
  if (ninst > kMix64MaxInst) return cudaErrorInvalidValue;
  const int smem = sweep64_smem();
  static_assert(64 * 64 * (int)sizeof(float2) <= kPlanePad * (int)sizeof(float2), "z tile fits the plane buffer");
  int capacity = 0;
  cudaError_t e = sweep64_capacity(&capacity);
  if (e != cudaSuccess) return e;
  Sweep64Table T;
  memset(&T, 0, sizeof T);
  unsigned total = 0;
  for (int k = 0; k < ninst; k++) {
    if (insts[k].N < 1 || (k > 0 && insts[k].N > insts[k - 1].N)) return cudaErrorInvalidValue;  // job order
    T.m.inst[k] = insts[k];
    T.m.tmE[k] = tmE[k];
    T.m.tmH[k] = tmH[k];
    T.ht[k] = ht[k];
    total += 64u + 128u * (unsigned)(insts[k].N - 1);
  }
  T.m.err = err;
  T.m.nz = 64;
  T.ctr = ctr;
  T.ninst = ninst;
  T.total = total;
  const double sc = 1.0 / (64.0 * 64.0 * 64.0);
  T.s_hi = (float)sc;
  T.s_lo = (float)(sc - (double)T.s_hi);
  // at most 64 tasks of one instance are ready at a time
  int grid = capacity;
  const int useful = 128 * ninst;
  if (grid > useful) grid = useful;
  if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
  e = cudaMemsetAsync(ctr, 0, sizeof(unsigned) * (size_t)sweep64_counters(ninst), st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(512);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, k_mix_sweep64, T, reinterpret_cast<const float2 *>(tw64));
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}


// One plane-pass launch per chunk of at most CAP instances, the table by value.
template <int CAP, class K>
static cudaError_t launch_plane64_chunks(K kfn64, K kfn0, const MixInst *insts, const CUtensorMap *tmE,
                                         const CUtensorMap *tmH, int ninst, int nz, const void *tw64, int n, int *err,
                                         int smem, cudaStream_t st) {
  auto kfn = (nz == 64) ? kfn64 : kfn0;
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
    kfn<<<nz * cnt, 512, smem, st>>>(T, reinterpret_cast<const float2 *>(tw64), n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_mix_plane64w(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                                int nz, const void *tw64, int n, int *err, cudaStream_t st) {
  if (ninst <= 0) return cudaSuccess;
  const int smem = 1024 + 3 * 4096 * (int)sizeof(float2);
  if (ninst <= 4)
    return launch_plane64_chunks<4>(k_mix_plane64w<64, 4>, k_mix_plane64w<0, 4>, insts, tmE, tmH, ninst, nz, tw64, n,
                                    err, smem, st);
  if (ninst <= 16)
    return launch_plane64_chunks<16>(k_mix_plane64w<64, 16>, k_mix_plane64w<0, 16>, insts, tmE, tmH, ninst, nz, tw64,
                                     n, err, smem, st);
  return launch_plane64_chunks<kMix64MaxInst>(k_mix_plane64w<64, kMix64MaxInst>, k_mix_plane64w<0, kMix64MaxInst>,
                                              insts, tmE, tmH, ninst, nz, tw64, n, err, smem, st);
}

cudaError_t launch_mix_plane64(const MixInst *insts, const CUtensorMap *tmE, const CUtensorMap *tmH, int ninst,
                               int nz, const void *tw64, int n, int *err, cudaStream_t st) {
  if (ninst <= 0) return cudaSuccess;
  const int smem = 1024 + 2 * 4096 * (int)sizeof(float2) + kPlanePad * (int)sizeof(float2);
  if (ninst <= 4)
    return launch_plane64_chunks<4>(k_mix_plane64<64, 4>, k_mix_plane64<0, 4>, insts, tmE, tmH, ninst, nz, tw64, n,
                                    err, smem, st);
  if (ninst <= 16)
    return launch_plane64_chunks<16>(k_mix_plane64<64, 16>, k_mix_plane64<0, 16>, insts, tmE, tmH, ninst, nz, tw64, n,
                                     err, smem, st);
  return launch_plane64_chunks<kMix64MaxInst>(k_mix_plane64<64, kMix64MaxInst>, k_mix_plane64<0, kMix64MaxInst>,
                                              insts, tmE, tmH, ninst, nz, tw64, n, err, smem, st);
}

cudaError_t launch_mix_col64(const ColJob *jobs, int njobs, const void *tw, int nx, int ny, int nz, int tx,
                             cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  const double s = 1.0 / ((double)nx * ny * nz);
  const float s_hi = (float)s, s_lo = (float)(s - (double)s_hi);
  const float2 *t2 = reinterpret_cast<const float2 *>(tw);
  if (nz == 256) return launch_mix_col256(jobs, njobs, tw, nx, ny, tx, st);
  if (nz == 128) {
    switch (tx) {
      case 8: k_mix_col128<8><<<njobs, 64, 0, st>>>(jobs, t2, nx, ny, s_hi, s_lo); break;
      case 16: k_mix_col128<16><<<njobs, 128, 0, st>>>(jobs, t2, nx, ny, s_hi, s_lo); break;
      case 32: k_mix_col128<32><<<njobs, 256, 0, st>>>(jobs, t2, nx, ny, s_hi, s_lo); break;
      default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
  if (nz != 64) return cudaErrorInvalidValue;
  switch (tx) {
    case 8: k_mix_col64<8><<<njobs, 64, 0, st>>>(jobs, t2, nx, ny, s_hi, s_lo); break;
    case 16: k_mix_col64<16><<<njobs, 128, 0, st>>>(jobs, t2, nx, ny, s_hi, s_lo); break;
    case 32: k_mix_col64<32><<<njobs, 256, 0, st>>>(jobs, t2, nx, ny, s_hi, s_lo); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace scft
