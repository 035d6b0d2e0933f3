// mix_core.cuh -- building blocks of the specialised mixed-form propagator
// kernels (kernels_mixed64.cu, kernels_mixed128.cu): the 64-point transform of
// a group of 8 threads, the 16-point transform in registers, error-free FP32
// sums, cache-hinted stores and the swizzled staging layout.
//
// A 64-point transform is done by a group of 8 threads, thread t holding the
// 8 values x[t + 8a], a = 0..7 ("four-step", 64 = 8 x 8):
//   Y[t][c]  = sum_a x[8a + t] w8^(a c)          (DFT8 in registers)
//   Y[t][c] *= w64^(t c)                          (twiddle)
//   exchange through shared memory so that thread t holds Y[b][t], b = 0..7
//   X[t + 8d] = sum_b Y[b][t] w8^(b d)            (DFT8 in registers)
// so the output comes back in the same "t + 8j" order as the input.
#pragma once

#include "async_copy.cuh"
#include "fft_core.cuh"

namespace scft {

namespace {

constexpr int kRowPad = 72;              // padded row stride (float2) of a 64 x 64 plane
constexpr int kPlanePad = 64 * kRowPad;  // float2 per padded plane

template <int SIGN> __device__ __forceinline__ void dft8f(float2 *v) { Dft<8, SIGN, float2>::run(v); }

template <int SIGN> __device__ __forceinline__ void tw64(float2 *v, int t, const float2 *tw) {
#pragma unroll
  for (int c = 1; c < 8; c++) v[c] = ctw<SIGN>(v[c], tw[t * c]);
}

// 64-point transform of a group of 8 threads (see above).  Element (b, c) of
// the exchange lives at xch[b * sb + c * sc].  WARP: the 8 threads and their
// exchange area belong to one warp, so a warp barrier suffices.
template <int SIGN, bool WARP>
__device__ __forceinline__ void fft64_group(float2 *v, int t, float2 *xch, int sb, int sc, const float2 *tw) {
  dft8f<SIGN>(v);
  tw64<SIGN>(v, t, tw);
#pragma unroll
  for (int c = 0; c < 8; c++) xch[t * sb + c * sc] = v[c];
  if (WARP) __syncwarp(); else __syncthreads();
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = xch[b * sb + t * sc];
  if (WARP) __syncwarp(); else __syncthreads();
  dft8f<SIGN>(v);
}

// The same transform for the column phase of a 512-thread, 64 x 64 plane
// task (thread tid holds column tid % 64): the 8 threads of a column lie in
// the even warps (columns 0-31) or the odd ones (32-63), so the exchange's
// write-to-read barrier is a named barrier over those 8 warps only.  AFTER:
// 1 ends with a block barrier (the caller reuses the exchange area), 0 with
// none (the caller leaves the area untouched until its own next barrier).
template <int SIGN, int AFTER>
__device__ __forceinline__ void fft64_colhalf(float2 *v, int t, float2 *xch, const float2 *tw) {
  dft8f<SIGN>(v);
  tw64<SIGN>(v, t, tw);
#pragma unroll
  for (int c = 0; c < 8; c++) xch[t * 512 + c * 64] = v[c];
  if (threadIdx.x & 32)  // odd warps: columns 32-63
    asm volatile("bar.sync 2, 256;\n" ::: "memory");
  else
    asm volatile("bar.sync 1, 256;\n" ::: "memory");
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = xch[b * 512 + t * 64];
  if (AFTER) __syncthreads();
  dft8f<SIGN>(v);
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// The per-step arrays (propagator, factors, accumulators) stay in L2 while
// the history streams past with evict-first (async_copy.cuh).
__device__ __forceinline__ void st_stream(float2 *g, float2 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;\n" ::"l"(g), "f"(v.x), "f"(v.y), "l"(pol)
               : "memory");
}

// Element (row, x) of a plane staged by four 64 x 128 B boxes with the
// 128-byte swizzle: box x / 16, 16-byte chunk ((x % 16) / 2) ^ (row % 8).
__device__ __forceinline__ float2 swz(const float2 *plane, int row, int x) {
  return plane[(x >> 4) * 1024 + row * 16 + ((((x & 15) >> 1) ^ (row & 7)) << 1) + (x & 1)];
}


// Thread-block clusters: rank in the cluster, barrier (arrive with release,
// wait with acquire), and loads from a partner CTA's shared memory.
__device__ __forceinline__ uint32_t cl_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release;\n" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory"); }
__device__ __forceinline__ void cl_sync() {
  cl_arrive();
  cl_wait();
}
// address of this CTA's shared object p in the shared memory of CTA `rank` of the cluster
__device__ __forceinline__ uint32_t cl_map(const void *p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ float2 ld_cl(uint32_t a) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ double ld_cl_d(uint32_t a) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];\n" : "=d"(v) : "r"(a) : "memory");
  return v;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// 32-point transform of a group of 4 threads, thread t holding the 8 values
// x[t + 4a] (32 = 8 x 4):
//   Y[t][c]  = sum_a x[t + 4a] w8^(a c)          (DFT8 in registers)
//   Y[t][c] *= w32^(t c)
//   exchange: thread t takes c = t and c = t + 4
//   X[c + 8d] = sum_b Y[b][c] w4^(b d)            (two DFT4)
// so X[t + 4j] returns in v[j], the input order.  Element (b, c) of the
// exchange lives at xch[b * sb + c * sc]; WARP: the 4 threads and their
// exchange area belong to one warp.
template <int SIGN, bool WARP>
__device__ __forceinline__ void fft32_group(float2 *v, int t, float2 *xch, int sb, int sc, const float2 *tw32) {
  dft8f<SIGN>(v);
#pragma unroll
  for (int c = 1; c < 8; c++) v[c] = ctw<SIGN>(v[c], tw32[t * c]);
#pragma unroll
  for (int c = 0; c < 8; c++) xch[t * sb + c * sc] = v[c];
  if (WARP) __syncwarp(); else __syncthreads();
  float2 p[4], q[4];
#pragma unroll
  for (int b = 0; b < 4; b++) {
    p[b] = xch[b * sb + t * sc];
    q[b] = xch[b * sb + (t + 4) * sc];
  }
  if (WARP) __syncwarp(); else __syncthreads();
  Dft<4, SIGN, float2>::run(p);
  Dft<4, SIGN, float2>::run(q);
#pragma unroll
  for (int d = 0; d < 4; d++) {
    v[2 * d] = p[d];
    v[2 * d + 1] = q[d];
  }
}


// 12-point transform in registers (a = n1 + 3 n2, c = k2 + 4 k1): DFT4 over
// n2, twiddle w12^(n1 k2) = tw48[4 n1 k2], DFT3 over n1; output in natural
// order (tw48: the 48-point twiddles).
template <int SIGN> __device__ __forceinline__ void dft12f(float2 *v, const float2 *tw48) {
  float2 u[3][4];
#pragma unroll
  for (int n1 = 0; n1 < 3; n1++) {
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) u[n1][n2] = v[n1 + 3 * n2];
    Dft<4, SIGN, float2>::run(u[n1]);
  }
#pragma unroll
  for (int n1 = 1; n1 < 3; n1++)
#pragma unroll
    for (int k2 = 1; k2 < 4; k2++) u[n1][k2] = ctw<SIGN>(u[n1][k2], tw48[4 * n1 * k2]);
#pragma unroll
  for (int k2 = 0; k2 < 4; k2++) {
    float2 w[3] = {u[0][k2], u[1][k2], u[2][k2]};
    Dft<3, SIGN, float2>::run(w);
#pragma unroll
    for (int k1 = 0; k1 < 3; k1++) v[k2 + 4 * k1] = w[k1];
  }
}

// 48-point transform of a group of 4 threads, thread t holding the 12
// values x[t + 4a] (48 = 12 x 4):
//   Y[t][c]  = sum_a x[t + 4a] w12^(a c)          (DFT12 in registers)
//   Y[t][c] *= w48^(t c)
//   exchange: thread t takes c = t, t + 4, t + 8
//   X[c + 12d] = sum_b Y[b][c] w4^(b d)            (three DFT4)
// so X[t + 4j] returns in v[j], the input order.  Element (b, c) of the
// exchange lives at xch[b * sb + c * sc]; WARP: the 4 threads and their
// exchange area belong to one warp.
template <int SIGN, bool WARP>
__device__ __forceinline__ void fft48_group(float2 *v, int t, float2 *xch, int sb, int sc, const float2 *tw48) {
  dft12f<SIGN>(v, tw48);
#pragma unroll
  for (int c = 1; c < 12; c++) v[c] = ctw<SIGN>(v[c], tw48[t * c]);
#pragma unroll
  for (int c = 0; c < 12; c++) xch[t * sb + c * sc] = v[c];
  if (WARP) __syncwarp(); else __syncthreads();
  float2 p[3][4];
#pragma unroll
  for (int e = 0; e < 3; e++)
#pragma unroll
    for (int b = 0; b < 4; b++) p[e][b] = xch[b * sb + (t + 4 * e) * sc];
  if (WARP) __syncwarp(); else __syncthreads();
#pragma unroll
  for (int e = 0; e < 3; e++) {
    Dft<4, SIGN, float2>::run(p[e]);
#pragma unroll
    for (int d = 0; d < 4; d++) v[e + 3 * d] = p[e][d];
  }
}

}  // namespace

// 16-point transform in registers, n = a + 4b, k = c + 4d: DFT4 over b,
// twiddle w16^(a c) = tw[S a c] (tw: the 16 S-point twiddles), DFT4 over a;
// the output is in natural order.
template <int SIGN, int S = 8> __device__ __forceinline__ void dft16f(float2 *v, const float2 *tw) {
  float2 z[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
#pragma unroll
    for (int b = 0; b < 4; b++) z[a][b] = v[a + 4 * b];
    Dft<4, SIGN, float2>::run(z[a]);
  }
#pragma unroll
  for (int a = 1; a < 4; a++)
#pragma unroll
    for (int c = 1; c < 4; c++) z[a][c] = ctw<SIGN>(z[a][c], tw[S * a * c]);
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float2 u[4] = {z[0][c], z[1][c], z[2][c], z[3][c]};
    Dft<4, SIGN, float2>::run(u);
#pragma unroll
    for (int d = 0; d < 4; d++) v[c + 4 * d] = u[d];
  }
}

}  // namespace scft
